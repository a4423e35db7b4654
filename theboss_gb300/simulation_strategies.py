"""Drop-in GB300 replacements for theboss's generalized Clifford & Clifford samplers.

  SimulationStrategyInterface                          simulation_strategy_interface.py:7-23
  GeneralizedCliffordsBSimulationStrategy              generalized_cliffords_b_simulation_strategy.py:31-110
  GeneralizedCliffordsBUniformLossesSimulationStrategy generalized_cliffords_b_uniform_losses_simulation_strategy.py:24-121
  LossyNetworksGeneralizedCliffordsSimulationStrategy  lossy_networks_generalized_cliffords_simulation_strategy.py:24-88
  GeneralizedCliffordsSimulationStrategy               generalized_cliffords_simulation_strategy.py:20-266
  GeneralizedCliffordsUniformLossesSimulationStrategy  generalized_cliffords_uniform_losses_simulation_strategy.py:19-173

The B-version samplers hand the whole request to the batched GPU sampler
(libboss_gb300.so, boss_gccb_sample): it consumes numpy's global RandomState
exactly as theboss does (same calls, same order), so with the same seed it
returns the samples theboss returns (given the same probabilities) and leaves
the generator in the same state.  Return types follow theboss: tuples for the
lossless and network-loss samplers, int64 arrays for the uniform-loss sampler.

GCCBPlainDriver is the reference's per-step loop with the GPU all-minors
calculator dropped in (one GPU launch per sampling step); it exists to measure
what batching buys.
"""
from __future__ import annotations

import abc
import random as _stdlib_random
from collections import defaultdict
from copy import copy
from math import factorial
from typing import List, Sequence, Tuple

import numpy as np

from . import _native
from .permanent_calculators import BSPermanentCalculatorInterface
from .submatrices_calculators import BSCCRyserSubmatricesPermanentCalculator
from .utilities import mode_occupation_to_mode_assignment, prepare_interferometer_matrix_in_expanded_space


class SimulationStrategyInterface(abc.ABC):
    @abc.abstractmethod
    def simulate(self, input_state: Sequence[int], samples_number: int = 1):
        raise NotImplementedError


def _binomial_weights(n: int, eta: float) -> List[float]:
    """generalized_cliffords_b_uniform_losses_simulation_strategy.py:50-65 (same
    expression, same evaluation order)."""
    from scipy.special import binom

    return [binom(n, l) * pow(eta, l) * pow(1 - eta, n - l) for l in range(n + 1)]


class GeneralizedCliffordsBSimulationStrategy(SimulationStrategyInterface):
    """C&C-B, lossless.  simulate() -> list of tuples."""

    def __init__(self, bs_permanent_calculator: BSPermanentCalculatorInterface) -> None:
        self._bs_permanent_calculator = bs_permanent_calculator
        self.r_sample: List[int] = []
        self.input_state: Sequence[int] = []
        self.number_of_input_photons = 0

    def set_new_matrix(self, new_matrix) -> None:
        self._bs_permanent_calculator.matrix = new_matrix

    def _gpu_samples(self, input_state, samples_number: int, weights) -> np.ndarray:
        U = _native.as_matrix(self._bs_permanent_calculator.matrix)
        inp = np.asarray(input_state)
        if inp.dtype.kind == "f":
            inp = np.rint(inp)
        return _native.gccb_sample(U, inp.astype(np.int32), weights, int(samples_number))

    def simulate(self, input_state: Sequence[int], samples_number: int = 1) -> List[Tuple[int, ...]]:
        self.input_state = input_state
        self.number_of_input_photons = int(sum(input_state))
        out = self._gpu_samples(input_state, samples_number, None)
        return [tuple(row) for row in out.tolist()]


class GeneralizedCliffordsBUniformLossesSimulationStrategy(GeneralizedCliffordsBSimulationStrategy):
    """C&C-B with uniform losses (binomial number of surviving particles).
    simulate() -> list of int64 arrays."""

    def __init__(self, bs_permanent_calculator: BSPermanentCalculatorInterface, transmissivity: float = 1.0) -> None:
        super().__init__(bs_permanent_calculator)
        self._transmissivity = transmissivity
        self._binomial_weights: List[float] = []

    def simulate(self, input_state, samples_number: int = 1) -> List[np.ndarray]:
        self.input_state = input_state
        self.number_of_input_photons = int(sum(input_state))
        self._binomial_weights = _binomial_weights(self.number_of_input_photons, self._transmissivity)
        out = self._gpu_samples(input_state, samples_number, self._binomial_weights).astype(np.int64)
        return list(out)


class LossyNetworksGeneralizedCliffordsSimulationStrategy(SimulationStrategyInterface):
    """Non-uniform (mode-dependent) losses: lossless C&C-B in the 2m-mode unitary
    dilation of the lossy matrix, extra modes trimmed.  simulate() -> list of tuples."""

    def __init__(self, bs_permanent_calculator: BSPermanentCalculatorInterface) -> None:
        bs_permanent_calculator.matrix = prepare_interferometer_matrix_in_expanded_space(
            bs_permanent_calculator.matrix)
        self._helper_strategy = GeneralizedCliffordsBSimulationStrategy(bs_permanent_calculator)

    def simulate(self, input_state: Sequence[int], samples_number: int = 1) -> List[Tuple[int, ...]]:
        m = len(input_state)
        expanded = np.concatenate([np.asarray(input_state), np.zeros(m, dtype=int)])
        out = self._helper_strategy._gpu_samples(expanded, samples_number, None)
        return [tuple(row[:m]) for row in out.tolist()]

    def set_new_matrix(self, matrix) -> None:
        self._helper_strategy.set_new_matrix(prepare_interferometer_matrix_in_expanded_space(matrix))


class GCCBPlainDriver(GeneralizedCliffordsBUniformLossesSimulationStrategy):
    """theboss's own per-sample, per-step C&C-B loop
    (generalized_cliffords_b_simulation_strategy.py:69-110 with the uniform-loss
    particle count of generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-121),
    calling the GPU all-minors calculator once per step.  Same samples and random
    stream as the batched sampler."""

    def simulate(self, input_state, samples_number: int = 1) -> List[np.ndarray]:
        self.input_state = input_state
        self.number_of_input_photons = int(sum(input_state))
        self._binomial_weights = _binomial_weights(self.number_of_input_photons, self._transmissivity)
        particles = list(mode_occupation_to_mode_assignment(input_state))
        U = self._bs_permanent_calculator.matrix
        m = len(input_state)
        samples = []
        while len(samples) < samples_number:
            kept, acc, thr = 0, 0, np.random.random()
            for w in self._binomial_weights:
                acc += w
                if acc > thr:
                    break
                kept += 1
            current = np.zeros(m, dtype=np.int64)
            work = particles.copy()
            r = [0] * m
            while kept > sum(r):
                current[work.pop(np.random.randint(0, len(work)))] += 1
                sub = BSCCRyserSubmatricesPermanentCalculator(U, current, r).compute_permanents()
                perms = np.asarray(U) @ (current * np.asarray(sub))
                pmf = [abs(p) ** 2 for p in perms]
                total = sum(pmf)
                pmf = [v / total for v in pmf]
                r[np.random.choice(range(m), p=pmf)] += 1
            samples.append(np.array(r, dtype=np.int64))
        return samples


class GeneralizedCliffordsSimulationStrategy(SimulationStrategyInterface):
    """Plain (A-version) generalized C&C (generalized_cliffords_simulation_strategy.py:20-266).

    Per new output prefix r, every output r + e_j gets the probability
    sum_S w_S |perm(U[r + e_j, S])|^2 / (prod S! |S|!) over the input's
    sub-multisets S with |r| + 1 particles; layers are memoised per prefix.  theboss
    draws exactly one numpy random() per sampling step, so the whole stream is drawn
    up front (same calls, same order) and all samples advance together step by
    step: each step's new prefixes become one batched GPU permanent launch."""

    def __init__(self, bs_permanent_calculator: BSPermanentCalculatorInterface) -> None:
        self.r_sample: List[int] = []
        self.number_of_input_photons = 0
        self.pmfs = dict()
        self._bs_permanent_calculator = bs_permanent_calculator
        self.input_state: Sequence[int] = []
        self._labeled_states = defaultdict(list)
        self.possible_outputs = dict()
        self.current_key = tuple(self.r_sample)
        self.current_sample_probability = 1

    def set_new_matrix(self, new_matrix) -> None:
        self._bs_permanent_calculator.matrix = new_matrix

    def simulate(self, input_state, samples_number: int = 1):
        self._initialize(input_state)
        n = self.number_of_input_photons
        steps = [n] * int(samples_number)
        uniforms = np.random.random(n * int(samples_number)) if n > 0 else np.zeros(0)
        return [tuple(r) for r in self._run(steps, uniforms, len(input_state))]

    def _initialize(self, input_state) -> None:
        self.input_state = input_state
        self.number_of_input_photons = int(sum(input_state))
        self._get_sorted_possible_states()
        self.pmfs = dict()

    def _get_sorted_possible_states(self) -> None:
        states = [()]
        for v in reversed(list(self.input_state)):  # generalized_cliffords_simulation_strategy.py:95-121 order
            states = [(i,) + s for i in range(int(v) + 1) for s in states]
        self._labeled_states = defaultdict(list)
        for s in states:
            self._labeled_states[sum(s)].append(np.array(s, dtype=np.int64))

    def _run(self, steps, uniforms, width: int) -> List[List[int]]:
        """Advances every sample step by step; steps[s] sampling steps for sample s,
        uniforms consumed in sample-major order (theboss's order)."""
        N = len(steps)
        offsets = np.concatenate([[0], np.cumsum(steps)]).astype(np.int64)
        r = [[0] * width for _ in range(N)]
        self._last_modes = []  # modes sampled for the last sample, in order
        for k in range(max(steps, default=0)):
            active = [sidx for sidx in range(N) if steps[sidx] > k]
            missing = []
            seen = set()
            for sidx in active:
                key = tuple(r[sidx])
                if key not in self.pmfs and key not in seen:
                    seen.add(key)
                    missing.append(list(key))
            if missing:
                self._calculate_layers(missing)
            for sidx in active:
                key = tuple(r[sidx])
                r[sidx] = self._sample(key, uniforms[offsets[sidx] + k])
                if sidx == N - 1:
                    self._last_modes.append(self._last_index)
        if N:
            self.r_sample = r[-1]
            self.current_key = tuple(self.r_sample)
        return r

    def _sample(self, key, u: float) -> List[int]:
        """generalized_cliffords_simulation_strategy.py:249-266."""
        pmf = self.pmfs[key]
        idx = 0
        rv = u * sum(pmf)
        acc = 0
        for p in pmf:
            acc += p
            if acc > rv:
                break
            idx += 1
        self.current_sample_probability = pmf[idx]
        self._last_index = idx
        return self.possible_outputs[key][idx]

    def _weights(self, k_vectors) -> np.ndarray:
        """generalized_cliffords_simulation_strategy.py:173-205."""
        from scipy.special import binom

        n = int(sum(self.input_state))
        out = []
        for kv in k_vectors:
            l = int(sum(kv))
            w = factorial(l) * factorial(n - l) / factorial(n)
            for mm in range(len(self.input_state)):
                w *= binom(self.input_state[mm], kv[mm])
            out.append(w)
        return np.asarray(out, dtype=np.float64)

    def _calculate_layers(self, prefixes: List[List[int]]) -> None:
        """Layers of every prefix in `prefixes` (all with the same particle count):
        one batched permanent launch for all (prefix, output, input) triples."""
        k = sum(prefixes[0]) + 1
        inputs = self._labeled_states[k]
        weights = self._weights([[self.input_state[i] - st[i] for i in range(len(st))] for st in inputs])
        weights /= sum(weights)
        m = len(prefixes[0])
        outs = []
        for pre in prefixes:
            layer = []
            for j in range(m):
                o = list(pre)
                o[j] += 1
                layer.append(o)
            outs.append(layer)
        P, C = len(prefixes), len(inputs)
        L = len(self.input_state)
        T = np.repeat(np.asarray(outs, dtype=np.int32).reshape(P * m, 1, m), C, axis=1).reshape(-1, m)
        S = np.tile(np.asarray(inputs, dtype=np.int32).reshape(1, C, L), (P * m, 1, 1)).reshape(-1, L)
        calc = self._bs_permanent_calculator
        variant = getattr(calc, "_VARIANT", _native.RYSER)
        perms = _native.perm_batch(_native.as_matrix(calc.matrix), np.ascontiguousarray(S),
                                   np.ascontiguousarray(T), variant)
        prob = (np.abs(perms) ** 2).reshape(P, m, C)
        # generalized_cliffords_simulation_strategy.py:240-245: one division per
        # occupied mode factorial, then by |S|!
        for i, st in enumerate(inputs):
            for v in st:
                prob[:, :, i] /= factorial(int(v))
            prob[:, :, i] /= factorial(int(sum(st)))
        pmf = np.zeros((P, m))
        for i in range(C):  # :160-169, sequential over the inputs
            pmf += prob[:, :, i] * weights[i]
        for p_idx, pre in enumerate(prefixes):
            key = tuple(pre)
            self.possible_outputs[key] = outs[p_idx]
            self.pmfs[key] = list(pmf[p_idx])


class GeneralizedCliffordsUniformLossesSimulationStrategy(GeneralizedCliffordsSimulationStrategy):
    """A-version with per-photon uniform losses: each photon survives when Python's
    random.random() < transmissivity (generalized_cliffords_uniform_losses_simulation_strategy.py:125-138),
    then one numpy random() per surviving photon.  The two generators are
    independent, so both streams are drawn up front in theboss's order."""

    def __init__(self, bs_permanent_calculator: BSPermanentCalculatorInterface, transmissivity: float = 0) -> None:
        self._transmissivity = transmissivity
        super().__init__(bs_permanent_calculator)

    def simulate(self, input_state, samples_number: int = 1) -> List[np.ndarray]:
        self._initialize(input_state)
        n = self.number_of_input_photons
        N = int(samples_number)
        kept = []
        for _ in range(N):
            c = 0
            for _photon in range(n):
                if _stdlib_random.random() >= self._transmissivity:
                    continue
                c += 1
            kept.append(c)
        uniforms = np.random.random(sum(kept)) if sum(kept) else np.zeros(0)
        width = len(self._bs_permanent_calculator.matrix)
        return [np.array(r, dtype=np.int64) for r in self._run(kept, uniforms, width)]


class ModeAssignmentGeneralizedCliffordsSimulationStrategyInterface(GeneralizedCliffordsSimulationStrategy):
    """Generalized C&C in the mode-assignment description
    (mode_assignment_generalized_cliffords_simulation_strategy.py:16-112): the
    prefix is the ordered tuple of sampled modes and layers are memoised per tuple.
    A layer's probabilities depend only on the prefix's occupation, and theboss
    draws the same one random() per step, so the samples equal the plain
    strategy's for the same stream; this runs the same batched engine.  Samples
    are occupation tuples; r_sample holds the last sample's modes in sampling order."""

    def simulate(self, input_state, samples_number: int = 1) -> List[Tuple[int, ...]]:
        samples = super().simulate(input_state, samples_number)
        if samples:
            self.r_sample = tuple(int(i) for i in self._last_modes)
            self.current_key = self.r_sample
        return [tuple(int(x) for x in s) for s in samples]
