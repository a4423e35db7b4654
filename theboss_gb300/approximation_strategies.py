"""Drop-in GB300 replacements for theboss's BOBS (Brod-Oszmaniec) approximate
samplers.

  LossyStateApproximationSimulationStrategy   lossy_state_approximated_simulation_strategy.py:36-362
  NonuniformLossesApproximationStrategy       nonuniform_losses_approximation_strategy.py:65-347

Each sample of these strategies is an independent lossless C&C-B sample of its
own (lossy) input state through its own matrix: the interferometer with random
phases and a QFT on the approximated modes (and, for non-uniform losses, the
2m-mode dilation of that matrix).  theboss draws the samples one at a time in
worker processes started with `spawn`, whose numpy generators are seeded from the
OS, so its streams cannot be reproduced.  Here every random number is drawn from
the caller's numpy global RandomState, in the per-sample order of theboss's
worker loop (the replay in libboss_gb300.so), the per-sample matrices are built
with theboss's own numpy expressions, and all samples run in one batched GPU
sampler call (boss_gccb_sample_instances).  With one worker theboss's loop would
produce the same samples.
"""
from __future__ import annotations

from math import sqrt
from multiprocessing import cpu_count
from typing import List, Sequence, Tuple

import numpy as np
from scipy.special import binom

from . import _native
from .utilities import (generate_lossy_n_particle_input_states, generate_qft_matrix_for_first_m_modes,
                        prepare_interferometer_matrix_in_expanded_space)


def _proper_threads_number(threads_number: int) -> int:
    if threads_number < 1 or threads_number > cpu_count():
        return cpu_count()
    return threads_number


def _check_probabilities(p) -> None:
    """numpy.random.choice's checks on p (legacy RandomState)."""
    p = np.asarray(p, dtype=np.float64)
    if np.any(p < 0):
        raise ValueError("probabilities are not non-negative")
    if abs(float(np.sum(p)) - 1.0) > np.sqrt(np.finfo(np.float64).eps):
        raise ValueError("probabilities do not sum to 1")


def _phases_matrix(uniforms: np.ndarray, m: int) -> np.ndarray:
    """generate_random_phases_matrix_for_first_m_modes with the phases' uniforms given."""
    random_phases = np.ones(m, dtype=np.complex128)
    random_phases[0:len(uniforms)] = np.exp(1j * 2 * np.pi * uniforms)
    return np.diag(random_phases)


class LossyStateApproximationSimulationStrategy:
    """BOBS for uniformly lossy experiments: losses applied to the input state
    (a mixed state over lossy inputs), the last m - k modes' particles bunched in
    mode k and spread by random phases and a QFT."""

    def __init__(self, bs_permanent_calculator, uniform_transmissivity: float, hierarchy_level: int,
                 threads_number: int = -1) -> None:
        self._approximated_input_state_part_possibilities = None
        self._approximated_input_state_part_possibilities_weights = None
        self._not_approximated_lossy_mixed_state_parts = None
        self._not_approximated_lossy_mixed_state_parts_weights = None
        self._hierarchy_level = hierarchy_level
        self._uniform_transmissivity = uniform_transmissivity
        self._threads_number = _proper_threads_number(threads_number)
        self._permanent_calculator = bs_permanent_calculator
        n_modes = len(bs_permanent_calculator.input_state)
        self._qft_matrix = generate_qft_matrix_for_first_m_modes(n_modes - hierarchy_level, n_modes)

    def _get_possible_lossy_inputs_weights(self, input_state: Sequence[int]) -> List[float]:
        n = int(sum(input_state))
        eta = self._uniform_transmissivity
        return [binom(n, l) * eta ** l * (1 - eta) ** (n - l) for l in range(n + 1)]

    def _prepare_tables(self, input_state: Sequence[int]) -> None:
        """lossy_state_approximated_simulation_strategy.py:132-246, same values."""
        k = self._hierarchy_level
        exact_part = list(input_state[:k])
        parts = []
        for left in range(int(sum(exact_part)) + 1):
            parts.extend(generate_lossy_n_particle_input_states(exact_part, left))
        self._not_approximated_lossy_mixed_state_parts = parts
        possible = self._get_possible_lossy_inputs_weights(parts[-1])
        n = sum(parts[-1])
        self._not_approximated_lossy_mixed_state_parts_weights = [possible[int(sum(p))] / binom(n, sum(p))
                                                                 for p in parts]
        approx_part = np.asarray(input_state[k:])
        if not 0 <= k < len(self._permanent_calculator.matrix):
            self._approximated_input_state_part_possibilities = [[]]
            self._approximated_input_state_part_possibilities_weights = [1]
            return
        poss = []
        for left in range(int(sum(approx_part)) + 1):
            p = np.zeros_like(approx_part)
            p[0] = left
            poss.append(p)
        self._approximated_input_state_part_possibilities = poss
        self._approximated_input_state_part_possibilities_weights = self._get_possible_lossy_inputs_weights(poss[-1])

    def simulate(self, input_state: Sequence[int], samples_number: int = 1) -> List[Tuple[int, ...]]:
        if samples_number < 1:
            return []
        self._prepare_tables(input_state)
        U = np.array(self._permanent_calculator.matrix)
        m = len(U)
        if not 0 <= self._hierarchy_level <= m:
            raise ValueError("hierarchy_level must lie in [0, number of modes]")
        k = self._hierarchy_level  # k == m: exact sampling, nothing approximated
        exact_w = self._not_approximated_lossy_mixed_state_parts_weights
        approx_w = self._approximated_input_state_part_possibilities_weights
        _check_probabilities(exact_w)
        _check_probabilities(approx_w)
        exact = np.array([list(p) for p in self._not_approximated_lossy_mixed_state_parts], dtype=np.int32).reshape(
            len(exact_w), k)
        approx = np.array([list(p) for p in self._approximated_input_state_part_possibilities],
                          dtype=np.int32).reshape(len(approx_w), m - k)
        stride = int(exact.sum(axis=1).max(initial=0) + approx.sum(axis=1).max(initial=0))
        N = int(samples_number)
        inputs, ph, perms, ri, uu = _native.bobs_uniform_predraw(N, m, k, exact, exact_w, approx, approx_w, stride)
        mq = len(self._qft_matrix) - self._hierarchy_level  # phases on the QFT's modes
        mats = np.empty((N, m, m), dtype=np.complex128)
        for s in range(N):  # lossy_state_approximated_simulation_strategy.py:334-362, same expression
            mats[s] = U[:, perms[s]] @ _phases_matrix(ph[s, :max(mq, 0)], m) @ self._qft_matrix
        out = _native.gccb_sample_instances(mats, inputs, ri, uu)
        return [tuple(int(x) for x in row) for row in out]


class NonuniformLossesApproximationStrategy:
    """BOBS for non-uniformly lossy networks: the uniform part of the losses is
    taken out of the matrix and applied to the input; the first
    approximated_modes_number modes' particles are bunched into one of them at
    random; each sample then runs the lossy-network C&C-B (2m-mode dilation) of the
    matrix with random phases and a QFT on the approximated modes."""

    def __init__(self, bs_permanent_calculator, approximated_modes_number: int, threads_number: int = -1) -> None:
        total = len(bs_permanent_calculator.matrix)
        self._approximated_modes_number = min(max(approximated_modes_number, 0), total)
        self._uniform_losses = 0
        self._initial_matrix = None
        self._extract_losses_from_the_interferometer(bs_permanent_calculator.matrix)
        self._binomial_weights = dict()
        self._threads_number = _proper_threads_number(threads_number)
        self._permanent_calculator = bs_permanent_calculator
        self._state_without_approximated_modes: List[int] = []
        self._approximated_modes_particles_number = 0

    def _extract_losses_from_the_interferometer(self, interferometer_matrix) -> None:
        """nonuniform_losses_approximation_strategy.py:120-144, same expressions."""
        u, s, v = np.linalg.svd(interferometer_matrix)
        transmissivities = [singular_value ** 2 for singular_value in s]
        losses = [1 - eta for eta in transmissivities]
        self._uniform_losses = min(losses)
        transmissivities = [eta / (1 - self._uniform_losses) for eta in transmissivities]
        s = [sqrt(eta) for eta in transmissivities]
        self._initial_matrix = u @ np.diag(s) @ v

    def _compute_binomial_weights(self, max_particles_number: int):
        eta = 1 - self._uniform_losses

        def w(total, left):
            return pow(eta, left) * binom(total, left) * pow(1.0 - eta, total - left)

        return {n: [w(n, left) for left in range(n + 1)] for n in range(1, max_particles_number + 1)}

    def _samples_count(self, samples_number: int) -> int:
        """theboss hands every worker (samples + threads - samples % threads) // threads samples."""
        t = self._threads_number
        per = int((samples_number + t - (samples_number % t)) / t)
        return per * t

    def simulate(self, input_state: Sequence[int], samples_number: int = 1) -> List[Tuple[int, ...]]:
        if samples_number < 1:
            return []
        ka = self._approximated_modes_number
        self._state_without_approximated_modes = list(input_state)
        self._approximated_modes_particles_number = 0
        for i in range(ka):
            self._approximated_modes_particles_number += input_state[i]
            self._state_without_approximated_modes[i] = 0
        top = max(max(input_state), self._approximated_modes_particles_number)
        self._binomial_weights = self._compute_binomial_weights(top)
        table = np.zeros((top + 1, top + 1))
        for n, ws in self._binomial_weights.items():
            table[n, :n + 1] = ws
        lossy = not np.isclose(self._uniform_losses, 0)
        stride = int(sum(self._state_without_approximated_modes) + self._approximated_modes_particles_number)
        N = self._samples_count(int(samples_number))
        inputs, ph, ri, uu = _native.bobs_nonuniform_predraw(
            N, self._state_without_approximated_modes, ka, self._approximated_modes_particles_number, table, lossy,
            stride)
        m = len(self._initial_matrix)
        qft = generate_qft_matrix_for_first_m_modes(ka, m)
        mats = np.empty((N, 2 * m, 2 * m), dtype=np.complex128)
        for s in range(N):  # nonuniform_losses_approximation_strategy.py:331-347, then the dilation
            M = self._initial_matrix @ _phases_matrix(ph[s], m) @ qft
            mats[s] = prepare_interferometer_matrix_in_expanded_space(M)
        expanded = np.concatenate([inputs, np.zeros_like(inputs)], axis=1)
        out = _native.gccb_sample_instances(mats, expanded, ri, uu)[:, :m]
        return [tuple(int(x) for x in row) for row in out]
