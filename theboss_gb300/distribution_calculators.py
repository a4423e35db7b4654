"""Drop-in GB300 replacements for theboss's exact distribution calculators.

  BosonSamplingExperimentConfiguration       bs_distribution_calculator_interface.py:11-26
  BSDistributionCalculatorInterface          bs_distribution_calculator_interface.py:29-52
  BSDistributionCalculatorWithFixedLosses    bs_distribution_calculator_with_fixed_losses.py:23-169
  BSDistributionCalculatorWithUniformLosses  bs_exact_distribution_with_uniform_losses.py:22-104

theboss evaluates one outcome at a time: a loop over the lossy inputs, one
permanent each (the uniform-loss calculator spreads the outcomes over a process
pool).  Here every requested outcome, with every lossy input, is one call of
boss_lossy_probabilities (libboss_gb300.so): one GPU thread per (lossy input,
outcome) pair, then one per outcome for the sum and the normalisation, in
theboss's operation order.  The permanent calculator passed in is kept for API
compatibility; the GPU computes the permanents whatever its type (they agree to
rounding).
"""
from __future__ import annotations

import abc
from copy import deepcopy
from dataclasses import dataclass
from typing import Any, List, Sequence

import numpy as np
from scipy import special

from . import _native
from .utilities import generate_possible_states, possible_states_array


@dataclass
class BosonSamplingExperimentConfiguration:
    interferometer_matrix: Sequence[Sequence[complex]]
    initial_state: Sequence[int]
    initial_number_of_particles: int
    number_of_modes: int
    number_of_particles_lost: int
    number_of_particles_left: int
    uniform_transmissivity: float = 1
    network_simulation_strategy: Any = None
    hierarchy_level: int = 0


class BSDistributionCalculatorInterface(abc.ABC):
    @abc.abstractmethod
    def calculate_distribution(self) -> List[float]:
        raise NotImplementedError

    @abc.abstractmethod
    def calculate_probabilities_of_outcomes(self, outcomes: List[Sequence[int]]) -> List[float]:
        raise NotImplementedError

    @abc.abstractmethod
    def get_outcomes_in_proper_order(self) -> List[Sequence[int]]:
        raise NotImplementedError


def _outcome_array(outcomes, m: int) -> np.ndarray:
    """Outcomes (tuples, lists, int or integer-valued float arrays) -> int32 rows."""
    if isinstance(outcomes, np.ndarray):
        a = outcomes
    else:
        rows = [list(o) for o in outcomes]
        if not rows:
            return np.zeros((0, m), dtype=np.int32)
        a = np.asarray(rows, dtype=np.float64)
    return np.ascontiguousarray(np.rint(a).astype(np.int32).reshape(-1, m))


class BSDistributionCalculatorWithFixedLosses(BSDistributionCalculatorInterface):
    """Exact output distribution when exactly number_of_particles_lost particles
    of the initial state are lost (uniformly at random)."""

    def __init__(self, configuration: BosonSamplingExperimentConfiguration, permanent_calculator) -> None:
        self.configuration = deepcopy(configuration)
        self._permanent_calculator = permanent_calculator

    def get_outcomes_in_proper_order(self) -> List[tuple]:
        return generate_possible_states(self.configuration.number_of_particles_left,
                                        self.configuration.number_of_modes)

    def _outcomes_in_proper_order_array(self) -> np.ndarray:
        return possible_states_array(self.configuration.number_of_particles_left, self.configuration.number_of_modes)

    def calculate_distribution(self) -> List[float]:
        return self._probabilities(self._outcomes_in_proper_order_array()).tolist()

    def calculate_probabilities_of_outcomes(self, outcomes) -> List[float]:
        T = _outcome_array(outcomes, self.configuration.number_of_modes)
        left = self.configuration.number_of_particles_left
        if T.shape[0] and np.any(T.sum(axis=1) != left):
            raise AttributeError("every outcome must hold number_of_particles_left particles")
        return self._probabilities(T).tolist()

    def _probabilities(self, T: np.ndarray) -> np.ndarray:
        c = self.configuration
        return _native.lossy_probabilities(np.asarray(c.interferometer_matrix), c.initial_state, T)


class BSDistributionCalculatorWithUniformLosses(BSDistributionCalculatorWithFixedLosses):
    """Exact output distribution when every particle is transmitted with probability
    uniform_transmissivity: the fixed-loss probability of each outcome weighted by
    the binomial probability of its particle count."""

    def __init__(self, configuration: BosonSamplingExperimentConfiguration, permanent_calculator) -> None:
        super().__init__(configuration, permanent_calculator)
        self.weights = self._initialize_weights()
        self.weightless = False

    def set_weightless(self, weightless: bool) -> None:
        if not weightless:
            self.weights = self._initialize_weights()
        else:
            self.weights = [1 for _ in self.weights]
        self.weightless = weightless

    def _initialize_weights(self) -> List[float]:
        # bs_exact_distribution_with_uniform_losses.py:42-60, same expression
        def weight(n, l, eta):
            return pow(eta, l) * special.binom(n, l) * pow(1.0 - eta, n - l)

        n = self.configuration.initial_number_of_particles
        return [weight(n, l, self.configuration.uniform_transmissivity) for l in range(n + 1)]

    def get_outcomes_in_proper_order(self) -> List[tuple]:
        return generate_possible_states(self.configuration.initial_number_of_particles,
                                        self.configuration.number_of_modes, losses=True)

    def _outcomes_in_proper_order_array(self) -> np.ndarray:
        return possible_states_array(self.configuration.initial_number_of_particles,
                                     self.configuration.number_of_modes, losses=True)

    def calculate_probabilities_of_outcomes(self, outcomes) -> List[float]:
        return self._probabilities(_outcome_array(outcomes, self.configuration.number_of_modes)).tolist()

    def _probabilities(self, T: np.ndarray) -> np.ndarray:
        # bs_exact_distribution_with_uniform_losses.py:73-97: l = 0 gives weights[0]
        p = super()._probabilities(T)
        ls = T.sum(axis=1)
        w = np.asarray(self.weights, dtype=np.float64)
        return np.where(ls == 0, w[0], p * w[ls])


def _register_with_reference() -> None:
    """When theboss itself is importable, make its abstract interface recognise
    these classes."""
    try:
        from theboss.distribution_calculators.bs_distribution_calculator_interface import (
            BSDistributionCalculatorInterface as _Ref,
        )
    except Exception:
        return
    for cls in (BSDistributionCalculatorWithFixedLosses, BSDistributionCalculatorWithUniformLosses):
        _Ref.register(cls)


_register_with_reference()


class BosonSamplingSimulator:
    """boson_sampling_simulator.py:18-25: runs a strategy."""

    def __init__(self, simulation_strategy) -> None:
        self._simulation_strategy = simulation_strategy

    def get_classical_simulation_results(self, input_state, samples_number: int = 1):
        return self._simulation_strategy.simulate(input_state, samples_number)


class BSSampleBasedDistributionCalculator(BSDistributionCalculatorInterface):
    """Empirical distribution of a strategy's samples over a list of outcomes
    (bs_sample_based_distribution_calculator.py:18-113).  The samples are counted
    on the GPU (boss_count_outcomes) instead of theboss's sample-by-outcome scan.
    As in theboss, calculate_distribution() and calculate_probabilities_of_outcomes()
    draw calculate_approximate_distribution's default 5000 samples."""

    def __init__(self, experiment_configuration: BosonSamplingExperimentConfiguration, strategy,
                 samples_number=5000, outcomes=None) -> None:
        self._configuration = experiment_configuration
        self._strategy = strategy
        self._outcomes = outcomes
        self._samples_number = samples_number

    @property
    def configuration(self) -> BosonSamplingExperimentConfiguration:
        return self._configuration

    @configuration.setter
    def configuration(self, new_configuration: BosonSamplingExperimentConfiguration) -> None:
        self._configuration = new_configuration

    @property
    def strategy(self):
        return self._strategy

    @strategy.setter
    def strategy(self, new_strategy) -> None:
        self._strategy = new_strategy

    @property
    def outcomes(self):
        return self._outcomes

    @outcomes.setter
    def outcomes(self, new_outcomes) -> None:
        self._outcomes = new_outcomes

    @property
    def samples_number(self) -> int:
        return self._samples_number

    @samples_number.setter
    def samples_number(self, new_samples_number: int) -> None:
        self._samples_number = new_samples_number

    def calculate_distribution(self) -> List[float]:
        return self.calculate_approximate_distribution()

    def calculate_probabilities_of_outcomes(self, outcomes) -> List[float]:
        self._outcomes = outcomes
        return self.calculate_approximate_distribution()

    def calculate_approximate_distribution(self, samples_number: int = 5000) -> List[float]:
        m = self.configuration.number_of_modes
        if self._outcomes is not None:
            outcomes = self._outcomes
        else:
            outcomes = possible_states_array(self.configuration.number_of_particles_left, m)
        samples = BosonSamplingSimulator(self._strategy).get_classical_simulation_results(
            self.configuration.initial_state, samples_number)
        counts = _native.count_outcomes(samples, outcomes, m)
        return list(counts.astype(np.float64) / samples_number)

    def get_outcomes_in_proper_order(self):
        return self._outcomes
