"""Sample frequencies on the GPU (boss_count_outcomes) against theboss's scan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan(samples, outcomes):
    """bs_sample_based_distribution_calculator.py:94-106, as written."""
    counts = np.zeros(len(outcomes))
    for s in samples:
        for j in range(len(outcomes)):
            if all(np.asarray(s) == outcomes[j]):
                counts[j] += 1
                break
    return counts


def test_counts_match_the_reference_scan():
    from theboss_gb300 import _native
    from theboss_gb300.utilities import possible_states_array

    rng = np.random.default_rng(3)
    outcomes = possible_states_array(3, 5)
    outcomes = np.concatenate([outcomes, outcomes[:7], outcomes[::5]])  # repeated outcomes
    samples = possible_states_array(3, 5)[rng.integers(0, 35, 900)]
    samples = np.concatenate([samples, possible_states_array(2, 5)[:20]])  # samples matching nothing
    got = _native.count_outcomes(samples, outcomes, 5)
    assert got.tolist() == _scan(samples, outcomes).tolist()
    assert got.sum() == 900


def test_counts_large_and_edge_cases():
    from theboss_gb300 import _native
    from theboss_gb300.utilities import possible_states_array

    outs = possible_states_array(6, 12)  # 12,376 outcomes
    rng = np.random.default_rng(4)
    idx = rng.integers(0, len(outs), 200_000)
    got = _native.count_outcomes(outs[idx], outs, 12)
    assert np.array_equal(got, np.bincount(idx, minlength=len(outs)))
    assert _native.count_outcomes(np.zeros((0, 12)), outs, 12).sum() == 0
    assert _native.count_outcomes(outs[:3], np.zeros((0, 12)), 12).shape == (0,)
    with pytest.raises(ValueError):
        _native.count_outcomes([[255, 0]], [[1, 0]], 2)


def test_sample_based_distribution_counts_the_strategy_samples():
    from theboss_gb300.distribution_calculators import (BosonSamplingExperimentConfiguration,
                                                        BSSampleBasedDistributionCalculator)
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator
    from theboss_gb300.simulation_strategies import GeneralizedCliffordsBSimulationStrategy
    from theboss_gb300.utilities import generate_possible_states, haar_unitary

    U = haar_unitary(5, 11)
    inp = [1, 1, 1, 0, 0]
    cfg = BosonSamplingExperimentConfiguration(interferometer_matrix=U, initial_state=inp,
                                               initial_number_of_particles=3, number_of_modes=5,
                                               number_of_particles_lost=0, number_of_particles_left=3)
    strat = GeneralizedCliffordsBSimulationStrategy(RyserPermanentCalculator(U))
    calc = BSSampleBasedDistributionCalculator(cfg, strat)
    np.random.seed(5)
    dist = calc.calculate_distribution()
    np.random.seed(5)
    samples = strat.simulate(inp, 5000)
    outs = generate_possible_states(3, 5)
    assert np.allclose(dist, _scan(samples, outs) / 5000, rtol=0, atol=0)
    assert abs(sum(dist) - 1.0) < 1e-12
