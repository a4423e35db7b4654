"""Exact lossy distributions on the GPU (boss_lossy_probabilities) against
theboss's own outputs and the oracle."""
import numpy as np
import pytest

from conftest import as_matrix, load_golden

pytestmark = pytest.mark.gpu


def _cfg(U, inp, lost, eta=1.0):
    from theboss_gb300.distribution_calculators import BosonSamplingExperimentConfiguration

    n = int(sum(inp))
    return BosonSamplingExperimentConfiguration(interferometer_matrix=U, initial_state=list(inp),
                                                initial_number_of_particles=n, number_of_modes=len(inp),
                                                number_of_particles_lost=lost, number_of_particles_left=n - lost,
                                                uniform_transmissivity=eta)


def test_lossy_distributions_match_reference_fixtures():
    from theboss_gb300.distribution_calculators import (BSDistributionCalculatorWithFixedLosses,
                                                        BSDistributionCalculatorWithUniformLosses)
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator

    for rec in load_golden("lossy_distributions.json"):
        U = as_matrix(rec["U"])
        cls = BSDistributionCalculatorWithFixedLosses if rec["kind"] == "fixed" else BSDistributionCalculatorWithUniformLosses
        c = cls(_cfg(U, rec["input"], rec["lost"], rec.get("eta", 1.0)), RyserPermanentCalculator(U))
        got = c.calculate_probabilities_of_outcomes(rec["outcomes"])
        # relative error bound of the tolerance: 1e-12 (FP64 permanents, different summation order)
        assert np.allclose(got, rec["probabilities"], rtol=1e-12, atol=1e-300)
        if len(rec["outcomes"]) > 3 and not (rec["kind"] == "uniform" and sum(rec["input"]) == 5):
            assert [list(t) for t in c.get_outcomes_in_proper_order()] == rec["outcomes"]
            assert np.allclose(c.calculate_distribution(), rec["probabilities"], rtol=1e-12, atol=1e-300)


def test_known_answer_permutation_distribution():
    """tests/test_exact_distribution_calculator.py:75-141 of the reference."""
    from theboss_gb300.distribution_calculators import BSDistributionCalculatorWithUniformLosses
    from theboss_gb300.permanent_calculators import ChinHuhPermanentCalculator

    P = np.zeros((5, 5), dtype=complex)
    for r, c in ((0, 2), (1, 0), (2, 3), (3, 4), (4, 1)):
        P[r, c] = 1
    calc = BSDistributionCalculatorWithUniformLosses(_cfg(P, [1, 1, 1, 0, 0], 2, 0.8), ChinHuhPermanentCalculator(P))
    d = calc.calculate_distribution()
    expect = np.zeros(56)
    for i, v in ((0, 0.008), (1, 0.032), (2, 0.032), (5, 0.032), (7, 0.128), (10, 0.128), (14, 0.128), (29, 0.512)):
        expect[i] = v
    assert np.allclose(d, expect, rtol=1e-12, atol=1e-15)
    for rec in load_golden("distributions.json"):
        U = as_matrix(rec["U"])
        c = BSDistributionCalculatorWithUniformLosses(_cfg(U, rec["input"], 0, rec["eta"]), ChinHuhPermanentCalculator(U))
        assert np.allclose(c.calculate_distribution(), rec["distribution"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("inp,eta", [([1, 1, 1, 1, 1, 1, 0, 0], 0.6), ([2, 0, 1, 3, 0, 0], 0.5)])
def test_uniform_distribution_matches_oracle_and_sums_to_one(oracle, inp, eta):
    from theboss_gb300.distribution_calculators import BSDistributionCalculatorWithUniformLosses
    from theboss_gb300.utilities import haar_unitary

    U = haar_unitary(len(inp), 90 + len(inp))
    c = BSDistributionCalculatorWithUniformLosses(_cfg(U, inp, 0, eta), None)
    got = np.array(c.calculate_distribution())
    assert abs(got.sum() - 1.0) < 1e-12
    outs = c.get_outcomes_in_proper_order()
    pick = list(range(0, len(outs), max(1, len(outs) // 60)))
    w = oracle.binomial_weights(sum(inp), eta)
    ref = [w[0] if sum(outs[i]) == 0 else oracle.fixed_loss_probability(U, inp, outs[i]) * w[sum(outs[i])]
           for i in pick]
    assert np.allclose(got[pick], ref, rtol=1e-12, atol=1e-300)


def test_fixed_distribution_sums_to_one_for_every_particle_count():
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary, possible_states_array

    U = haar_unitary(7, 5)
    inp = [2, 1, 1, 0, 1, 0, 0]
    for left in range(0, 6):
        p = _native.lossy_probabilities(U, inp, possible_states_array(left, 7))
        assert abs(p.sum() - 1.0) < 1e-12


def test_large_particle_count_path_and_errors():
    """l = 11 runs on the sweep engine; more particles than the input is an error;
    an empty request returns nothing."""
    from theboss_gb300 import _native

    rec = [r for r in load_golden("lossy_distributions.json") if sum(r["input"]) == 12][0]
    got = _native.lossy_probabilities(as_matrix(rec["U"]), rec["input"], rec["outcomes"])
    assert np.allclose(got, rec["probabilities"], rtol=1e-12, atol=1e-300)
    U = np.eye(3, dtype=complex)
    with pytest.raises(ValueError):
        _native.lossy_probabilities(U, [1, 0, 0], [[1, 1, 0]])
    assert _native.lossy_probabilities(U, [1, 0, 0], np.zeros((0, 3))).shape == (0,)
    assert _native.lossy_probabilities(U, [1, 1, 0], [[0, 0, 0]]).tolist() == [1.0]
