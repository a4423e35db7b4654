"""Host-side pieces of the exact distribution calculators (no GPU): outcome and
lossy-input enumeration in theboss's order, the configuration dataclass, the
uniform-loss weights."""
import numpy as np
import pytest

from conftest import load_golden


def test_outcome_order_matches_reference():
    from theboss_gb300.utilities import generate_possible_states, possible_states_array

    for rec in load_golden("lossy_distributions.json"):
        n, m = sum(rec["input"]), len(rec["input"])
        if rec["kind"] == "fixed" and len(rec["outcomes"]) > 3:
            got = generate_possible_states(n - rec["lost"], m)
            assert [list(t) for t in got] == rec["outcomes"]
        if rec["kind"] == "uniform" and rec["input"] == [3, 1, 2, 0]:
            got = possible_states_array(n, m, losses=True)
            assert got.tolist() == rec["outcomes"]


def test_lossy_input_order_matches_reference():
    from theboss_gb300.utilities import generate_lossy_n_particle_input_states

    for rec in load_golden("lossy_distributions.json"):
        if "lossy_inputs" in rec:
            got = generate_lossy_n_particle_input_states(rec["input"], sum(rec["input"]) - rec["lost"])
            assert [list(t) for t in got] == rec["lossy_inputs"]
    assert generate_lossy_n_particle_input_states([0, 0, 0], 0) == [(0, 0, 0)]


def test_state_counts():
    from math import comb

    from theboss_gb300.utilities import possible_states_array

    for n, m in ((0, 3), (4, 5), (8, 16)):
        assert possible_states_array(n, m).shape == (comb(n + m - 1, m - 1), m)
    assert possible_states_array(3, 4, losses=True).shape[0] == comb(3 + 4, 4)
    a = possible_states_array(8, 16)
    assert (a.sum(axis=1) == 8).all() and len({tuple(r) for r in a.tolist()}) == a.shape[0]


def test_uniform_weights_and_weightless():
    from theboss_gb300.distribution_calculators import (BosonSamplingExperimentConfiguration,
                                                        BSDistributionCalculatorWithUniformLosses)
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator

    U = np.eye(3, dtype=complex)
    cfg = BosonSamplingExperimentConfiguration(interferometer_matrix=U, initial_state=[1, 1, 0],
                                               initial_number_of_particles=2, number_of_modes=3,
                                               number_of_particles_lost=0, number_of_particles_left=2,
                                               uniform_transmissivity=0.25)
    c = BSDistributionCalculatorWithUniformLosses(cfg, RyserPermanentCalculator(U))
    assert np.allclose(c.weights, [0.75 ** 2, 2 * 0.25 * 0.75, 0.25 ** 2])
    c.set_weightless(True)
    assert c.weights == [1, 1, 1] and c.weightless
    c.set_weightless(False)
    assert np.isclose(sum(c.weights), 1.0)
    assert len(c.get_outcomes_in_proper_order()) == 10  # C(2 + 3, 3)


def test_fixed_losses_rejects_wrong_particle_count():
    from theboss_gb300.distribution_calculators import (BosonSamplingExperimentConfiguration,
                                                        BSDistributionCalculatorWithFixedLosses)

    U = np.eye(3, dtype=complex)
    cfg = BosonSamplingExperimentConfiguration(interferometer_matrix=U, initial_state=[1, 1, 0],
                                               initial_number_of_particles=2, number_of_modes=3,
                                               number_of_particles_lost=1, number_of_particles_left=1)
    c = BSDistributionCalculatorWithFixedLosses(cfg, None)
    with pytest.raises(AttributeError):
        c.calculate_probabilities_of_outcomes([(1, 1, 0)])
