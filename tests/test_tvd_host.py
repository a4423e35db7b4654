"""Total-variation distances (no GPU) against theboss's own values."""
import numpy as np

from conftest import load_golden


def test_tvd_matches_reference_bit_for_bit():
    from theboss_gb300.quantum_computations_utilities import (count_total_variation_distance,
                                                              count_total_variation_distance_dicts)

    for rec in load_golden("tvd.json"):
        if rec["kind"] == "list":
            assert count_total_variation_distance(rec["a"], rec["b"]) == rec["tvd"]
            assert count_total_variation_distance(np.array(rec["a"]), np.array(rec["b"])) == rec["tvd"]
        else:
            d1 = {tuple(k): v for k, v in rec["d1"]}
            d2 = {tuple(k): v for k, v in rec["d2"]}
            assert count_total_variation_distance_dicts(d1, d2) == rec["tvd"]


def test_tvd_edge_cases():
    import pytest

    from theboss_gb300.quantum_computations_utilities import (count_total_variation_distance,
                                                              count_total_variation_distance_dicts)

    assert count_total_variation_distance([], []) == 0.0
    assert count_total_variation_distance_dicts({}, {}) == 0
    assert count_total_variation_distance_dicts({(1,): 1.0}, {(0,): 1.0}) == 1.0
    with pytest.raises(AssertionError):
        count_total_variation_distance([0.5, 0.5], [1.0])
