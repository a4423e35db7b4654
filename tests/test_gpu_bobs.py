"""BOBS strategies on the GPU: seeded streams equal to theboss's per-sample loop."""
import numpy as np
import pytest

from conftest import as_matrix, load_golden

pytestmark = pytest.mark.gpu


def test_bobs_streams_match_reference():
    from theboss_gb300.approximation_strategies import (LossyStateApproximationSimulationStrategy,
                                                        NonuniformLossesApproximationStrategy)
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator

    for rec in load_golden("bobs_samples.json"):
        U = as_matrix(rec["U"])
        calc = RyserPermanentCalculator(U, input_state=rec["input"])
        np.random.seed(rec["seed"])
        if rec["kind"] == "uniform_bobs":
            strat = LossyStateApproximationSimulationStrategy(calc, rec["eta"], rec["k"], threads_number=1)
            got = strat.simulate(rec["input"], rec["N"])
        else:
            strat = NonuniformLossesApproximationStrategy(calc, rec["k"], threads_number=1)
            got = strat.simulate(rec["input"], rec["N"] - 1)  # one worker: N - 1 + 1 - 0 samples
        assert all(isinstance(s, tuple) for s in got)
        assert [list(s) for s in got] == rec["samples"], rec["kind"]
        assert np.random.random() == rec["next_random"], rec["kind"]


def test_instances_sampler_equals_shared_matrix_sampler():
    """One matrix per sample with identical matrices gives the shared-matrix stream."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    U = haar_unitary(10, 3)
    inp = np.array([1, 1, 2, 0, 1, 0, 0, 1, 0, 0], dtype=np.int32)
    N = 300
    rng = np.random.default_rng(4)
    n = int(inp.sum())
    ri = np.array([[rng.integers(0, n - k) for k in range(n)] for _ in range(N)], dtype=np.int32)
    uu = rng.random((N, n))
    shared = _native.gccb_sample_instances(U, np.tile(inp, (N, 1)), ri, uu)
    per = _native.gccb_sample_instances(np.repeat(U[None], N, axis=0), np.tile(inp, (N, 1)), ri, uu)
    assert np.array_equal(shared, per)
    assert (shared.sum(axis=1) == n).all()
    with pytest.raises(ValueError):
        bad = ri.copy()
        bad[0, 0] = n
        _native.gccb_sample_instances(U, np.tile(inp, (N, 1)), bad, uu)
