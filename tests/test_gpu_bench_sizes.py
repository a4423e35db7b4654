"""Sampler parity at the benchmark's own sizes.

The headline C&C-B stream is checked at its benchmark size (10^4 samples) by the
bench itself and by test_gpu_sampling.py; these two check the other samplers the
bench times, at the sizes it times them:
  * plain generalized C&C (A-version): 8 photons in 16 modes, lossless, 1000
    samples (generalized_cliffords_simulation_strategy.py).  Its sampling is host
    code in theboss's order; the GPU computes every layer's permanents.  The same
    stream with the oracle's permanents (theboss's Glynn-Gray calculator restated)
    must give the same samples.
  * uniform-loss BOBS: 20 photons in 40 modes, eta = 0.5, hierarchy level 10,
    2000 samples (lossy_state_approximated_simulation_strategy.py).  Every
    per-sample matrix, input and pre-drawn stream the strategy hands to the GPU's
    instance sampler is sampled again by the oracle's C&C-B restatement.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 2026


def test_plain_gcc_at_benchmark_size_matches_oracle_permanents(oracle, monkeypatch):
    from theboss_gb300 import _native
    from theboss_gb300.permanent_calculators import GlynnGrayPermanentCalculator
    from theboss_gb300.simulation_strategies import GeneralizedCliffordsSimulationStrategy
    from theboss_gb300.utilities import haar_unitary

    U = haar_unitary(16, SEED + 8)
    inp = [1] * 8 + [0] * 8
    np.random.seed(SEED)
    got = GeneralizedCliffordsSimulationStrategy(GlynnGrayPermanentCalculator(U)).simulate(inp, 1000)
    after = np.random.random()
    monkeypatch.setattr(_native, "perm_batch", lambda Um, S, T, v: oracle.perm_batch(Um, S, T, v))
    np.random.seed(SEED)
    ref = GeneralizedCliffordsSimulationStrategy(GlynnGrayPermanentCalculator(U)).simulate(inp, 1000)
    assert np.random.random() == after
    assert len(got) == 1000 and all(sum(s) == 8 for s in got)
    assert got == ref


def test_uniform_bobs_at_benchmark_size_matches_oracle(oracle, monkeypatch):
    from theboss_gb300 import _native
    from theboss_gb300.approximation_strategies import LossyStateApproximationSimulationStrategy
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator
    from theboss_gb300.utilities import haar_unitary

    calls = []
    real = _native.gccb_sample_instances

    def spy(mats, inputs, ri, uu):
        out = real(mats, inputs, ri, uu)
        calls.append((np.array(mats), np.array(inputs), np.array(ri), np.array(uu), out.copy()))
        return out

    monkeypatch.setattr(_native, "gccb_sample_instances", spy)
    U = haar_unitary(40, SEED + 40)
    inp = [1] * 20 + [0] * 20
    strat = LossyStateApproximationSimulationStrategy(RyserPermanentCalculator(U, input_state=inp), 0.5, 10,
                                                      threads_number=1)
    np.random.seed(SEED)
    samples = strat.simulate(inp, 2000)
    assert len(samples) == 2000 and len(calls) == 1
    mats, inputs, ri, uu, out = calls[0]
    assert [tuple(int(x) for x in r) for r in out] == samples
    checked = 0
    for s in range(len(inputs)):
        # the popped modes: theboss pops the ri-th remaining particle of the list ordered by mode
        work = [i for i, v in enumerate(inputs[s]) for _ in range(int(v))]
        L = len(work)
        if L == 0:
            assert not out[s].any()
            continue
        A = [work.pop(int(ri[s][k])) for k in range(L)]
        ref = oracle.gccb_run(mats[s], np.array([L], dtype=np.int32), np.array([A], dtype=np.int32),
                              np.array([uu[s][:L]]))
        assert np.array_equal(ref[0], out[s]), s
        checked += 1
    assert checked > 1900
