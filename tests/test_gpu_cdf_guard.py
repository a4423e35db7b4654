"""The sampler's cdf guard and headline-size sampling parity.

Every draw of the batched C&C-B sampler is theboss's numpy.random.choice rule
(generalized_cliffords_b_simulation_strategy.py:107-110: cdf = cumsum(p), divided
by its last entry, searchsorted(cdf, u, 'right')) on the pmf of
generalized_cliffords_b_simulation_strategy.py:82-92.  The GPU decides from a
fast scan and hands every draw whose uniform lies within the pmf's error bound of
a cdf step to the exact sequential rule.  These tests place uniforms 1e-13 ..
1e-8 (relative) from a cdf step, pre-drawn on the host, and check each decision
against an accurate reference: the oracle where its own minors are accurate to
~1e-15 (6 photons), and a pmf built from double-double minors at the headline
size (20 photons in 40 modes), where theboss's Ryser-form minors are only
accurate to ~1e-10 and would decide such near ties by their own rounding.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cdf(U, S, sub):
    """theboss's normalised pmf from the minors and numpy's cdf, in float64."""
    m = U.shape[0]
    pmf = []
    for o in range(m):
        p = 0j
        for i in range(m):
            p += S[i] * sub[i] * U[o][i]
        pmf.append(abs(p) ** 2)
    total = sum(pmf)
    cdf = np.cumsum([v / total for v in pmf])
    return cdf / cdf[-1]


def _bases(oracle, U, n, count, seed, accurate):
    """Random lossless draws for `count` samples; for each, the state before its
    last step and that step's cdf (from the oracle, or from double-double minors
    when `accurate`)."""
    m = U.shape[0]
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        ri = np.array([rng.integers(0, n - k) for k in range(n)], dtype=np.int32)
        uu = rng.random(n)
        work = list(range(n))
        S = np.zeros(m, dtype=np.int32)
        T = np.zeros(m, dtype=np.int32)
        for k in range(n - 1):
            S[work.pop(ri[k])] += 1
            o, _ = oracle.gccb_step(U, S, T, uu[k])
            T[o] += 1
        S[work.pop(ri[n - 1])] += 1
        if accurate:
            sub = oracle.submatrices_dd(U, list(S), list(T))
        else:
            sub = oracle.submatrices(U, list(S), list(T), oracle.RYSER)
        cdf = _cdf(U, S, sub)
        out.append((ri, uu, S, T, sub, cdf))
    return out


def _crafted(oracle, U, bases, deltas):
    """One instance per (base, delta, side): the last uniform placed `delta` above
    or below a cdf step with substantial mass on both sides."""
    ri_rows, uu_rows, expect, dist = [], [], [], []
    for ri, uu, S, T, sub, cdf in bases:
        steps = [b for b in range(len(cdf) - 1) if 0.05 < cdf[b] < 0.95 and cdf[b + 1] - cdf[b] > 1e-3]
        b = steps[len(steps) // 2]
        for d in deltas:
            for side in (-1.0, 1.0):
                u = cdf[b] + side * d
                u = (np.ceil if side > 0 else np.floor)(u * 2.0 ** 53) / 2.0 ** 53  # numpy's 53-bit grid
                o = oracle.choice_from_minors(U, S, sub, u)
                Tx = T.copy()
                Tx[o] += 1
                r = uu.copy()
                r[-1] = u
                ri_rows.append(ri)
                uu_rows.append(r)
                expect.append(Tx)
                dist.append(d)
    return np.array(ri_rows), np.array(uu_rows), np.array(expect), np.array(dist)


def test_cdf_guard_small_case_matches_oracle(oracle, minors_arith):
    """6 photons in 16 modes: uniforms 1e-13 .. 1e-8 from a cdf step decide as the
    oracle (whose minors are accurate to ~2e-15 here) decides.  FP64 (the default):
    every offset.  Float pairs (opt-in): offsets beyond their error window."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    n, m = 6, 16
    U = haar_unitary(m, 616)
    bases = _bases(oracle, U, n, 12, 5, accurate=False)
    deltas = [1e-13, 1e-12, 1e-11, 1e-10, 1e-9, 1e-8]
    R, Uu, expect, dist = _crafted(oracle, U, bases, deltas)
    inputs = np.zeros((len(R), m), dtype=np.int32)
    inputs[:, :n] = 1
    _native.gccb_near_ties(reset=True)
    got = _native.gccb_sample_instances(U, inputs, R, Uu)
    ties = _native.gccb_near_ties(reset=True)
    bad = (got != expect).any(axis=1)
    if minors_arith == "fp64":
        assert not bad.any(), f"offsets {sorted(set(dist[bad]))} decided differently"
        assert ties >= (dist <= 1e-12).sum()  # the guard fires for the nearest offsets
    else:
        assert not bad[dist >= 1e-8].any()
        assert ties >= (dist <= 1e-10).sum()


def test_cdf_guard_headline_size_matches_double_double(oracle):
    """20 photons in 40 modes (the benchmark's geometry), FP64: uniforms 1e-13 ..
    1e-10 from a cdf step decide as the pmf of double-double minors decides."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    n, m = 20, 40
    U = haar_unitary(m, 2040)
    bases = _bases(oracle, U, n, 2, 9, accurate=True)
    deltas = [1e-13, 1e-12, 1e-11, 1e-10]
    R, Uu, expect, dist = _crafted(oracle, U, bases, deltas)
    inputs = np.zeros((len(R), m), dtype=np.int32)
    inputs[:, :n] = 1
    assert _native.minors_arithmetic(-1) == _native.FP64
    _native.gccb_near_ties(reset=True)
    got = _native.gccb_sample_instances(U, inputs, R, Uu)
    ties = _native.gccb_near_ties(reset=True)
    bad = (got != expect).any(axis=1)
    assert not bad.any(), f"offsets {sorted(set(dist[bad]))} decided differently"
    assert ties >= (dist <= 1e-12).sum()


def test_headline_workload_stream_matches_oracle(oracle):
    """The benchmark's workload at full size: 10^4 uniform-loss (eta = 0.5) samples
    of 20 photons in 40 modes, FP64.  Every sample equals the oracle's (theboss's
    algorithm restated) for the same numpy seed, and numpy's generator ends in the
    same state.  A sample may differ only at a draw whose uniform lies within
    theboss's own pmf error of a cdf step; any difference is checked against the
    double-double pmf at that step, which the GPU must agree with."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    n, m, N, seed = 20, 40, 10000, 2026
    U = haar_unitary(m, seed)
    inp = [1] * n + [0] * (m - n)
    w = oracle.binomial_weights(n, 0.5)
    np.random.seed(seed)
    L, A, Uu = oracle.predraw_gccb(inp, N, w)
    ref = oracle.gccb_run(U, L, A, Uu)
    ref_next = np.random.random()
    np.random.seed(seed)
    got = _native.gccb_sample(U, np.array(inp, dtype=np.int32), w, N)
    assert np.random.random() == ref_next
    rep = oracle.classify_mismatches(U, L, A, Uu, got, ref)
    assert rep["gpu_disagrees_with_double_double"] == 0, rep
    assert rep["mismatches"] <= 2, rep
