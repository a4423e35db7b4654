"""The allocation-free permanent entry point (boss_perm_batch_noalloc).

It serves callers that cannot let a library call cudaMalloc: a process whose
own pool allocator owns the GPU's memory, a service under a hard memory cap,
or a loop that cannot afford cudaMalloc's implicit device synchronisation.  The
caller owns the output buffer; the library's scratch is one static device
array.  Checked against the oracle (theboss's calculators restated; a
double-double evaluator for the larger permanents) on two different requests
in a row, so the second call runs on scratch the first one left behind, and on
a caller's stream with both requests queued back to back and one
synchronisation at the end.  This file is collected last on purpose: it is the
newest entry point, and a run that stops at the first failure has run
everything else first.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _requests():
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    rng = np.random.default_rng(99)
    # first request: 12 permanents of 14 photons (one product size), Glynn
    m = 28
    U1 = haar_unitary(m, 11)
    S1 = np.zeros((12, m), dtype=np.int32)
    S1[:, :14] = 1
    T1 = np.zeros((12, m), dtype=np.int32)
    for k in range(12):
        for i in rng.choice(m, size=14):
            T1[k, i] += 1
    # second request: mixed product sizes (two sweep images reuse the scratch) and
    # three permanents that need no sweep (theboss's empty-state rules), Ryser
    m2 = 16
    U2 = haar_unitary(m2, 12)
    S2 = np.zeros((9, m2), dtype=np.int32)
    T2 = np.zeros((9, m2), dtype=np.int32)
    for k in range(6):
        n = 6 if k % 2 else 9
        S2[k, :n] = 1
        for i in rng.choice(m2, size=n):
            T2[k, i] += 1
    S2[7, 0] = 1  # one input particle, no output: 0
    T2[8, 3] = 1  # no input, one output particle: 0; row 6 (both empty): 1
    return [(U1, S1, T1, _native.GLYNN), (U2, S2, T2, _native.RYSER)]


def _oracle_values(oracle, U, S, T, variant):
    """theboss's values: the double-double permanent (rounded) for the 14-photon
    request, the oracle's Ryser restatement (every edge case included) for the other."""
    from theboss_gb300 import _native

    out = []
    for s, t in zip(S, T):
        if variant == _native.GLYNN:
            hi, lo = oracle.perm_dd(U, list(s), list(t))
            out.append(hi + lo)
        else:
            out.append(oracle.perm(U, list(s), list(t), oracle.RYSER))
    return np.array(out)


def _check(got, ref):
    assert got.shape == ref.shape
    for a, b in zip(got, ref):
        assert abs(a - b) <= REL_TOL * max(abs(b), 1e-300), (a, b)


def test_noalloc_matches_oracle_on_two_calls(oracle):
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native

    for U, S, T, variant in _requests():
        ref = _oracle_values(oracle, U, S, T, variant)
        out = torch.full((2 * len(S),), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _native.perm_batch_noalloc(U, S, T, variant, out.data_ptr(), 0)
        torch.cuda.synchronize()
        _check(out.cpu().numpy().view(np.complex128), ref)


def test_noalloc_back_to_back_on_a_caller_stream(oracle):
    """Both requests queued on one non-default stream without a synchronisation in
    between (the second call refills the host staging array and the scratch while
    the first one's work may still be in flight), one synchronisation at the end."""
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native

    reqs = _requests()
    refs = [_oracle_values(oracle, U, S, T, v) for U, S, T, v in reqs]
    stream = torch.cuda.Stream()
    outs = [torch.full((2 * len(S),), float("nan"), dtype=torch.float64, device="cuda") for _, S, _, _ in reqs]
    torch.cuda.synchronize()
    for (U, S, T, v), out in zip(reqs, outs):
        _native.perm_batch_noalloc(U, S, T, v, out.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    for out, ref in zip(outs, refs):
        _check(out.cpu().numpy().view(np.complex128), ref)


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    # 4096 single-photon permanents of 24 photons need about 36 MiB of fixed-point
    # rows, more than the 8 MiB scratch.  The request is planned whole and rejected
    # before anything is queued: the caller's buffer keeps its contents.
    m, n, count = 48, 24, 4096
    U = haar_unitary(m, 3)
    S = np.zeros((count, m), dtype=np.int32)
    S[:, :n] = 1
    T = np.zeros((count, m), dtype=np.int32)
    T[:, n:] = 1
    S[0, :] = 0  # an empty-state permanent too, which would be written first if queued
    T[0, :] = 0
    out = torch.full((2 * count,), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(_native.GB300Error, match="scratch"):
        _native.perm_batch_noalloc(U, S, T, _native.GLYNN, out.data_ptr(), 0)
    torch.cuda.synchronize()
    assert bool((out == 7.0).all())
