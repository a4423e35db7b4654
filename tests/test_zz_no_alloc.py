"""The allocation-free permanent entry point (boss_perm_batch_noalloc).

It serves callers that cannot let a library call cudaMalloc: a process whose
own pool allocator owns the GPU's memory, a service under a hard memory cap,
or a loop that cannot afford cudaMalloc's implicit device synchronisation.  The
caller owns the output buffer; the library's scratch is one static device
array.  Checked against the allocating entry point (boss_perm_batch) on two
different requests in a row, so the second call runs on scratch the first one
left behind.  This file is collected last on purpose: it is the newest entry
point, and a run that stops at the first failure has run everything else first.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _requests():
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    rng = np.random.default_rng(99)
    # first call: 12 permanents of 14 photons (one product size), Glynn
    m = 28
    U1 = haar_unitary(m, 11)
    S1 = np.zeros((12, m), dtype=np.int32)
    S1[:, :14] = 1
    T1 = np.zeros((12, m), dtype=np.int32)
    for k in range(12):
        for i in rng.choice(m, size=14):
            T1[k, i] += 1
    # second call: mixed product sizes (two sweep groups reuse the scratch) plus an
    # empty-state permanent that needs no sweep, Ryser
    m2 = 16
    U2 = haar_unitary(m2, 12)
    S2 = np.zeros((7, m2), dtype=np.int32)
    T2 = np.zeros((7, m2), dtype=np.int32)
    for k in range(6):
        n = 6 if k % 2 else 9
        S2[k, :n] = 1
        for i in rng.choice(m2, size=n):
            T2[k, i] += 1
    return [(U1, S1, T1, _native.GLYNN), (U2, S2, T2, _native.RYSER)]


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native

    for U, S, T, variant in _requests():
        ref = _native.perm_batch(U, S, T, variant)
        out = torch.full((2 * len(S),), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _native.perm_batch_noalloc(U, S, T, variant, out.data_ptr(), 0)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.complex128)
        assert got.shape == ref.shape
        for a, b in zip(got, ref):
            assert abs(a - b) <= REL_TOL * max(abs(b), 1e-300), (a, b)


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    # 4096 single-photon permanents of 24 photons need about 36 MiB of fixed-point
    # rows, more than the 8 MiB scratch: rejected before anything is queued.
    m, n, count = 48, 24, 4096
    U = haar_unitary(m, 3)
    S = np.zeros((count, m), dtype=np.int32)
    S[:, :n] = 1
    T = np.zeros((count, m), dtype=np.int32)
    T[:, n:] = 1
    out = torch.zeros(2 * count, dtype=torch.float64, device="cuda")
    with pytest.raises(_native.GB300Error, match="scratch"):
        _native.perm_batch_noalloc(U, S, T, _native.GLYNN, out.data_ptr(), 0)
