"""GPU parity on degenerate matrices: exact zeros (a phased permutation matrix, a
Haar matrix with half its entries zeroed, a zero column) and rows scaled over
ten binades.  The sweeps multiply most factors in block floating point on the
integer pipe; where every term has a zero factor the result must be exactly
zero, elsewhere it must agree with the double-double oracle to 1e-12 of the
largest term the sum can hold (the FP64 sums' own error is of that order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M = 16


def _haar(m, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    Q, R = np.linalg.qr(A)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def _matrices():
    rng = np.random.default_rng(77)
    P = np.zeros((M, M), dtype=np.complex128)
    P[np.arange(M), rng.permutation(M)] = np.exp(2j * np.pi * rng.random(M))
    Z = _haar(M, 3)
    Z[rng.random((M, M)) < 0.5] = 0.0
    C = _haar(M, 4)
    C[:, 5] = 0.0
    R = _haar(M, 5) * (2.0 ** -rng.integers(0, 10, size=M))[:, None]
    return {"permutation": P, "half_zero": Z, "zero_column": C, "row_scaled": R}


def _term_bound(U, S, T):
    """The larger of prod over the output particles of sum over the input
    particles of |U| and the same with the sides exchanged: no term of a Ryser,
    Glynn or Chin-Huh sum over either side (binomial weights included) exceeds
    it by more than 2^n."""
    A = np.abs(U)
    by_rows = np.prod([A[j, :] @ np.array(S, dtype=float) for j, t in enumerate(T) for _ in range(int(t))])
    by_cols = np.prod([np.array(T, dtype=float) @ A[:, i] for i, s in enumerate(S) for _ in range(int(s))])
    return float(max(by_rows, by_cols))


def _patterns(rng, n):
    S = [1] * n + [0] * (M - n)
    out = []
    for _ in range(3):
        T = [0] * M
        k = 0
        while k < n:
            i = int(rng.integers(0, M))
            if T[i] < 2:
                T[i] += 1
                k += 1
        out.append(T)
    out.append(list(S))  # the input modes themselves
    return S, out


@pytest.mark.parametrize("name", ["permutation", "half_zero", "zero_column", "row_scaled"])
def test_permanents_on_degenerate_matrices(oracle, name):
    from theboss_gb300 import permanent_calculators as pc

    U = _matrices()[name]
    rng = np.random.default_rng(11)
    for n in (6, 10):
        S, Ts = _patterns(rng, n)
        for T in Ts:
            hi, lo = oracle.perm_dd(U, S, T)
            ref = hi + lo
            scale = max(abs(ref), _term_bound(U, S, T) * 2.0 ** n)
            for cls, tol in ((pc.GlynnGrayPermanentCalculator, 1e-12), (pc.ChinHuhPermanentCalculator, 1e-12),
                             (pc.RyserPermanentCalculator, 1e-12)):
                got = cls(U, S, T).compute_permanent()
                if scale == 0.0:  # every term of either side's sum has a zero factor
                    assert got == 0, (name, cls.__name__, T, got)
                else:
                    assert abs(got - ref) <= tol * scale, (name, cls.__name__, T, got, ref)


@pytest.mark.parametrize("name", ["permutation", "half_zero", "zero_column", "row_scaled"])
def test_minors_on_degenerate_matrices(oracle, name):
    from theboss_gb300.submatrices_calculators import BSCCRyserSubmatricesPermanentCalculator

    U = _matrices()[name]
    rng = np.random.default_rng(12)
    k = 10
    S = [0] * M
    for i in rng.choice(M, size=k, replace=False):
        S[i] = 1
    T = [0] * M
    c = 0
    while c < k - 1:
        i = int(rng.integers(0, M))
        if T[i] < 2:
            T[i] += 1
            c += 1
    got = BSCCRyserSubmatricesPermanentCalculator(U, S, T).compute_permanents()
    ref = oracle.submatrices_dd(U, S, T)
    scale = max(max(abs(v) for v in ref), _term_bound(U, S, T) * 2.0 ** k)
    for a, b in zip(got, ref):
        if scale == 0.0:
            assert a == 0
        else:
            assert abs(a - b) <= 1e-12 * scale, (name, a, b)


def test_sampler_on_a_sparse_matrix(oracle):
    """The batched sampler on a sparse unitary (four 4-mode Haar blocks, modes
    shuffled: three quarters of the entries and many probabilities exactly zero)
    draws the oracle's samples."""
    from theboss_gb300 import _native

    rng = np.random.default_rng(13)
    B = np.zeros((M, M), dtype=np.complex128)
    for b in range(4):
        B[4 * b:4 * b + 4, 4 * b:4 * b + 4] = _haar(4, 20 + b)
    p = rng.permutation(M)
    U = B[p][:, rng.permutation(M)]
    n, N = 8, 300
    inp = [1] * n + [0] * (M - n)
    w = oracle.binomial_weights(n, 0.5)
    np.random.seed(5)
    L, A, Uu = oracle.predraw_gccb(inp, N, w)
    ref = oracle.gccb_run(U, L, A, Uu)
    np.random.seed(5)
    got = _native.gccb_sample(U, np.array(inp, dtype=np.int32), w, N)
    assert int((got != ref).any(axis=1).sum()) == 0
