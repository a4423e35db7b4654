"""The CPU oracle pinned against fixtures produced by theboss itself (CPU only)."""
import numpy as np
import pytest

from conftest import as_matrix, load_golden

VARIANTS = (("ryser", 0), ("chin_huh", 1), ("glynn", 2), ("classic", 3))


def test_single_permanents_match_reference(oracle):
    for rec in load_golden("perms.json"):
        U = as_matrix(rec["U"])
        for name, v in VARIANTS:
            if name not in rec:
                continue
            ref = complex(*rec[name])
            got = oracle.perm(U, rec["S"], rec["T"], v)
            assert abs(got - ref) <= 1e-15 * max(1.0, abs(ref)), (name, rec["S"], rec["T"], got, ref)


def test_submatrix_permanents_match_reference(oracle):
    for rec in load_golden("submatrices.json"):
        U = as_matrix(rec["U"])
        S = [int(x) for x in rec["S"]]
        T = [int(x) for x in rec["T"]]
        for name, v in (("ryser", 0), ("chin_huh", 1)):
            ref = [complex(*z) for z in rec[name]]
            got = oracle.submatrices(U, S, T, v)
            assert len(got) == len(ref)
            for a, b in zip(got, ref):
                assert abs(a - b) <= 1e-15 * max(1.0, abs(b)), (name, S, T)


def test_guan_sequences_match_reference(oracle):
    for rec in load_golden("guan.json"):
        idx, r = oracle.guan_sequence(rec["S"])
        assert idx.tolist() == rec["idx"]
        assert r.tolist() == rec["r"]


def test_gccb_sample_streams_match_reference(oracle):
    for rec in load_golden("gcc_samples.json"):
        if rec["kind"] not in ("gccb", "gccb_uniform", "lossy_net"):
            continue
        m = len(rec["input"])
        if rec["kind"] == "lossy_net":
            U = as_matrix(rec["expanded"])
            inp = list(rec["input"]) + [0] * m
            eta = None
        else:
            U = as_matrix(rec["U"])
            inp = rec["input"]
            eta = rec["eta"] if rec["kind"] == "gccb_uniform" else None
        np.random.seed(rec["seed"])
        out = oracle.gccb_simulate(U, inp, rec["N"], eta)
        assert out[:, :m].tolist() == rec["samples"]
        assert np.random.random() == rec["next_random"]


def test_exact_distributions_match_reference(oracle):
    for rec in load_golden("distributions.json"):
        got = oracle.uniform_loss_distribution(as_matrix(rec["U"]), rec["input"], rec["eta"])
        assert np.allclose(got, rec["distribution"], rtol=0, atol=1e-15)


def test_lossy_distributions_match_reference(oracle):
    """Fixed- and uniform-loss probabilities (standard, binned and 11-particle
    cases) against theboss's own calculators."""
    for rec in load_golden("lossy_distributions.json"):
        U = as_matrix(rec["U"])
        got = [oracle.fixed_loss_probability(U, rec["input"], T) for T in rec["outcomes"]]
        if rec["kind"] == "uniform":
            n = sum(rec["input"])
            w = oracle.binomial_weights(n, rec["eta"])
            got = [w[0] if sum(T) == 0 else p * w[sum(T)] for p, T in zip(got, rec["outcomes"])]
        assert np.allclose(got, rec["probabilities"], rtol=1e-12, atol=1e-300)


def test_known_answer_permutation_distribution(oracle):
    """tests/test_exact_distribution_calculator.py:75-141 of the reference."""
    P = np.zeros((5, 5), dtype=complex)
    for r, c in ((0, 2), (1, 0), (2, 3), (3, 4), (4, 1)):
        P[r, c] = 1
    d = oracle.uniform_loss_distribution(P, [1, 1, 1, 0, 0], 0.8)
    expect = np.zeros(56)
    for i, v in ((0, 0.008), (1, 0.032), (2, 0.032), (5, 0.032), (7, 0.128), (10, 0.128), (14, 0.128), (29, 0.512)):
        expect[i] = v
    assert np.allclose(d, expect)


@pytest.mark.parametrize("n", [6, 9, 12])
def test_double_double_oracle_agrees_with_fp64(oracle, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(2 * n, 2 * n)) + 1j * rng.normal(size=(2 * n, 2 * n))
    Q, R = np.linalg.qr(A)
    U = Q * (np.diag(R) / np.abs(np.diag(R)))
    S = [1] * n + [0] * n
    T = [0] * (2 * n)
    for i in rng.choice(2 * n, size=n, replace=True):
        T[i] += 1
    hi, lo = oracle.perm_dd(U, S, T)
    ref = hi + lo
    for v in (0, 1, 2):
        got = oracle.perm(U, S, T, v)
        assert abs(got - ref) <= 1e-11 * abs(ref)


def test_size_mismatch_raises_attribute_error(oracle):
    U = np.eye(3, dtype=complex)
    with pytest.raises(AttributeError):
        oracle.perm(U, [1, 1], [1, 1, 0])
