"""GPU parity of the single-permanent and all-minors calculators (calls go
through libboss_gb300.so's C ABI)."""
import copy
import pickle

import numpy as np
import pytest

from conftest import as_matrix, load_golden

pytestmark = pytest.mark.gpu

# Reference values are FP64 results of theboss itself; the GPU sums in a different
# order, so agreement is to a few thousand ULP of the largest term.
REL_TOL_SMALL = 1e-12


def haar(m, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    Q, R = np.linalg.qr(A)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def pattern_with_doubles(m, n, rng):
    T = [0] * m
    k = 0
    while k < n:
        i = int(rng.integers(0, m))
        if T[i] < 2 and (T[i] == 0 or rng.random() < 0.25) and k + 1 <= n:
            T[i] += 1
            k += 1
    return T


@pytest.fixture(scope="module")
def calcs():
    from theboss_gb300 import permanent_calculators as pc

    return {"ryser": pc.RyserPermanentCalculator, "chin_huh": pc.ChinHuhPermanentCalculator,
            "glynn": pc.GlynnGrayPermanentCalculator, "classic": pc.ClassicPermanentCalculator}


def test_fixture_permanents_all_variants(calcs):
    for rec in load_golden("perms.json"):
        U = as_matrix(rec["U"])
        for name, cls in calcs.items():
            if name not in rec and not (name == "classic" and "glynn" in rec):
                continue
            ref = complex(*rec[name if name in rec else "glynn"])
            got = cls(U, rec["S"], rec["T"]).compute_permanent()
            assert isinstance(got, np.complex128)
            assert abs(got - ref) <= REL_TOL_SMALL * max(abs(ref), 1e-3), (name, rec["S"], rec["T"], got, ref)


@pytest.mark.parametrize("n", [12, 16, 20])
def test_single_photon_permanents_against_double_double(calcs, oracle, n):
    rng = np.random.default_rng(100 + n)
    m = 2 * n
    U = haar(m, n)
    S = [1] * n + [0] * n
    for _ in range(2):
        T = pattern_with_doubles(m, n, rng)
        hi, lo = oracle.perm_dd(U, S, T)
        ref = hi + lo
        for name in ("glynn", "chin_huh", "ryser"):
            got = calcs[name](U, S, T).compute_permanent()
            tol = 1e-10 if name != "ryser" else 1e-8
            assert abs(got - ref) <= tol * abs(ref), (name, n, got, ref, abs(got - ref) / abs(ref))


@pytest.mark.parametrize("n,names", [(24, ("glynn", "chin_huh", "ryser"))])
def test_large_permanents_against_double_double(calcs, oracle, n, names):
    """One pattern: the double-double oracle's cost grows as 2^n (7 s at n = 24 on
    16 Arm cores, 170 s at n = 28)."""
    rng = np.random.default_rng(200 + n)
    m = 2 * n
    U = haar(m, n)
    S = [1] * n + [0] * n
    T = pattern_with_doubles(m, n, rng)
    hi, lo = oracle.perm_dd(U, S, T)
    ref = hi + lo
    for name in names:
        got = calcs[name](U, S, T).compute_permanent()
        tol = 1e-10 if name != "ryser" else 1e-8
        assert abs(got - ref) <= tol * abs(ref), (name, n, got, ref, abs(got - ref) / abs(ref))


def test_edge_cases(calcs):
    U = haar(4, 1)
    z = [0, 0, 0, 0]
    for name in ("ryser", "chin_huh", "glynn", "classic"):
        assert calcs[name](U, z, z).compute_permanent() == 1
    # classic: empty input, nonempty output -> 0; glynn: empty matrix -> 1
    assert calcs["classic"](U, z, [1, 0, 0, 0]).compute_permanent() == 0
    assert calcs["glynn"](U, z, [1, 0, 0, 0]).compute_permanent() == 1
    with pytest.raises(AttributeError):
        calcs["ryser"](U, [1, 1], [1, 1, 0]).compute_permanent()
    with pytest.raises(AttributeError):
        calcs["glynn"](U, [1, 1, 0, 0], [1, 0, 0, 0]).compute_permanent()
    # float-valued occupations (tests/test_bs_submatrices_permanent_calculators.py:48)
    a = calcs["ryser"](U, np.array([1.0, 1.0, 0.0, 0.0]), np.array([0.0, 2.0, 0.0, 0.0])).compute_permanent()
    b = calcs["ryser"](U, [1, 1, 0, 0], [0, 2, 0, 0]).compute_permanent()
    assert a == b


def test_in_place_matrix_update_is_seen(calcs):
    U = haar(6, 2)
    c = calcs["chin_huh"](U, [1, 1, 1, 0, 0, 0], [0, 1, 1, 1, 0, 0])
    p1 = c.compute_permanent()
    c.matrix *= 0.5 ** 0.5
    p2 = c.compute_permanent()
    assert abs(p2 - p1 * 0.5 ** 1.5) <= 1e-14


def test_runs_are_bit_identical(calcs):
    U = haar(32, 3)
    S = [1] * 16 + [0] * 16
    T = pattern_with_doubles(32, 16, np.random.default_rng(3))
    vals = {calcs["glynn"](U, S, T).compute_permanent() for _ in range(3)}
    assert len(vals) == 1


def test_calculators_pickle_and_deepcopy(calcs):
    U = haar(4, 5)
    c = calcs["ryser"](U, [1, 1, 0, 0], [0, 1, 1, 0])
    for d in (copy.deepcopy(c), pickle.loads(pickle.dumps(c))):
        assert d.compute_permanent() == c.compute_permanent()


def test_factory_defaults():
    from theboss_gb300.permanent_calculators import (BSPermanentCalculatorFactory, ChinHuhPermanentCalculator,
                                                     PermanentCalculatorType, RyserPermanentCalculator)

    assert isinstance(BSPermanentCalculatorFactory(None, None, None).generate_calculator(), RyserPermanentCalculator)
    f = BSPermanentCalculatorFactory(None, None, None, calculator_type=99)
    assert isinstance(f.generate_calculator(), ChinHuhPermanentCalculator)
    assert PermanentCalculatorType.GLYNN == 2


def test_fixture_submatrices():
    from theboss_gb300.submatrices_calculators import (BSCCCHSubmatricesPermanentCalculator,
                                                       BSCCRyserSubmatricesPermanentCalculator)

    for rec in load_golden("submatrices.json"):
        U = as_matrix(rec["U"])
        for name, cls in (("ryser", BSCCRyserSubmatricesPermanentCalculator),
                          ("chin_huh", BSCCCHSubmatricesPermanentCalculator)):
            ref = [complex(*z) for z in rec[name]]
            got = cls(U, np.array(rec["S"]), np.array(rec["T"])).compute_permanents()
            assert len(got) == len(ref)
            for a, b in zip(got, ref):
                assert abs(a - b) <= REL_TOL_SMALL * max(abs(b), 1e-3), (name, rec["S"], rec["T"], a, b)


@pytest.mark.parametrize("k", [8, 14, 18, 20])
def test_submatrices_against_double_double(oracle, k, minors_arith):
    from theboss_gb300.submatrices_calculators import BSCCRyserSubmatricesPermanentCalculator

    rng = np.random.default_rng(k)
    m = 2 * k
    U = haar(m, 50 + k)
    S = [0] * m
    for i in rng.choice(m, size=k, replace=False):
        S[i] = 1
    T = pattern_with_doubles(m, k - 1, rng)
    got = BSCCRyserSubmatricesPermanentCalculator(U, S, T).compute_permanents()
    ref = oracle.submatrices_dd(U, S, T)
    scale = max(abs(v) for v in ref)
    err = max(abs(a - b) for a, b in zip(got, ref)) / scale
    assert err <= 1e-10, (k, minors_arith, err)


def test_large_permanents_against_double_double_fixture():
    """C2 patterns at n = 26, 28, 30 (single photons in 2n modes, ~20% doubly
    occupied outputs) against double-double values computed once by the oracle
    (tests/golden/make_c2_dd.py), one permanent per call: FP64 (the default) and
    float pairs both within 1e-10."""
    import json
    import os

    from conftest import ROOT
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    recs = json.load(open(os.path.join(ROOT, "tests", "golden", "c2_dd_large.json")))
    assert {r["n"] for r in recs} == {26, 28, 30}
    for r in recs:
        n = r["n"]
        U = haar_unitary(2 * n, r["seed"])
        assert abs(U[0, 0] - complex(*r["U00"])) <= 1e-12, "matrix generator changed"
        S = np.zeros((1, 2 * n), dtype=np.int32)
        S[0, :n] = 1
        T = np.array([r["T"]], dtype=np.int32)
        ref = complex(r["dd"][0], r["dd"][1]) + complex(r["dd"][2], r["dd"][3])
        for mode in (_native.FLOAT_PAIRS, _native.FP64):
            prev = _native.perm_arithmetic(mode)
            try:
                got = _native.perm_batch(U, S, T, _native.GLYNN)[0]
            finally:
                _native.perm_arithmetic(prev)
            assert abs(got - ref) <= 1e-10 * abs(ref), (n, r["pattern"], mode, abs(got - ref) / abs(ref))


@pytest.mark.parametrize("n", [26, 28, 30])
def test_benchmark_batches_against_double_double_fixture(n):
    """The benchmark's own C2 batches (64 patterns per call, bench.c2_patterns with
    the benchmark's seed): every pattern of the double-double fixture within 1e-10,
    for Glynn in both arithmetics and for Chin-Huh (which sweeps the input side)
    in both.  Sharing one launch among many permanents gives every thread a longer
    code range, so this is the case that bounds a thread's accumulated rounding."""
    import json
    import os

    import bench
    from conftest import ROOT
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    recs = [r for r in json.load(open(os.path.join(ROOT, "tests", "golden", "c2_dd_large.json"))) if r["n"] == n]
    assert recs
    seed = recs[0]["seed"]
    U = haar_unitary(2 * n, seed)
    assert abs(U[0, 0] - complex(*recs[0]["U00"])) <= 1e-12, "matrix generator changed"
    T = bench.c2_patterns(n, 64, seed)
    for r in recs:
        assert T[r["pattern"]].tolist() == r["T"], "pattern generator changed"
    S = np.zeros_like(T)
    S[:, :n] = 1
    for variant, count in ((_native.GLYNN, 64), (_native.CHIN_HUH, 64 if n < 30 else 16)):
        for mode in (_native.FP64, _native.FLOAT_PAIRS):
            prev = _native.perm_arithmetic(mode)
            try:
                got = _native.perm_batch(U, S[:count], T[:count], variant)
            finally:
                _native.perm_arithmetic(prev)
            for r in recs:
                ref = complex(r["dd"][0], r["dd"][1]) + complex(r["dd"][2], r["dd"][3])
                err = abs(got[r["pattern"]] - ref) / abs(ref)
                assert err <= 1e-10, (n, variant, mode, r["pattern"], err)
