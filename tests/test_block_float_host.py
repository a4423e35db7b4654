"""Block floating point of the sweeps (theboss_gb300/csrc/boss_sweep.cuh): the
helpers compiled for the host with nvcc and checked against exact integer
arithmetic.  The bounds are the ones the sweeps rely on: normal form (larger
component in [2^61, 2^62]), exact pair products truncated once (2^-60), products
of normal values within 2^-56.5 of the product's magnitude, and one rounding to
FP64 (2^-53)."""
import math
import os
import shutil
import subprocess
from fractions import Fraction as F

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def cases(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("bf") / "block_float_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", os.path.join(HERE, "native", "block_float_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    out = []
    for seed in (7, 11):
        out += subprocess.run([exe, str(seed), "4000"], check=True, capture_output=True, text=True).stdout.splitlines()
    return out


def _normal(re, im):
    if re == 0 and im == 0:
        return True
    return abs(re) <= 2 ** 62 and abs(im) <= 2 ** 62 and max(abs(re), abs(im)) >= 2 ** 61


def _val(x):
    return F(x[0]) * F(2) ** x[2], F(x[1]) * F(2) ** x[2]


def _cmul(x, y):
    return x[0] * y[0] - x[1] * y[1], x[0] * y[1] + x[1] * y[0]


def test_block_float_bounds(cases):
    worst = {"pair": 0.0, "mul": 0.0, "to_double": 0.0}
    zeros = 0
    for line in cases:
        if line.startswith("edge"):
            continue
        parts = line.split("|")
        v = list(map(int, parts[0].split()))
        A, B, C, M, M2 = (list(map(int, p.split())) for p in parts[1:6])
        D = [float.fromhex(h) for h in parts[6].split()]
        assert all(abs(x) < 2 ** 61 for x in v)
        # exact pairs and the normalised single factor
        for (ex, got, e0) in (((v[0] * v[2] - v[1] * v[3], v[0] * v[3] + v[1] * v[2]), A, -100),
                              ((v[4] * v[6] - v[5] * v[7], v[4] * v[7] + v[5] * v[6]), B, -100),
                              ((v[0], v[1]), C, -50)):
            assert _normal(got[0], got[1]), got
            mag = max(abs(ex[0]), abs(ex[1]))
            if mag == 0:
                assert got[0] == 0 and got[1] == 0
                zeros += 1
                continue
            for c in range(2):
                err = abs(F(got[c]) * F(2) ** got[2] - F(ex[c]) * F(2) ** e0) / (F(mag) * F(2) ** e0)
                worst["pair"] = max(worst["pair"], float(err))
        assert F(C[0]) * F(2) ** (C[2] + 50) == v[0] and F(C[1]) * F(2) ** (C[2] + 50) == v[1]  # exact
        # products of normal values, relative to the exact product's magnitude
        for (X, Y, got) in ((A, B, M), (M, C, M2)):
            assert _normal(got[0], got[1]), got
            ex = _cmul(_val(X), _val(Y))
            mag2 = ex[0] ** 2 + ex[1] ** 2
            if mag2 == 0:
                assert got[0] == 0 and got[1] == 0
                continue
            g = _val(got)
            for c in range(2):
                worst["mul"] = max(worst["mul"], float(abs(g[c] - ex[c])) / math.sqrt(float(mag2)))
        g = _val(M2)
        for c in range(2):
            if g[c] == 0:
                assert D[c] == 0.0
            else:
                worst["to_double"] = max(worst["to_double"], float(abs(F(D[c]) - g[c]) / abs(g[c])))
    assert worst["pair"] < 2.0 ** -60, worst
    assert worst["mul"] < 2.0 ** -56.5, worst
    assert worst["to_double"] <= 2.0 ** -53, worst
    assert zeros > 0


def test_block_float_edges(cases):
    edge = cases[-1].split()
    assert edge[0] == "edge"
    x = 3 * 2 ** 60
    assert float.fromhex(edge[1]) == math.ldexp(float(x), -1200)  # subnormal result
    assert float.fromhex(edge[2]) == math.ldexp(float(x), 900)  # overflows to inf
    assert float.fromhex(edge[3]) == math.ldexp(-float(x), -1150)
    assert float.fromhex(edge[4]) == 0.0
