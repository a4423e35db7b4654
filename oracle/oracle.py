"""Test infrastructure, not product code.

ctypes front end of the CPU restatement in ``oracle/boss_oracle.c`` plus the
numpy-level pieces of theboss's samplers that decide *which* random numbers are
drawn (they must call numpy's global RandomState in exactly the reference's
order).  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference leg use this module, always to check results or as the CPU
baseline, never as the thing being measured on the GPU.

Reference files followed (paths inside theboss):
  - theboss/boson_sampling_utilities/permanent_calculators/*.py   (via boss_oracle.c)
  - theboss/simulation_strategies/generalized_cliffords_b_simulation_strategy.py:94-110
  - theboss/simulation_strategies/generalized_cliffords_b_uniform_losses_simulation_strategy.py:50-121
  - theboss/distribution_calculators/bs_distribution_calculator_with_fixed_losses.py:84-169
  - theboss/distribution_calculators/bs_exact_distribution_with_uniform_losses.py:42-104
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from typing import List, Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libboss_oracle.so")
_SRC = os.path.join(_HERE, "boss_oracle.c")

RYSER, CHIN_HUH, GLYNN, CLASSIC = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compiles the C restatement (gcc, no FMA contraction, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(
            ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-o", tmp, _SRC, "-lm"]
        )
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        for name in (
            "oracle_perm_ryser",
            "oracle_perm_chin_huh",
            "oracle_perm_glynn",
            "oracle_perm_classic",
            "oracle_submatrices_ryser",
            "oracle_submatrices_chin_huh",
            "oracle_dd_perm",
            "oracle_dd_submatrices",
        ):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [dp, ctypes.c_int, ip, ip, ctypes.c_int, dp]
        L.oracle_gccb_step.restype = ctypes.c_int
        L.oracle_gccb_step.argtypes = [dp, ctypes.c_int, ip, ip, ctypes.c_double, dp]
        L.oracle_gccb_run.restype = ctypes.c_int
        L.oracle_gccb_run.argtypes = [
            dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ip, dp, ctypes.POINTER(ctypes.c_int64)
        ]
        L.oracle_perm_batch.restype = ctypes.c_int
        L.oracle_perm_batch.argtypes = [dp, ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_guan_sequence.restype = ctypes.c_long
        L.oracle_guan_sequence.argtypes = [ip, ctypes.c_int, ip, ip, ctypes.c_long]
        L.oracle_set_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """Threads of the OpenMP sample loop (gccb_run), overriding an inherited
    OMP_NUM_THREADS (torchrun sets 1); returns the count in force."""
    return int(lib().oracle_set_threads(int(n)))


def _mat(U) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(U, dtype=np.complex128))


def _occ(v, m: int) -> np.ndarray:
    a = np.zeros(m, dtype=np.int32)
    v = np.asarray(v)
    a[: len(v)] = np.rint(v.astype(np.float64)).astype(np.int32) if len(v) else []
    return a


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


_PERM_FN = {RYSER: "oracle_perm_ryser", CHIN_HUH: "oracle_perm_chin_huh", GLYNN: "oracle_perm_glynn",
            CLASSIC: "oracle_perm_classic"}


def perm(U, S: Sequence[int], T: Sequence[int], variant: int = RYSER) -> complex:
    """FP64 permanent following the reference calculator named by ``variant``."""
    U = _mat(U)
    m = U.shape[0]
    if len(S) != len(T):
        raise AttributeError("input and output state lengths differ")
    n = len(S)
    s, t = _occ(S, n), _occ(T, n)
    out = np.zeros(2)
    rc = getattr(lib(), _PERM_FN[variant])(_dp(U), m, _ip(s), _ip(t), n, _dp(out))
    if rc == 1:
        raise AttributeError("size mismatch")
    if rc:
        raise ValueError(f"oracle rc={rc}")
    return complex(out[0], out[1])


def perm_batch(U, S: np.ndarray, T: np.ndarray, variant: int = RYSER) -> np.ndarray:
    """perm() of every row pair of the occupation arrays S and T (count x len):
    the same values, one call (oracle_perm_batch)."""
    U = _mat(U)
    S = np.ascontiguousarray(S, dtype=np.int32)
    T = np.ascontiguousarray(T, dtype=np.int32)
    if S.shape != T.shape:
        raise AttributeError("input and output state lengths differ")
    count, n = S.shape
    out = np.zeros(2 * count)
    rc = lib().oracle_perm_batch(_dp(U), U.shape[0], _ip(S), _ip(T), n, count, variant, _dp(out))
    if rc == 1:
        raise AttributeError("size mismatch")
    if rc:
        raise ValueError(f"oracle rc={rc}")
    return out.view(np.complex128)


def perm_dd(U, S, T) -> Tuple[complex, complex]:
    """Double-double permanent: returns (hi, lo) complex parts; value = hi + lo."""
    U = _mat(U)
    n = len(S)
    s, t = _occ(S, n), _occ(T, n)
    out = np.zeros(4)
    rc = lib().oracle_dd_perm(_dp(U), U.shape[0], _ip(s), _ip(t), n, _dp(out))
    if rc:
        raise ValueError(f"oracle rc={rc}")
    return complex(out[0], out[2]), complex(out[1], out[3])


def submatrices(U, S, T, variant: int = RYSER) -> List[complex]:
    U = _mat(U)
    n = len(S)
    s, t = _occ(S, n), _occ(T, n)
    out = np.zeros(2 * n)
    fn = lib().oracle_submatrices_ryser if variant == RYSER else lib().oracle_submatrices_chin_huh
    rc = fn(_dp(U), U.shape[0], _ip(s), _ip(t), n, _dp(out))
    if rc:
        raise ValueError(f"oracle rc={rc}")
    return [complex(out[2 * i], out[2 * i + 1]) for i in range(n)]


def submatrices_dd(U, S, T) -> List[complex]:
    U = _mat(U)
    n = len(S)
    s, t = _occ(S, n), _occ(T, n)
    out = np.zeros(4 * n)
    rc = lib().oracle_dd_submatrices(_dp(U), U.shape[0], _ip(s), _ip(t), n, _dp(out))
    if rc:
        raise ValueError(f"oracle rc={rc}")
    return [complex(out[4 * i] + out[4 * i + 1], out[4 * i + 2] + out[4 * i + 3]) for i in range(n)]


def guan_sequence(S: Sequence[int]) -> Tuple[np.ndarray, np.ndarray]:
    s = np.asarray(S, dtype=np.int32)
    total = int(np.prod(s.astype(np.int64) + 1))
    idx = np.zeros(total, dtype=np.int32)
    r = np.zeros((total, len(s)), dtype=np.int32)
    c = lib().oracle_guan_sequence(_ip(s), len(s), _ip(idx), _ip(r), total)
    assert c == total
    return idx, r


def gccb_step(U, S, T, u: float) -> Tuple[int, np.ndarray]:
    U = _mat(U)
    m = U.shape[0]
    s, t = _occ(S, m), _occ(T, m)
    pmf = np.zeros(m)
    o = lib().oracle_gccb_step(_dp(U), m, _ip(s), _ip(t), float(u), _dp(pmf))
    return int(o), pmf


# ----------------------------------------------------------------------------
# Random-stream replay in the reference's call order (numpy global RandomState).
# ----------------------------------------------------------------------------
def binomial_weights(n: int, eta: float) -> List[float]:
    """generalized_cliffords_b_uniform_losses_simulation_strategy.py:50-65."""
    from scipy.special import binom

    return [binom(n, l) * pow(eta, l) * pow(1 - eta, n - l) for l in range(n + 1)]


def predraw_gccb(input_state: Sequence[int], samples_number: int, weights: Optional[Sequence[float]] = None):
    """Draws, from numpy's global RandomState, every number the reference GCC-B
    sampler would draw for ``samples_number`` samples, in the same order.

    Returns (L, add_mode, uniform): per-sample particle counts, the input mode of
    the particle popped at each step, and the uniform numpy.random.choice uses.
    ``weights`` None means lossless GCC-B (every particle kept).
    """
    particles = []
    for i, v in enumerate(input_state):
        particles += [i] * int(v)
    n = len(particles)
    Ls, adds, us = [], [], []
    for _ in range(samples_number):
        if weights is None:
            L = n
        else:  # generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-85
            L, acc, thr = 0, 0, np.random.random()
            for w in weights:
                acc += w
                if acc > thr:
                    break
                L += 1
        work = list(particles)
        a, u = [], []
        for _k in range(L):  # generalized_cliffords_b_simulation_strategy.py:97-110
            a.append(work.pop(np.random.randint(0, len(work))))
            u.append(np.random.random_sample())
        Ls.append(L)
        adds.append(a)
        us.append(u)
    maxL = max([1] + Ls)
    A = np.zeros((samples_number, maxL), dtype=np.int32)
    Uu = np.zeros((samples_number, maxL), dtype=np.float64)
    for s in range(samples_number):
        A[s, : Ls[s]] = adds[s]
        Uu[s, : Ls[s]] = us[s]
    return np.asarray(Ls, dtype=np.int32), A, Uu


def gccb_run(U, L, A, Uu) -> np.ndarray:
    """All samples from a pre-drawn stream (C restatement, OpenMP over samples)."""
    U = _mat(U)
    m = U.shape[0]
    N, maxL = A.shape
    out = np.zeros((N, m), dtype=np.int64)
    L = np.ascontiguousarray(L, dtype=np.int32)
    A = np.ascontiguousarray(A, dtype=np.int32)
    Uu = np.ascontiguousarray(Uu, dtype=np.float64)
    rc = lib().oracle_gccb_run(
        _dp(U), m, N, maxL, _ip(L), _ip(A), _dp(Uu), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    )
    if rc:
        raise ValueError("probabilities contain NaN")
    return out


def choice_from_minors(U, S, sub, u: float) -> int:
    """One C&C-B draw from given minors: the Laplace expansion, |.|^2 and the
    normalisation of generalized_cliffords_b_simulation_strategy.py:82-92 in
    Python floats, then numpy.random.choice's rule (cumsum, divided by the last
    entry, searchsorted 'right')."""
    U = _mat(U)
    m = U.shape[0]
    pmf = []
    for o in range(m):
        p = 0j
        for i in range(m):
            p += S[i] * sub[i] * U[o][i]
        pmf.append(abs(p) ** 2)
    total = sum(pmf)
    cdf = np.cumsum([v / total for v in pmf])
    cdf /= cdf[-1]
    return min(int(np.searchsorted(cdf, u, side="right")), m - 1)


def classify_mismatches(U, L, A, Uu, got, ref, max_check: int = 4) -> dict:
    """Compares GPU samples `got` with the oracle's `ref` for the same pre-drawn
    stream (predraw_gccb's L, A, Uu).  theboss's Ryser-form minors carry rounding
    errors (about 1e-10 relative at 20 particles), so a uniform that falls that
    close to a cdf step can be decided by the rounding.  Each differing sample (up
    to max_check) is re-sampled with minors from the double-double evaluator
    (accurate to far below 1e-15): `oracle_near_ties` counts samples the GPU draws
    as the accurate minors do; `gpu_disagrees_with_double_double` counts the rest
    and every differing sample left unchecked."""
    U = _mat(U)
    m = U.shape[0]
    got = np.asarray(got)
    bad = np.nonzero((got != np.asarray(ref)).any(axis=1))[0]
    rep = {"samples": int(len(got)), "mismatches": int(len(bad)), "oracle_near_ties": 0,
           "gpu_disagrees_with_double_double": 0}
    for s in bad[:max_check]:
        S = np.zeros(m, dtype=np.int32)
        T = np.zeros(m, dtype=np.int32)
        for k in range(int(L[s])):
            S[int(A[s, k])] += 1
            T[choice_from_minors(U, S, submatrices_dd(U, list(S), list(T)), float(Uu[s, k]))] += 1
        if np.array_equal(T, got[s]):
            rep["oracle_near_ties"] += 1
        else:
            rep["gpu_disagrees_with_double_double"] += 1
    rep["gpu_disagrees_with_double_double"] += max(0, len(bad) - max_check)
    return rep


def gccb_simulate(U, input_state, samples_number: int, transmissivity: Optional[float] = None) -> np.ndarray:
    """Reference-order GCC-B (uniform losses when ``transmissivity`` is given)."""
    n = int(sum(int(v) for v in input_state))
    w = None if transmissivity is None else binomial_weights(n, transmissivity)
    L, A, Uu = predraw_gccb(input_state, samples_number, w)
    return gccb_run(U, L, A, Uu)


# ----------------------------------------------------------------------------
# Exact distributions (small cases): the reference's fixed/uniform-loss
# distribution calculators restated with oracle permanents.
# ----------------------------------------------------------------------------
def _states(n: int, m: int) -> List[Tuple[int, ...]]:
    """All n-particle m-mode states in the reference's order
    (boson_sampling_utilities.py generate_possible_states / _generate_possible_n_particle_states)."""
    if n == 0:
        return [tuple([0] * m)]
    out = []
    state = [0] * m
    state[0] = n
    out.append(tuple(state))
    while state[-1] != n:
        k = m - 1
        while state[k - 1] == 0:
            k -= 1
        state[k - 1] -= 1
        state[k:] = [0] * (m - k)
        state[k] = n - sum(state[:k])
        out.append(tuple(state))
    return sorted(out, reverse=True)


def lossy_inputs(initial: Sequence[int], left: int) -> List[Tuple[int, ...]]:
    """Distinct sub-occupations of ``initial`` with ``left`` particles."""
    res = []

    def rec(i, rem, cur):
        if i == len(initial):
            if rem == 0:
                res.append(tuple(cur))
            return
        for k in range(min(initial[i], rem), -1, -1):
            rec(i + 1, rem - k, cur + [k])

    rec(0, left, [])
    return res


def fixed_loss_probability(U, initial, outcome, variant: int = CHIN_HUH) -> float:
    """bs_distribution_calculator_with_fixed_losses.py:84-151."""
    from scipy.special import binom

    left = int(sum(outcome))
    n = int(sum(initial))
    p = 0.0
    for li in lossy_inputs(initial, left):
        mult = 1
        for i in range(len(li)):
            mult *= binom(initial[i], initial[i] - li[i])
        sub = abs(perm(U, li, outcome, variant)) ** 2
        for v in li:
            sub /= math.factorial(v)
        p += sub * int(mult)
    p /= math.factorial(left)
    p /= binom(n, left)
    p *= math.factorial(left)
    for v in outcome:
        p /= math.factorial(v)
    return p


def uniform_loss_distribution(U, initial, eta: float, variant: int = CHIN_HUH) -> List[float]:
    """bs_exact_distribution_with_uniform_losses.py:42-104 over all lossy outcomes."""
    from scipy.special import binom

    n = int(sum(initial))
    m = len(initial)
    weights = [pow(eta, l) * binom(n, l) * pow(1.0 - eta, n - l) for l in range(n + 1)]
    out = []
    for left in range(n + 1):
        for st in _states(left, m):
            if left == 0:
                out.append(weights[0])
            else:
                out.append(fixed_loss_probability(U, initial, st, variant) * weights[left])
    return out
