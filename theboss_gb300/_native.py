"""ctypes binding of libboss_gb300.so (the C ABI declared in include/boss.h).

The library is built in-tree by ``theboss_gb300.build``.  There is no CPU
fallback: when the library cannot be loaded, or no GPU is present, the calls
raise instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

BOSS_OK = 0
BOSS_ERR_SIZE = 1
BOSS_ERR_LIMIT = 2
BOSS_ERR_CUDA = 3
BOSS_ERR_ARG = 4
BOSS_ERR_PMF = 5
BOSS_ERR_NODEVICE = 6

RYSER, CHIN_HUH, GLYNN, CLASSIC = 0, 1, 2, 3

_lock = threading.Lock()
_lib = None


class GB300Error(RuntimeError):
    """A CUDA or library failure inside libboss_gb300.so."""


def load() -> ctypes.CDLL:
    """Loads the in-tree library (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not _build.up_to_date():
            path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.boss_last_error.restype = ctypes.c_char_p
        L.boss_last_error.argtypes = []
        L.boss_abi_version.restype = ctypes.c_int
        L.boss_select_device.restype = ctypes.c_int
        L.boss_select_device.argtypes = [ctypes.c_int32]
        L.boss_device_sm_count.restype = ctypes.c_int
        L.boss_device_sm_count.argtypes = [ip]
        for name in ("boss_perm_batch", "boss_submatrices_batch"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [dp, ctypes.c_int32, ip, ip, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp]
        L.boss_perm_batch_noalloc.restype = ctypes.c_int
        L.boss_perm_batch_noalloc.argtypes = [dp, ctypes.c_int32, ip, ip, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        L.boss_perm_grad_batch.restype = ctypes.c_int
        L.boss_perm_grad_batch.argtypes = [dp, ctypes.c_int32, ip, ip, ctypes.c_int32, ctypes.c_int32, dp, dp]
        L.boss_fp64_peak.restype = ctypes.c_int
        L.boss_fp64_peak.argtypes = [dp, dp]
        L.boss_fp32_peak.restype = ctypes.c_int
        L.boss_fp32_peak.argtypes = [dp, dp]
        up = ctypes.POINTER(ctypes.c_uint32)
        L.boss_gccb_predraw.restype = ctypes.c_int
        L.boss_gccb_predraw.argtypes = [ip, ctypes.c_int32, dp, ctypes.c_int32, up, ip, ctypes.c_int32, ip, ip, dp]
        L.boss_gccb_sample.restype = ctypes.c_int
        L.boss_gccb_sample.argtypes = [dp, ctypes.c_int32, ip, dp, ctypes.c_int32, up, ip, ctypes.c_int32, ip]
        L.boss_gccb_bench.restype = ctypes.c_int
        L.boss_gccb_bench.argtypes = [dp, ctypes.c_int32, ip, dp, ctypes.c_int32, up, ip, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, dp, dp, dp, ip]
        L.boss_perm_bench.restype = ctypes.c_int
        L.boss_perm_bench.argtypes = [dp, ctypes.c_int32, ip, ip, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, dp, dp, dp]
        L.boss_lossy_probabilities.restype = ctypes.c_int
        L.boss_lossy_probabilities.argtypes = [dp, ctypes.c_int32, ip, ip, ctypes.c_int32, dp,
                                               ctypes.POINTER(ctypes.c_float)]
        L.boss_count_outcomes.restype = ctypes.c_int
        L.boss_count_outcomes.argtypes = [ip, ctypes.c_int64, ip, ctypes.c_int64, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_int64)]
        L.boss_gccb_sample_instances.restype = ctypes.c_int
        L.boss_gccb_sample_instances.argtypes = [dp, ctypes.c_int32, ctypes.c_int32, ip, ctypes.c_int32, ip, dp,
                                                 ctypes.c_int32, ip]
        L.boss_bobs_uniform_predraw.restype = ctypes.c_int
        L.boss_bobs_uniform_predraw.argtypes = [up, ip, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ip, dp,
                                                ctypes.c_int32, ip, dp, ctypes.c_int32, ctypes.c_int32, ip, dp, ip,
                                                ip, dp]
        L.boss_bobs_nonuniform_predraw.restype = ctypes.c_int
        L.boss_bobs_nonuniform_predraw.argtypes = [up, ip, ctypes.c_int32, ctypes.c_int32, ip, ctypes.c_int32,
                                                   ctypes.c_int32, dp, ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.c_int32, ip, dp, ip, dp]
        L.boss_gccb_sample_slice.restype = ctypes.c_int
        L.boss_gccb_sample_slice.argtypes = [dp, ctypes.c_int32, ip, dp, ctypes.c_int32, up, ip, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_int32, ip]
        L.boss_perm_arithmetic.restype = ctypes.c_int
        L.boss_perm_arithmetic.argtypes = [ctypes.c_int32, ip]
        L.boss_minors_arithmetic.restype = ctypes.c_int
        L.boss_minors_arithmetic.argtypes = [ctypes.c_int32, ip]
        L.boss_gccb_autotune.restype = ctypes.c_int
        L.boss_gccb_autotune.argtypes = [dp, ctypes.c_int32, ip, dp, ctypes.c_int32, up, ip, ctypes.c_int32,
                                         ctypes.c_int32, dp]
        L.boss_gccb_near_ties.restype = ctypes.c_int
        L.boss_gccb_near_ties.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]
        _lib = L
        return L


def library_path() -> str:
    return _build.LIB


def check(status: int) -> None:
    if status == BOSS_OK:
        return
    msg = load().boss_last_error().decode(errors="replace")
    if status == BOSS_ERR_SIZE:
        raise AttributeError(msg)
    if status == BOSS_ERR_PMF:
        raise ValueError(msg)
    if status == BOSS_ERR_ARG:
        raise ValueError(msg)
    raise GB300Error(f"libboss_gb300 status {status}: {msg}")


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def as_matrix(matrix) -> np.ndarray:
    U = np.asarray(matrix)
    if U.dtype != np.complex128 or not U.flags.c_contiguous:
        U = np.ascontiguousarray(U, dtype=np.complex128)
    if U.ndim != 2:
        raise AttributeError("matrix must be two-dimensional")
    return U


def as_states(states, length: int) -> np.ndarray:
    """Occupation vectors (ints or integer-valued floats) -> int32 array."""
    a = np.asarray(states)
    if a.dtype.kind == "f":
        a = np.rint(a)
    return np.ascontiguousarray(a, dtype=np.int32).reshape(-1, length)


def perm_batch(U: np.ndarray, S: np.ndarray, T: np.ndarray, variant: int) -> np.ndarray:
    """Permanents of U[T_k, S_k]; S, T int32 (count x len).  Returns complex128 (count,)."""
    U = as_matrix(U)
    L = load()
    count, n = S.shape
    out = np.empty(count, dtype=np.complex128)
    if count == 0:
        return out
    check(L.boss_perm_batch(_dp(U.view(np.float64)), U.shape[0], _ip(S), _ip(T), n, count, variant,
                            _dp(out.view(np.float64))))
    return out


def perm_grad_batch(U: np.ndarray, S: np.ndarray, T: np.ndarray):
    """Permanents of U[T_k, S_k] and d perm_k / d U[j][i] (count x len x len)."""
    U = as_matrix(U)
    L = load()
    count, n = S.shape
    perms = np.empty(count, dtype=np.complex128)
    grads = np.empty((count, n, n), dtype=np.complex128)
    if count == 0:
        return perms, grads
    check(L.boss_perm_grad_batch(_dp(U.view(np.float64)), U.shape[0], _ip(S), _ip(T), n, count,
                                 _dp(perms.view(np.float64)), _dp(grads.view(np.float64))))
    return perms, grads


def submatrices_batch(U: np.ndarray, S: np.ndarray, T: np.ndarray, variant: int) -> np.ndarray:
    """All-minors permanents; returns complex128 (count x len)."""
    U = as_matrix(U)
    L = load()
    count, n = S.shape
    out = np.empty((count, n), dtype=np.complex128)
    if count == 0:
        return out
    check(L.boss_submatrices_batch(_dp(U.view(np.float64)), U.shape[0], _ip(S), _ip(T), n, count, variant,
                                   _dp(out.view(np.float64))))
    return out


def perm_batch_noalloc(U: np.ndarray, S: np.ndarray, T: np.ndarray, variant: int, results_device_ptr: int,
                       stream_ptr: int = 0) -> None:
    """Queues the permanents of U[T_k, S_k] into a caller-owned device buffer of
    count complex128 without any GPU allocation (boss_perm_batch_noalloc).  The
    caller synchronises the stream before reading the buffer."""
    U = as_matrix(U)
    L = load()
    count, n = S.shape
    check(L.boss_perm_batch_noalloc(_dp(U.view(np.float64)), U.shape[0], _ip(S), _ip(T), n, count, variant,
                                    ctypes.c_void_p(int(results_device_ptr)), ctypes.c_void_p(int(stream_ptr))))


def lossy_probabilities(U: np.ndarray, initial_state, outcomes, timed: bool = False):
    """Probability of each outcome with sum(outcome) of the initial particles
    surviving (theboss's fixed-loss formula, boss_lossy_probabilities).  Returns a
    float64 array, and the GPU kernel milliseconds when `timed`."""
    L = load()
    U = as_matrix(U)
    m = U.shape[0]
    S = np.ascontiguousarray(np.rint(np.asarray(initial_state, dtype=np.float64)).astype(np.int32))
    T = np.asarray(outcomes)
    if T.dtype.kind in "iu":
        T = np.ascontiguousarray(T, dtype=np.int32).reshape(-1, m)
    else:  # integer-valued floats or sequences
        T = np.ascontiguousarray(np.rint(np.asarray(outcomes, dtype=np.float64)).astype(np.int32).reshape(-1, m))
    if len(S) != m:
        raise AttributeError("initial state length differs from the matrix dimension")
    out = np.zeros(T.shape[0], dtype=np.float64)
    ms = ctypes.c_float(0.0)
    check(L.boss_lossy_probabilities(_dp(U.view(np.float64)), m, _ip(S), _ip(T), T.shape[0], _dp(out),
                                     ctypes.byref(ms)))
    return (out, float(ms.value)) if timed else out


def _state_rows(states, m: int) -> np.ndarray:
    a = np.asarray(states)
    if a.size == 0:
        return np.zeros((0, m), dtype=np.int32)
    if a.dtype.kind not in "iu":
        a = np.rint(np.asarray(a, dtype=np.float64))
    return np.ascontiguousarray(a, dtype=np.int32).reshape(-1, m)


def count_outcomes(samples, outcomes, m: int) -> np.ndarray:
    """For each listed outcome, how many samples equal it (the first listed copy of
    a repeated outcome gets the counts); boss_count_outcomes.  int64 array."""
    L = load()
    S = _state_rows(samples, m)
    O = _state_rows(outcomes, m)
    out = np.zeros(O.shape[0], dtype=np.int64)
    check(L.boss_count_outcomes(_ip(S), S.shape[0], _ip(O), O.shape[0], m,
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
    return out


def gccb_sample_slice(U: np.ndarray, input_state, weights, n_samples: int, first: int, count: int) -> np.ndarray:
    """Samples [first, first + count) of the stream of n_samples C&C-B samples;
    numpy's global RandomState advances over the whole stream.  int32 (count x m)."""
    U = as_matrix(U)
    L = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    m = U.shape[0]
    if len(inp) != m:
        raise AttributeError("input state length differs from the matrix dimension")
    w, nw, wp = _weights_arg(weights)
    st, key, pos = _get_mt()
    out = np.zeros((max(count, 0), m), dtype=np.int32)
    check(L.boss_gccb_sample_slice(_dp(U.view(np.float64)), m, _ip(inp), wp, nw,
                                   key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _ip(pos), n_samples, first,
                                   count, _ip(out)))
    _set_mt(st, key, pos)
    return out


def gccb_sample_instances(matrices: np.ndarray, input_states: np.ndarray, randint_results: np.ndarray,
                          uniforms: np.ndarray) -> np.ndarray:
    """One lossless C&C-B sample per (matrix, input) instance with pre-drawn numbers
    (boss_gccb_sample_instances).  matrices: (m, m) shared or (N, m, m).  Returns
    int32 (N x m)."""
    L = load()
    Mx = np.ascontiguousarray(matrices, dtype=np.complex128)
    m = Mx.shape[-1]
    n_mats = 1 if Mx.ndim == 2 else Mx.shape[0]
    S = np.ascontiguousarray(input_states, dtype=np.int32).reshape(-1, m)
    N = S.shape[0]
    R = np.ascontiguousarray(randint_results, dtype=np.int32).reshape(N, -1)
    Uu = np.ascontiguousarray(uniforms, dtype=np.float64).reshape(N, -1)
    stride = R.shape[1]
    if Uu.shape[1] != stride:
        raise ValueError("randint results and uniforms need the same row length")
    out = np.zeros((N, m), dtype=np.int32)
    check(L.boss_gccb_sample_instances(_dp(Mx.view(np.float64)), n_mats, m, _ip(S), N, _ip(R), _dp(Uu), stride,
                                       _ip(out)))
    return out


def _up(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def bobs_uniform_predraw(n_samples: int, m: int, k: int, exact_parts, exact_weights, approx_parts, approx_weights,
                         stride: int):
    """Random numbers of the uniform-loss BOBS strategy from numpy's global
    RandomState (advanced as theboss advances it).  Returns (inputs, phase
    uniforms, permutations, randint results, uniforms)."""
    L = load()
    st, key, pos = _get_mt()
    E = np.ascontiguousarray(exact_parts, dtype=np.int32).reshape(-1, max(k, 0)) if k else np.zeros(
        (len(exact_weights), 0), dtype=np.int32)
    A = np.ascontiguousarray(approx_parts, dtype=np.int32).reshape(len(approx_weights), m - k)
    ew = np.ascontiguousarray(exact_weights, dtype=np.float64)
    aw = np.ascontiguousarray(approx_weights, dtype=np.float64)
    inputs = np.zeros((n_samples, m), dtype=np.int32)
    ph = np.zeros((n_samples, max(m - k, 1)), dtype=np.float64)
    perms = np.zeros((n_samples, m), dtype=np.int32)
    ri = np.zeros((n_samples, max(stride, 1)), dtype=np.int32)
    uu = np.zeros((n_samples, max(stride, 1)), dtype=np.float64)
    check(L.boss_bobs_uniform_predraw(_up(key), _ip(pos), n_samples, m, k, _ip(np.ascontiguousarray(E)), _dp(ew),
                                      len(ew), _ip(A), _dp(aw), len(aw), max(stride, 1), _ip(inputs), _dp(ph),
                                      _ip(perms), _ip(ri), _dp(uu)))
    _set_mt(st, key, pos)
    return inputs, ph[:, :m - k], perms, ri, uu


def bobs_nonuniform_predraw(n_samples: int, base_state, approximated_modes: int, approximated_particles: int,
                            loss_weights, lossy: bool, stride: int):
    """Random numbers of the non-uniform-loss BOBS strategy from numpy's global
    RandomState.  loss_weights: square table, row o = weights of 0..o survivors.
    Returns (inputs, phase uniforms, randint results, uniforms)."""
    L = load()
    st, key, pos = _get_mt()
    base = np.ascontiguousarray(base_state, dtype=np.int32)
    m = len(base)
    W = np.ascontiguousarray(loss_weights, dtype=np.float64)
    inputs = np.zeros((n_samples, m), dtype=np.int32)
    ph = np.zeros((n_samples, max(approximated_modes, 1)), dtype=np.float64)
    ri = np.zeros((n_samples, max(stride, 1)), dtype=np.int32)
    uu = np.zeros((n_samples, max(stride, 1)), dtype=np.float64)
    check(L.boss_bobs_nonuniform_predraw(_up(key), _ip(pos), n_samples, m, _ip(base), approximated_modes,
                                         approximated_particles, _dp(W), W.shape[0] - 1, int(bool(lossy)),
                                         max(stride, 1), _ip(inputs), _dp(ph), _ip(ri), _dp(uu)))
    _set_mt(st, key, pos)
    return inputs, ph[:, :approximated_modes], ri, uu


def fp64_peak():
    """(TFLOP/s, ms) of the FP64 FMA microbenchmark on the current GPU."""
    L = load()
    t = np.zeros(1)
    ms = np.zeros(1)
    check(L.boss_fp64_peak(_dp(t), _dp(ms)))
    return float(t[0]), float(ms[0])


FLOAT_PAIRS = 0  # float pairs on the FP32 pipe (opt-in)
FP64 = 1         # FP64 (the default, theboss's float64)


def minors_arithmetic(mode: int = -1) -> int:
    """Sets the arithmetic of the all-minors sweeps and of the batched sampler's
    pmf (FP64, the default, or FLOAT_PAIRS; -1 only queries) and returns the
    previous one."""
    prev = np.zeros(1, dtype=np.int32)
    check(load().boss_minors_arithmetic(int(mode), _ip(prev)))
    return int(prev[0])


def fp32_peak():
    """(T FP32 FMA instructions/s, ms) of an FFMA stream on the current device."""
    t = np.zeros(1)
    ms = np.zeros(1)
    check(load().boss_fp32_peak(_dp(t), _dp(ms)))
    return float(t[0]), float(ms[0])


def perm_arithmetic(mode: int = -1) -> int:
    """Sets the arithmetic of the single-permanent sweeps (FP64, the default, or
    FLOAT_PAIRS; -1 only queries) and returns the previous one."""
    prev = np.zeros(1, dtype=np.int32)
    check(load().boss_perm_arithmetic(int(mode), _ip(prev)))
    return int(prev[0])


def gccb_autotune(U: np.ndarray, input_state, weights, n_samples: int, reps: int = 3) -> dict:
    """Tunes the sampler's launch shapes on the workload of gccb_sample(U,
    input_state, weights, n_samples) drawn from numpy's current global state
    (which is not advanced); boss_gccb_autotune."""
    U = as_matrix(U)
    L = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    m = U.shape[0]
    w, nw, wp = _weights_arg(weights)
    _, key, pos = _get_mt()
    rep = np.zeros(8)
    check(L.boss_gccb_autotune(_dp(U.view(np.float64)), m, _ip(inp), wp, nw,
                               key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _ip(pos), n_samples, reps,
                               _dp(rep)))
    return {"default_step_ms": float(rep[0]), "tuned_step_ms": float(rep[1]), "levels_changed": int(rep[2]),
            "pipeline_shift": int(rep[3]), "pipeline_growth": int(rep[7]), "e2e_default_split_ms": float(rep[4]),
            "e2e_tuned_split_ms": float(rep[5]), "levels_sum_ms": float(rep[6])}


def gccb_near_ties(reset: bool = False) -> int:
    """Draws of the batched sampler decided by the exact sequential rule because a
    cdf step lay within the pmf's error bound of the uniform (boss_gccb_near_ties),
    counted since the last reset."""
    v = ctypes.c_int64(0)
    check(load().boss_gccb_near_ties(ctypes.byref(v), int(bool(reset))))
    return int(v.value)


def select_device(device: int) -> None:
    check(load().boss_select_device(int(device)))


def sm_count() -> int:
    L = load()
    v = np.zeros(1, dtype=np.int32)
    check(L.boss_device_sm_count(_ip(v)))
    return int(v[0])


# ---------------------------------------------------------------------------
# numpy's global legacy RandomState <-> the library's MT19937 replay
# ---------------------------------------------------------------------------
def _get_mt():
    st = np.random.get_state()
    if st[0] != "MT19937":
        raise ValueError("numpy's global generator is not MT19937")
    key = np.array(st[1], dtype=np.uint32, copy=True)
    pos = np.array([st[2]], dtype=np.int32)
    return st, key, pos


def _set_mt(st, key, pos) -> None:
    np.random.set_state((st[0], key, int(pos[0]), st[3], st[4]))


def _weights_arg(weights):
    if weights is None:
        return None, 0, None
    w = np.ascontiguousarray(weights, dtype=np.float64)
    return w, len(w), _dp(w)


def gccb_predraw(input_state, weights, n_samples: int):
    """Replays, without a GPU, the numbers theboss's C&C-B sampler draws from numpy's
    global RandomState and advances that state the same way.  Returns
    (particles_kept, popped_modes, uniforms)."""
    L = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    n = int(inp.sum())
    w, nw, wp = _weights_arg(weights)
    st, key, pos = _get_mt()
    kept = np.zeros(n_samples, dtype=np.int32)
    popped = np.zeros((n_samples, max(n, 1)), dtype=np.int32)
    uni = np.zeros((n_samples, max(n, 1)), dtype=np.float64)
    check(L.boss_gccb_predraw(_ip(inp), len(inp), wp, nw, key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                              _ip(pos), n_samples, _ip(kept), _ip(popped), _dp(uni)))
    _set_mt(st, key, pos)
    return kept, popped[:, :n], uni[:, :n]


def gccb_sample(U: np.ndarray, input_state, weights, n_samples: int) -> np.ndarray:
    """n_samples C&C-B samples on the GPU; consumes numpy's global RandomState like
    theboss does.  Returns int32 (n_samples x m)."""
    U = as_matrix(U)
    L = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    m = U.shape[0]
    if len(inp) != m:
        raise AttributeError("input state length differs from the matrix dimension")
    w, nw, wp = _weights_arg(weights)
    st, key, pos = _get_mt()
    out = np.empty((n_samples, m), dtype=np.int32)  # every row is written
    check(L.boss_gccb_sample(_dp(U.view(np.float64)), m, _ip(inp), wp, nw,
                             key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _ip(pos), n_samples, _ip(out)))
    _set_mt(st, key, pos)
    return out


# ---------------------------------------------------------------------------
# Device-timed benchmark entry points
# ---------------------------------------------------------------------------
def gccb_bench(U: np.ndarray, input_state, weights, n_samples: int, warmup: int, steps: int,
               flush_bytes: int = 256 << 20):
    """Runs the captured sampler graph warmup + steps times on resident inputs.
    Returns dict(step_ms, sweep_ms, sweep_flops, h2d_bytes, d2h_bytes, kernels, sweeps, levels, samples)."""
    U = as_matrix(U)
    L = load()
    inp = np.ascontiguousarray(input_state, dtype=np.int32)
    m = U.shape[0]
    w, nw, wp = _weights_arg(weights)
    st, key, pos = _get_mt()
    step_ms = np.zeros(steps)
    sweep_ms = np.zeros(steps)
    info = np.zeros(8)
    samples = np.zeros((n_samples, m), dtype=np.int32)
    check(L.boss_gccb_bench(_dp(U.view(np.float64)), m, _ip(inp), wp, nw,
                            key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _ip(pos), n_samples, warmup, steps,
                            int(flush_bytes), _dp(step_ms), _dp(sweep_ms), _dp(info), _ip(samples)))
    _set_mt(st, key, pos)
    return dict(step_ms=step_ms, sweep_ms=sweep_ms, sweep_flops=float(info[0]), h2d_bytes=int(info[1]),
                d2h_bytes=int(info[2]), kernels=int(info[3]), sweeps=int(info[4]), levels=int(info[5]),
                ref_flops=float(info[6]), ff_inst=float(info[7]), samples=samples)


def perm_bench(U: np.ndarray, S: np.ndarray, T: np.ndarray, variant: int, warmup: int, steps: int,
               flush_bytes: int = 256 << 20):
    """Device-timed sweeps of a batch of permanents sharing one product size.
    Returns dict(sweep_ms, codes, flops, threads, nf, ff_inst, results)."""
    U = as_matrix(U)
    L = load()
    count, n = S.shape
    sweep_ms = np.zeros(steps)
    info = np.zeros(5)
    res = np.zeros(count, dtype=np.complex128)
    check(L.boss_perm_bench(_dp(U.view(np.float64)), U.shape[0], _ip(S), _ip(T), n, count, variant, warmup, steps,
                            int(flush_bytes), _dp(sweep_ms), _dp(info), _dp(res.view(np.float64))))
    return dict(sweep_ms=sweep_ms, codes=float(info[0]), flops=float(info[1]), threads=int(info[2]),
                nf=int(info[3]), ff_inst=float(info[4]), results=res)
