"""Benchmark of the GB300 permanent hot path (one JSON line on rank 0).

Workload (the configuration the headline metric is quoted on): generalized
Clifford & Clifford B sampling with uniform losses, transmissivity 0.5, n = 20
single photons in modes 0..19 of m = 40 modes, 10^4 samples per step, on a
seeded Haar-random 40 x 40 complex128 unitary (Mezzadri QR), numpy's global
generator seeded like theboss's own runs.  A step is one full batch of 10^4
samples through the captured sampler graph.

  value    samples/s on the GPU with the inputs (matrix, random stream) resident
           in HBM, CUDA-event timed per step, L2 flushed (256 MiB memset) between
           steps.
  e2e      samples/s through the C ABI with host buffers (boss_gccb_sample: host
           random-stream replay, H2D, graph, D2H), timed over `steps` calls after
           `warmup` untimed ones.
  roofline the all-minors sweep kernel (the dominant kernel) against the FP64 FMA
           peak measured live by boss_fp64_peak.
  plain_gpu / batched_vs_plain
           theboss's own per-step loop with the GPU all-minors calculator (one
           launch per sampling step) on a bounded number of samples.
  single_permanents
           64 permanents per size n in {16, 20, 24, 28, 30} of an m = 2n Haar
           unitary, single photons in, ~20% doubly-occupied outputs, Glynn sweep,
           device-timed, against the same FP64 peak.
  cpu_baseline
           the CPU restatement of theboss's sampler (oracle/, C + OpenMP on all
           host threads) on a bounded sample of the same workload.

--impl reference times that CPU restatement alone (theboss is pure Python; its
algorithm restated in C is the reference implementation that runs on the box).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GCC samples/s n=20,m=40 batched vs plain GPU; perms/s %FP64 peak; rel err≤10^-10".replace(
    "10^-10", "1e-10")
N_PHOTONS, N_MODES, ETA = 20, 40, 0.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=10000)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--quick", action="store_true", help="skip the single-permanent and plain-driver sections")
    ap.add_argument("--no-tune", action="store_true", help="time the heuristic launch shapes (no autotuner)")
    ap.add_argument("--case", choices=["perm", "grad", "dist", "c5"],
                    help="run one kernel case instead of the bench (for profiler captures): Glynn permanents or "
                         "permanents with all n^2 derivatives, n photons in 2n modes; c5: the full lossy-network "
                         "run (n=30 in 60 modes, 120 expanded, 2000 samples)")
    ap.add_argument("--n", type=int, default=24, help="photons of --case")
    ap.add_argument("--patterns", type=int, default=16, help="output patterns of --case")
    ap.add_argument("--arith", choices=["ff", "fp64"], default="fp64",
                    help="arithmetic of the sweeps and the sampler's pmf: FP64 (default, theboss's float64) or "
                         "float pairs on the FP32 pipe (boss_minors_arithmetic / boss_perm_arithmetic)")
    return ap.parse_args()


def set_arithmetic(args):
    from theboss_gb300 import _native

    mode = _native.FP64 if args.arith == "fp64" else _native.FLOAT_PAIRS
    _native.minors_arithmetic(mode)
    _native.perm_arithmetic(mode)


def run_case(args):
    """One warm-up call and one timed call of a single kernel case; prints a
    short JSON line (not a bench line)."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    set_arithmetic(args)
    if args.case == "c5":
        print(json.dumps(lossy_network_run(args.seed, 2000)), flush=True)
        return
    m = 2 * args.n
    U = haar_unitary(m, args.seed + args.n)
    T = c2_patterns(args.n, args.patterns, args.seed + args.n)
    S = np.zeros_like(T)
    S[:, :args.n] = 1
    if args.case == "dist":  # uniform-loss outcomes of n single photons in 2n modes
        from theboss_gb300.utilities import possible_states_array

        outs = possible_states_array(args.n, m, losses=True)
        inp = [1] * args.n + [0] * args.n
        call = lambda: _native.lossy_probabilities(U, inp, outs)  # noqa: E731
    elif args.case == "perm":
        call = lambda: _native.perm_batch(U, S, T, _native.GLYNN)  # noqa: E731
    else:
        call = lambda: _native.perm_grad_batch(U, S, T)  # noqa: E731
    call()
    t = time.perf_counter()
    call()
    dt = time.perf_counter() - t
    print(json.dumps({"case": args.case, "n": args.n, "m": m, "patterns": args.patterns, "ms": dt * 1e3}), flush=True)


def workload(seed):
    from scipy.special import binom

    from theboss_gb300.utilities import haar_unitary

    U = haar_unitary(N_MODES, seed)
    inp = np.array([1] * N_PHOTONS + [0] * (N_MODES - N_PHOTONS), dtype=np.int32)
    w = [binom(N_PHOTONS, l) * pow(ETA, l) * pow(1 - ETA, N_PHOTONS - l) for l in range(N_PHOTONS + 1)]
    return U, inp, w


def config(args, extra=None):
    c = {"workload": "GCC-B uniform losses eta=0.5, n=20 photons, m=40 modes, 10^4 samples/step, Haar unitary",
         "n": N_PHOTONS, "m": N_MODES, "eta": ETA, "samples_per_step": args.samples, "seed": args.seed,
         "l2": "flushed between timed steps (256 MiB memset)", "parallelism": f"replicas x{args.gpus}"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while a region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "20", "-i", str(self.idx)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi needs a moment to start: wait (at most 5 s) for its first sample
        # so that the region it watches is covered from the start
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(U, inp, w, seed, budget_s=10.0, gpu_samples=None):
    """theboss's sampler restated in C (oracle/) on all host threads, on a bounded
    sample of the workload sized to about budget_s seconds.  The sample starts at
    the same seed as the GPU's timed step, so its first len(gpu_samples) samples are
    the oracle's stream for the GPU's: they are compared (the parity record)."""
    from oracle import oracle as O

    cores = O.set_threads(os.cpu_count() or 1)

    def run(n):
        np.random.seed(seed)
        L, A, Uu = O.predraw_gccb(list(inp), n, w)
        t = time.perf_counter()
        out = O.gccb_run(U, L, A, Uu)
        return time.perf_counter() - t, (L, A, Uu, out)

    probe = 200
    dt, _ = run(probe)
    n = int(min(10 ** 5, max(probe, probe * budget_s / max(dt, 1e-6))))
    if gpu_samples is not None:
        n = max(n, len(gpu_samples))
    dt, (L, A, Uu, out) = run(n)
    res = {"value": n / dt, "unit": "samples/s", "cores": cores, "kind": "port",
           "sample": f"{n} samples of the workload (same seed and matrix), C restatement of theboss's "
                     f"GCC-B sampler, OpenMP over samples, {dt:.1f} s"}
    parity = None
    if gpu_samples is not None:
        N = len(gpu_samples)
        parity = O.classify_mismatches(U, L[:N], A[:N], Uu[:N], gpu_samples, out[:N])
    return res, parity


def theboss_python_line(U, inp, seed, gpu_samples, n=32):
    """theboss's own GCC-B sampler (its unmodified Python, installed in
    baseline/_ref: generalized_cliffords_b_uniform_losses_simulation_strategy.py
    with its Ryser calculator), single-threaded on the host, on the first n samples
    of the workload's stream (same seed and matrix as the GPU's timed step): its
    speed, and whether its samples equal the GPU's."""
    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "theboss")):
        return {"unavailable": "theboss is not installed in baseline/_ref"}
    sys.path.insert(0, ref)
    try:
        from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
            RyserPermanentCalculator)
        from theboss.simulation_strategies.generalized_cliffords_b_uniform_losses_simulation_strategy import (
            GeneralizedCliffordsBUniformLossesSimulationStrategy)
    finally:
        sys.path.remove(ref)
    np.random.seed(seed)
    strat = GeneralizedCliffordsBUniformLossesSimulationStrategy(RyserPermanentCalculator(U), ETA)
    t = time.perf_counter()
    out = strat.simulate(list(inp), n)
    dt = time.perf_counter() - t
    return {"value": n / dt, "unit": "samples/s", "cores": 1, "kind": "theboss's own Python (baseline/_ref)",
            "sample": f"the first {n} samples of the workload's stream (same seed and matrix), {dt:.1f} s",
            "samples_equal_to_gpu": bool(np.array_equal(np.array(out, dtype=np.int64),
                                                         np.asarray(gpu_samples[:n], dtype=np.int64)))}


def c2_patterns(n, count, seed):
    """Output patterns with about 20% of the occupied modes doubly occupied."""
    rng = np.random.default_rng(seed)
    m = 2 * n
    out = []
    for _ in range(count):
        distinct = int(round(n / 1.2))
        doubles = n - distinct
        modes = rng.choice(m, size=distinct, replace=False)
        T = np.zeros(m, dtype=np.int32)
        T[modes] = 1
        T[modes[:doubles]] = 2
        out.append(T)
    return np.array(out, dtype=np.int32)


def single_permanents(peak_tflops, seed, peak32=None):
    """C2: 64 Glynn permanents per size, device-timed, FP64 (the default); the
    relative error of the first pattern against the double-double oracle for
    n <= 24 (its CPU cost grows as 2^n: 7 s at n = 24 on 16 Arm cores, 170 s at
    n = 28), and for n = 26, 28, 30 against the double-double values computed once
    (tests/golden/c2_dd_large.json).  The opt-in float-pair kernel is timed on the
    same batches beside it, with its errors."""
    from oracle import oracle as O
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    res = {}
    large_dd = {}
    fixture = os.path.join(ROOT, "tests", "golden", "c2_dd_large.json")
    if os.path.exists(fixture):
        for rec in json.load(open(fixture)):
            large_dd.setdefault((rec["seed"], rec["n"]), []).append(rec)

    def errors(n, U, S, T, vals):
        out = {}
        if n <= 24:
            hi, lo = O.perm_dd(U, S[0], T[0])
            ref = hi + lo
            out["rel_err_vs_dd_pattern0"] = float(abs(vals[0] - ref) / abs(ref))
        else:  # double-double values computed once (tests/golden/make_c2_dd.py)
            for rec in large_dd.get((seed + n, n), []):
                if abs(U[0, 0] - complex(*rec["U00"])) <= 1e-12 and list(T[rec["pattern"]]) == rec["T"]:
                    ref = complex(rec["dd"][0], rec["dd"][1]) + complex(rec["dd"][2], rec["dd"][3])
                    out[f"rel_err_vs_dd_pattern{rec['pattern']}"] = float(abs(vals[rec["pattern"]] - ref) / abs(ref))
        return out

    for n in (16, 20, 24, 28, 30):
        U = haar_unitary(2 * n, seed + n)
        T = c2_patterns(n, 64, seed + n)
        S = np.zeros_like(T)
        S[:, :n] = 1
        b = _native.perm_bench(U, S, T, _native.GLYNN, warmup=1, steps=2 if n >= 28 else 5)
        ms = float(np.mean(b["sweep_ms"]))
        tf = b["flops"] / (ms / 1e3) / 1e12
        res[str(n)] = {"perms_per_s": 64 / (ms / 1e3), "ms_per_64": ms, "codes": b["codes"], "arithmetic": "fp64",
                       "arithmetic_note": "the first n - 8 factors of every product in block floating point on "
                                          "the integer pipe; frac_of_fp64_peak counts FP64-equivalent flops",
                       "achieved_tflops": tf, "frac_of_fp64_peak": tf / peak_tflops, **errors(n, U, S, T, b["results"])}
        prev = _native.perm_arithmetic(_native.FLOAT_PAIRS)
        try:
            f = _native.perm_bench(U, S, T, _native.GLYNN, warmup=1, steps=2 if n >= 28 else 5)
        finally:
            _native.perm_arithmetic(prev)
        fms = float(np.mean(f["sweep_ms"]))
        fp = {"perms_per_s": 64 / (fms / 1e3), "ms_per_64": fms, **errors(n, U, S, T, f["results"])}
        if f["ff_inst"] > 0 and peak32:  # float-pair sweep: its FP32 roofline
            t32 = f["ff_inst"] / (fms / 1e3) / 1e12
            fp.update({"achieved_t_fp32_inst": t32, "frac_of_fp32_peak": t32 / peak32})
        res[str(n)]["float_pairs"] = fp
    return res


def adjoint_section(seed):
    """C4: log-likelihood of 256 seeded output patterns (n=12, m=24, doubles
    allowed) under a 24-mode Clements mesh of 276 (theta, phi) phases;
    forward = mesh + permanents + log-likelihood, backward = torch autograd
    through the adjoint kernel and the mesh.  Plus 64 n=24 gradients in m=48."""
    import torch

    from theboss_gb300 import _native
    from theboss_gb300.adjoint import clements_unitary, log_likelihood
    from theboss_gb300.utilities import haar_unitary

    def patterns(m, n, count, s, maxm=2):
        rng = np.random.default_rng(s)
        out = np.zeros((count, m), dtype=np.int32)
        for k in range(count):
            c = 0
            while c < n:
                i = int(rng.integers(0, m))
                if out[k, i] < maxm:
                    out[k, i] += 1
                    c += 1
        return out

    m, n = 24, 12
    g = torch.Generator().manual_seed(seed)
    theta = (torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    phi = (torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    S = np.zeros((256, m), dtype=np.int32)
    S[:, :n] = 1
    T = patterns(m, n, 256, seed)
    fw, bw = [], []
    for it in range(6):
        theta.grad = None
        phi.grad = None
        t0 = time.perf_counter()
        L = log_likelihood(clements_unitary(theta, phi), S, T)
        t1 = time.perf_counter()
        L.backward()
        t2 = time.perf_counter()
        if it >= 2:
            fw.append(t1 - t0)
            bw.append(t2 - t1)
    c4 = {"forward_ms": 1e3 * float(np.median(fw)), "backward_ms": 1e3 * float(np.median(bw)),
          "backward_over_forward": float(np.median(bw) / np.median(fw)), "patterns": 256, "n": n, "m": m,
          "phases": 276, "log_likelihood": float(L.item())}
    # kernel-level: permanents vs permanents + all n^2 derivatives, n = 24
    m2, n2 = 48, 24
    U = haar_unitary(m2, seed + 1)
    S2 = np.zeros((64, m2), dtype=np.int32)
    S2[:, :n2] = 1
    T2 = patterns(m2, n2, 64, seed + 2)
    _native.perm_batch(U, S2, T2, _native.GLYNN)  # warm-up of both (buffers, kernel attributes)
    _native.perm_grad_batch(U, S2, T2)
    fw2, gr2 = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        _native.perm_batch(U, S2, T2, _native.GLYNN)
        t1 = time.perf_counter()
        _native.perm_grad_batch(U, S2, T2)
        t2 = time.perf_counter()
        fw2.append(t1 - t0)
        gr2.append(t2 - t1)
    c5 = {"forward_ms": 1e3 * min(fw2), "gradient_ms": 1e3 * min(gr2), "gradient_over_forward": min(gr2) / min(fw2),
          "patterns": 64, "n": n2, "m": m2, "timing": "minimum of 3 calls of each, after one warm-up call of each"}
    return {"clements_log_likelihood_n12_m24": c4, "gradients_n24_m48": c5}


def distribution_section(peak_tflops, seed):
    """Exact uniform-loss distribution (theboss's BSDistributionCalculatorWithUniformLosses):
    n=8 single photons in m=16 modes, eta=0.5, every one of the C(24, 8) = 735,471
    lossy outcomes; GPU permanents of every (lossy input, outcome) pair.  The CPU
    line is the oracle (C permanents, theboss's arithmetic in Python) on a bounded
    sample of the outcomes."""
    from math import comb

    from oracle import oracle as O
    from theboss_gb300 import _native
    from theboss_gb300.distribution_calculators import (BosonSamplingExperimentConfiguration,
                                                        BSDistributionCalculatorWithUniformLosses)
    from theboss_gb300.utilities import haar_unitary, possible_states_array

    n, m, eta = 8, 16, 0.5
    U = haar_unitary(m, seed + 16)
    inp = [1] * n + [0] * (m - n)
    cfg = BosonSamplingExperimentConfiguration(interferometer_matrix=U, initial_state=inp,
                                               initial_number_of_particles=n, number_of_modes=m,
                                               number_of_particles_lost=0, number_of_particles_left=n,
                                               uniform_transmissivity=eta)
    calc = BSDistributionCalculatorWithUniformLosses(cfg, None)
    calc.calculate_distribution()  # warm-up
    t = time.perf_counter()
    dist = np.array(calc.calculate_distribution())
    e2e_s = time.perf_counter() - t
    outs = possible_states_array(n, m, losses=True)
    _, kernel_ms = _native.lossy_probabilities(U, inp, outs, timed=True)
    ls = outs.sum(axis=1)
    # Glynn flops per pair: 2^(l-1) codes x (8 l - 4); pairs: C(n, l) lossy inputs x outcomes of l
    flops = float(sum(comb(n, l) * int((ls == l).sum()) * 2 ** (l - 1) * (8 * l - 4) for l in range(1, n + 1)))
    tf = flops / (kernel_ms / 1e3) / 1e12
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(outs), size=300, replace=False)
    w = O.binomial_weights(n, eta)
    t = time.perf_counter()
    ref = [w[0] if ls[i] == 0 else O.fixed_loss_probability(U, inp, outs[i]) * w[ls[i]] for i in pick]
    cpu_s = time.perf_counter() - t
    err = float(np.max(np.abs(dist[pick] - ref) / np.maximum(np.abs(ref), 1e-300)))
    return {"workload": "uniform losses eta=0.5, n=8, m=16, all 735,471 outcomes, Haar unitary",
            "outcomes_per_s_e2e": len(outs) / e2e_s, "e2e_ms": e2e_s * 1e3, "kernel_ms": kernel_ms,
            "sum": float(dist.sum()), "achieved_tflops": tf, "frac_of_fp64_peak": tf / peak_tflops,
            "max_rel_err_vs_oracle_sample": err,
            "cpu_oracle": {"outcomes_per_s": len(pick) / cpu_s, "cores": 1, "kind": "port",
                           "sample": f"{len(pick)} random outcomes of the same workload, {cpu_s:.1f} s"}}


def lossy_network_run(seed, samples):
    """C5: lossy-network C&C-B, n = 30 photons in m = 60 modes with per-mode
    transmissivities t ~ U[0.3, 0.9] (M = U diag(sqrt(t))), expanded to 120 modes
    (theboss's prepare_interferometer_matrix_in_expanded_space), through the
    drop-in strategy.  Every sample runs 30 levels of all-minors sweeps in the
    expanded space: sum_k 2^(k-1) (9k - 12) flops per sample."""
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator
    from theboss_gb300.simulation_strategies import LossyNetworksGeneralizedCliffordsSimulationStrategy
    from theboss_gb300.utilities import haar_unitary

    m, n = 60, 30
    V = haar_unitary(m, seed + 60)
    tr = np.random.default_rng(seed).uniform(0.3, 0.9, m)
    strat = LossyNetworksGeneralizedCliffordsSimulationStrategy(RyserPermanentCalculator(V @ np.diag(np.sqrt(tr))))
    np.random.seed(seed)
    strat.simulate([1] * n + [0] * (m - n), 4)  # warm-up
    np.random.seed(seed)
    t = time.perf_counter()
    smp = strat.simulate([1] * n + [0] * (m - n), samples)
    dt = time.perf_counter() - t
    flops = samples * sum(2.0 ** (k - 1) * (9 * k - 12) for k in range(2, n + 1))
    return {"workload": f"lossy network n={n} in m={m} (120 expanded), t~U[0.3,0.9], {samples} samples",
            "samples_per_s": samples / dt, "s": dt, "samples": samples,
            "mean_particles_detected": float(np.mean([sum(x) for x in smp])),
            "achieved_tflops_e2e": flops / dt / 1e12}


def strategies_section(seed):
    """The other samplers of the path, each timed through its drop-in class:
    C1 plain generalized C&C (n=8, m=16, 1000 samples), C5 lossy-network C&C-B
    (n=30 in m=60, 120 expanded modes, 64 of the configuration's 2000 samples;
    --case c5 runs all 2000), uniform-loss BOBS (n=20, m=40,
    eta=0.5, hierarchy level 10, 2000 samples) and the GPU outcome counter
    (10^6 samples over the 12,376 outcomes of n=6, m=12)."""
    from theboss_gb300 import _native
    from theboss_gb300.approximation_strategies import LossyStateApproximationSimulationStrategy
    from theboss_gb300.permanent_calculators import GlynnGrayPermanentCalculator, RyserPermanentCalculator
    from theboss_gb300.simulation_strategies import (GeneralizedCliffordsSimulationStrategy,
                                                     LossyNetworksGeneralizedCliffordsSimulationStrategy)
    from theboss_gb300.utilities import haar_unitary, possible_states_array

    out = {}
    U = haar_unitary(16, seed + 8)
    strat = GeneralizedCliffordsSimulationStrategy(GlynnGrayPermanentCalculator(U))
    np.random.seed(seed)
    strat.simulate([1] * 8 + [0] * 8, 50)  # warm-up
    np.random.seed(seed)
    t = time.perf_counter()
    strat.simulate([1] * 8 + [0] * 8, 1000)
    dt = time.perf_counter() - t
    out["c1_plain_gcc_n8_m16"] = {"samples_per_s": 1000 / dt, "s": dt, "samples": 1000}

    out["c5_lossy_network_n30_m60"] = lossy_network_run(seed, 64)

    U40 = haar_unitary(40, seed + 40)
    inp = [1] * 20 + [0] * 20
    strat = LossyStateApproximationSimulationStrategy(RyserPermanentCalculator(U40, input_state=inp), 0.5, 10,
                                                      threads_number=1)
    np.random.seed(seed)
    strat.simulate(inp, 100)
    np.random.seed(seed)
    t = time.perf_counter()
    strat.simulate(inp, 2000)
    dt = time.perf_counter() - t
    out["uniform_bobs_n20_m40_k10"] = {"samples_per_s": 2000 / dt, "s": dt, "samples": 2000}

    outs = possible_states_array(6, 12)
    idx = np.random.default_rng(seed).integers(0, len(outs), 10 ** 6)
    smp = np.ascontiguousarray(outs[idx])
    _native.count_outcomes(smp[:1000], outs, 12)
    t = time.perf_counter()
    cnt = _native.count_outcomes(smp, outs, 12)
    dt = time.perf_counter() - t
    assert int(cnt.sum()) == 10 ** 6
    out["outcome_counting_1e6_samples_12376_outcomes"] = {"samples_per_s": 1e6 / dt, "s": dt}
    return out


# arithmetic of the path (theboss computes in float64)
DTYPE = "f64"
DTYPE_NOTE = ("FP64 products, minors, Laplace step, |.|^2 and pmf; row sums in exact 64-bit fixed point; "
              "the first factors of every product multiplied in block floating point on the integer pipe "
              "(62-bit mantissas, each product within 2^-56.5 of its magnitude, one rounding to FP64); "
              "cdf decisions by an exact integer scan of the FP64 pmf, theboss's sequential FP64 rule "
              "inside the pmf's error window")


def roofline(b, sweep_s, achieved, peak, peak32, traffic):
    """The dominant kernel's roofline: the float-pair all-minors sweeps against the
    FP32 instruction peak (their FP64-equivalent rate beside it), or the FP64
    sweeps against the FP64 peak."""
    common = {"traffic": traffic, "sweep_ms_per_step": sweep_s * 1e3, "flops_per_step": b["sweep_flops"],
              "flops_note": "9k - 12 flops per Guan code at level k over the codes the Glynn-form all-minors "
                            "sweeps walk (half of theboss's Ryser-form codes for single photons); of these "
                            "the row-sum updates and the products of the first 8 factors (nf - 8 above 16 "
                            "factors; block floating point, 62-bit mantissas) run on the integer pipe, the "
                            "rest on the FP64 pipe, so "
                            "the FP64-equivalent rate can exceed the FP64 pipe's peak; ryser_form_* count "
                            "theboss's codes",
              "ryser_form_flops_per_step": b["ref_flops"],
              "ryser_form_equivalent_tflops": b["ref_flops"] / sweep_s / 1e12}
    if b["ff_inst"] > 0:
        ach32 = b["ff_inst"] / sweep_s / 1e12
        return {"bound": "fp32", "kernel": "minors_sweep_ff_kernel (all levels of a step)",
                "achieved": ach32, "peak": peak32, "unit": "T FP32 inst/s", "frac": ach32 / peak32,
                "peak_source": "boss_fp32_peak (independent FFMA chains), measured in this run",
                "inst_note": "float-pair arithmetic, 47.5625 nf FP32 instructions per Guan code at nf = k - 1 "
                             "factors (32 per complex product, 16 per complex sum, lazily renormalised, "
                             "resynchronised every 32 codes); integer, load and conversion instructions "
                             "not counted",
                "fp32_inst_per_step": b["ff_inst"],
                "fp64_equivalent": {"achieved_tflops": achieved, "fp64_peak_tflops": peak,
                                    "ratio_to_fp64_peak": achieved / peak}, **common}
    return {"bound": "fp64", "kernel": "minors_sweep_kernel (all levels of a step)", "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "boss_fp64_peak, measured in this run",
            "frac_note": "FP64-equivalent flops over the FP64 pipe's measured peak; the integer pipe carries "
                         "part of the products, so a fraction above 1 is reachable", **common}


def float_pair_section(U, inp, w, args, fp64_samples):
    """The opt-in float-pair arithmetic (boss_minors_arithmetic(0)): the same
    workload and seed, device-timed; its stream against the FP64 one."""
    from theboss_gb300 import _native

    prev = _native.minors_arithmetic(_native.FLOAT_PAIRS)
    try:
        np.random.seed(args.seed)
        _native.gccb_near_ties(reset=True)
        b = _native.gccb_bench(U, inp, w, args.samples, args.warmup, args.steps)
        ties = _native.gccb_near_ties(reset=True)
    finally:
        _native.minors_arithmetic(prev)
    ms = float(np.mean(b["step_ms"]))
    return {"value": args.samples / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms,
            "dtype": "i64 fixed point + f32x2 float pairs (~47-bit)",
            "sweep_ms_per_step": float(np.mean(b["sweep_ms"])),
            "samples_differing_from_fp64": int((b["samples"] != fp64_samples).any(axis=1).sum()),
            "near_ties_per_step": ties / (args.warmup + args.steps)}


def run_ours(args, rank, world):
    from theboss_gb300 import _native
    from theboss_gb300.simulation_strategies import GCCBPlainDriver
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator

    set_arithmetic(args)
    U, inp, w = workload(args.seed)
    peak, _ = _native.fp64_peak()
    peak32, _ = _native.fp32_peak()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    np.random.seed(args.seed + rank)
    # the autotuner picks each level's split and group size on this workload (numpy's state is not advanced)
    tune = _native.gccb_autotune(U, inp, w, args.samples, reps=3) if not args.no_tune else None
    np.random.seed(args.seed + rank)
    _native.gccb_near_ties(reset=True)
    _barrier(world)
    clocks.start()  # sampled over the device-timed steps and the e2e steps below
    t_wall = time.perf_counter()
    b = _native.gccb_bench(U, inp, w, args.samples, args.warmup, args.steps)
    t_wall = time.perf_counter() - t_wall
    _barrier(world)
    ties = _native.gccb_near_ties(reset=True)
    total_ms = float(np.sum(b["step_ms"]))
    total_ms = _max_over_ranks(total_ms, world)
    value = world * args.samples * args.steps / (total_ms / 1e3)
    sweep_s = float(np.mean(b["sweep_ms"])) / 1e3
    achieved = b["sweep_flops"] / sweep_s / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "sweep_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("dram_bytes_per_step")
        except Exception:
            traffic = None
    # e2e through the C ABI with host buffers; the samples must equal the device run's.
    # The same warm-up count as the device section, untimed, then `steps` timed calls.
    e2e_t = []
    for it in range(args.warmup + args.steps):
        np.random.seed(args.seed + rank)
        t = time.perf_counter()
        out = _native.gccb_sample(U, inp, w, args.samples)
        if it >= args.warmup:
            e2e_t.append(time.perf_counter() - t)
    clk = clocks.stop()
    if not np.array_equal(out, b["samples"]):
        raise SystemExit("e2e samples differ from the device-timed run")
    e2e = {"value": args.samples * args.steps / sum(e2e_t), "unit": "samples/s",
           "h2d_bytes_per_step": b["h2d_bytes"], "d2h_bytes_per_step": b["d2h_bytes"]}
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE if args.arith == "fp64" else "i64 fixed point + f32x2 float pairs (~47-bit)",
            "dtype_note": DTYPE_NOTE if args.arith == "fp64" else "float pairs (opt-in arithmetic)",
            "data": "synthetic (seeded Haar unitary)",
            "config": config(args), "clocks": clk, "e2e": e2e,
            "gpu_launches": b["kernels"] * args.steps,
            "roofline": roofline(b, sweep_s, achieved, peak, peak32, traffic),
            "near_ties_per_step": ties / (args.warmup + args.steps),
            "autotune": tune,
            "wall_s_device_section": t_wall}
    if rank == 0 and not args.quick:
        # theboss's per-step loop with the GPU all-minors calculator, bounded sample
        n_plain = 200
        np.random.seed(args.seed)
        t = time.perf_counter()
        GCCBPlainDriver(RyserPermanentCalculator(U), ETA).simulate(list(inp), n_plain)
        plain = n_plain / (time.perf_counter() - t)
        line["plain_gpu"] = {"value": plain, "unit": "samples/s", "samples": n_plain}
        line["batched_vs_plain"] = {"device": value / world / plain, "e2e": e2e["value"] / plain}
        if args.arith == "fp64":
            line["float_pairs"] = float_pair_section(U, inp, w, args, b["samples"])
        line["single_permanents"] = single_permanents(peak, args.seed, peak32)
        line["adjoint"] = adjoint_section(args.seed)
        line["exact_distribution"] = distribution_section(peak, args.seed)
        line["strategies"] = strategies_section(args.seed)
    if rank == 0:
        line["cpu_baseline"], parity = cpu_baseline(U, inp, w, args.seed, gpu_samples=b["samples"])
        line["parity"] = parity
        if not args.quick:
            line["theboss_python"] = theboss_python_line(U, inp, args.seed, b["samples"])
        print(json.dumps(line), flush=True)
        if parity["gpu_disagrees_with_double_double"]:
            raise SystemExit("the device-timed samples differ from the oracle's beyond its near ties")


def run_reference(args, rank):
    if rank != 0:
        return
    from oracle import oracle as O

    U, inp, w = workload(args.seed)
    cores = O.set_threads(os.cpu_count() or 1)  # all host threads, whatever OMP_NUM_THREADS torchrun set
    # calibrate a per-step sample of about 3 s
    np.random.seed(args.seed)
    L, A, Uu = O.predraw_gccb(list(inp), 200, w)
    t = time.perf_counter()
    O.gccb_run(U, L, A, Uu)
    per = (time.perf_counter() - t) / 200
    n = int(min(args.samples, max(200, 3.0 / max(per, 1e-9))))
    times = []
    for it in range(args.warmup + args.steps):
        np.random.seed(args.seed)
        L, A, Uu = O.predraw_gccb(list(inp), n, w)
        t = time.perf_counter()
        O.gccb_run(U, L, A, Uu)
        dt = time.perf_counter() - t
        if it >= args.warmup:
            times.append(dt)
    value = n * len(times) / sum(times)
    sample = (f"{n} of the {args.samples} samples per step (same seed and matrix), C restatement of theboss's "
              f"GCC-B sampler, OpenMP over samples")
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.samples / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Haar unitary)", "config": config(args),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        from theboss_gb300 import _native

        _native.select_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.case:
            run_case(args)
        else:
            run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
