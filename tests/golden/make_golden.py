"""Generates the golden fixtures in tests/golden/ by running theboss itself.

Run where the reference package is importable, giving the path of a theboss
checkout (the directory that holds the ``theboss`` package):

    python tests/golden/make_golden.py <theboss checkout> [--only <section>]

theboss's Glynn-Gray calculator imports ``guancodes`` (an un-vendored third-party
dependency pinned ``~=0.0.3`` in the reference's requirements.txt).  It is not
installable offline, so this script installs a test-only stand-in module that
yields the binary-reflected Gray code flip sequence (step t flips bit ctz(t)).
Only Glynn's summation order depends on it; its value does not.

Every fixture stores its input matrices, so nothing downstream needs scipy's
random generators or the reference package.
"""
import json
import os
import sys
import types

import numpy as np


def _install_gray_shim():
    mod = types.ModuleType("guancodes")
    sub = types.ModuleType("guancodes.GrayCode")

    def get_gray_code_update_indices(n):
        return [((t & -t).bit_length() - 1) for t in range(1, 1 << n)]

    sub.get_gray_code_update_indices = get_gray_code_update_indices
    mod.GrayCode = sub
    sys.modules["guancodes"] = mod
    sys.modules["guancodes.GrayCode"] = sub


def _c(z):
    z = complex(z)
    return [z.real, z.imag]


def _m(U):
    U = np.asarray(U, dtype=np.complex128)
    return {"re": U.real.tolist(), "im": U.imag.tolist()}


def main(ref_root):
    sys.path.insert(0, ref_root)
    sys.dont_write_bytecode = True
    _install_gray_shim()
    from scipy.stats import unitary_group

    from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
        RyserPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.chin_huh_permanent_calculator import (
        ChinHuhPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.glynn_gray_permanent_calculator import (
        GlynnGrayPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.classic_permanent_calculator import (
        ClassicPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.bs_cc_ryser_submatrices_permanent_calculator import (
        BSCCRyserSubmatricesPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.bs_cc_ch_submatrices_permanent_calculator import (
        BSCCCHSubmatricesPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.permanent_calculators.bs_permanent_calculator_base import (
        BSGuanCodeBasedPermanentCalculatorBase,
    )
    from theboss.simulation_strategies.generalized_cliffords_b_simulation_strategy import (
        GeneralizedCliffordsBSimulationStrategy,
    )
    from theboss.simulation_strategies.generalized_cliffords_b_uniform_losses_simulation_strategy import (
        GeneralizedCliffordsBUniformLossesSimulationStrategy,
    )
    from theboss.simulation_strategies.lossy_networks_generalized_cliffords_simulation_strategy import (
        LossyNetworksGeneralizedCliffordsSimulationStrategy,
    )
    from theboss.simulation_strategies.generalized_cliffords_simulation_strategy import (
        GeneralizedCliffordsSimulationStrategy,
    )
    from theboss.distribution_calculators.bs_exact_distribution_with_uniform_losses import (
        BSDistributionCalculatorWithUniformLosses,
        BosonSamplingExperimentConfiguration,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))
    rng = np.random.default_rng(20261203)

    # ---- single permanents ------------------------------------------------
    patterns4 = [  # tests/test_bs_permanent_calculators.py:88-122
        ([1, 1, 1, 1], [1, 1, 1, 1]),
        ([1, 1, 1, 0], [1, 0, 1, 1]),
        ([2, 1, 0, 0], [0, 1, 1, 1]),
        ([1, 1, 1, 0], [2, 1, 0, 0]),
        ([2, 1, 1, 0], [1, 1, 0, 2]),
        ([0, 0, 4, 0], [1, 1, 0, 2]),
        ([1, 1, 0, 2], [0, 1, 3, 0]),
        ([0, 2, 0, 2], [0, 0, 4, 0]),
        ([0, 0, 0, 0], [0, 0, 0, 0]),
    ]

    def rand_pattern(m, n, max_mult=3):
        s = np.zeros(m, dtype=int)
        for _ in range(n):
            while True:
                i = rng.integers(0, m)
                if s[i] < max_mult:
                    s[i] += 1
                    break
        return s.tolist()

    cases = []
    for seed in (11, 12):
        U = unitary_group.rvs(4, random_state=seed)
        for S, T in patterns4:
            cases.append((U, S, T, seed))
    for seed, m, n in [(21, 6, 3), (22, 6, 5), (23, 8, 4), (24, 8, 6), (25, 8, 7), (26, 10, 6), (27, 12, 8)]:
        U = unitary_group.rvs(m, random_state=seed)
        for _ in range(3):
            cases.append((U, rand_pattern(m, n), rand_pattern(m, n), seed))
    # larger single-photon-input cases (the C2 shape at small n)
    for seed, n in [(31, 9), (32, 10), (33, 11)]:
        m = 2 * n
        U = unitary_group.rvs(m, random_state=seed)
        S = [1] * n + [0] * n
        T = rand_pattern(m, n, max_mult=2)
        cases.append((U, S, T, seed))

    perms = []
    for U, S, T, seed in cases:
        n = sum(S)
        rec = {"seed": seed, "U": _m(U), "S": S, "T": T}
        rec["ryser"] = _c(RyserPermanentCalculator(U, S, T).compute_permanent())
        rec["chin_huh"] = _c(ChinHuhPermanentCalculator(U, S, T).compute_permanent())
        if sum(S) == sum(T):
            rec["glynn"] = _c(GlynnGrayPermanentCalculator(U, S, T).compute_permanent())
            if n <= 8:
                rec["classic"] = _c(ClassicPermanentCalculator(U, S, T).compute_permanent())
        perms.append(rec)
    with open(os.path.join(out_dir, "perms.json"), "w") as f:
        json.dump(perms, f)

    # ---- Guan code sequences ----------------------------------------------
    guan = []
    for S in ([1, 1, 1], [2, 1, 0, 3], [0, 2, 1], [1, 0, 2, 1, 1], [3]):
        calc = RyserPermanentCalculator(np.eye(len(S), dtype=complex), S, S)
        BSGuanCodeBasedPermanentCalculatorBase._initialize_guan_codes_variables(calc)
        seq_idx, seq_r = [-1], [list(calc._r_vector)]
        while True:
            calc._update_guan_code()
            if calc._index_to_update == len(calc._r_vector):
                break
            seq_idx.append(int(calc._index_to_update))
            seq_r.append([int(x) for x in calc._r_vector])
        guan.append({"S": S, "idx": seq_idx, "r": seq_r})
    with open(os.path.join(out_dir, "guan.json"), "w") as f:
        json.dump(guan, f)

    # ---- submatrices (all-minors) ------------------------------------------
    sub_cases = []
    U4 = unitary_group.rvs(4, random_state=41)
    # tests/test_bs_submatrices_permanent_calculators.py:41-73
    sub_cases.append((U4, [1, 1, 1, 1], [0, 1, 1, 1]))
    sub_cases.append((U4, [1.0, 3.0, 0.0, 0.0], [0, 1, 1, 1]))
    sub_cases.append((U4, [1.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0]))
    for seed, m, k in [(42, 6, 3), (43, 8, 5), (44, 8, 6), (45, 12, 8), (46, 16, 10)]:
        U = unitary_group.rvs(m, random_state=seed)
        for mm in (1, 2):
            S = rand_pattern(m, k, max_mult=mm)
            T = rand_pattern(m, k - 1, max_mult=2)
            sub_cases.append((U, S, T))
    subs = []
    for U, S, T in sub_cases:
        rec = {"U": _m(U), "S": [float(x) for x in S], "T": [float(x) for x in T]}
        rec["ryser"] = [_c(v) for v in BSCCRyserSubmatricesPermanentCalculator(U, np.array(S), np.array(T)).compute_permanents()]
        rec["chin_huh"] = [_c(v) for v in BSCCCHSubmatricesPermanentCalculator(U, np.array(S), np.array(T)).compute_permanents()]
        subs.append(rec)
    with open(os.path.join(out_dir, "submatrices.json"), "w") as f:
        json.dump(subs, f)

    # ---- seeded GCC-B sample streams -----------------------------------------
    gcc = []
    for seed, m, n, eta, N in [(51, 8, 4, 0.5, 40), (52, 10, 6, 0.7, 30), (53, 12, 6, None, 20), (54, 6, 3, 0.5, 60)]:
        U = unitary_group.rvs(m, random_state=seed)
        inp = [1] * n + [0] * (m - n)
        np.random.seed(seed)
        if eta is None:
            strat = GeneralizedCliffordsBSimulationStrategy(RyserPermanentCalculator(U))
        else:
            strat = GeneralizedCliffordsBUniformLossesSimulationStrategy(RyserPermanentCalculator(U), eta)
        samples = strat.simulate(inp, N)
        after = float(np.random.random())
        gcc.append({"kind": "gccb" if eta is None else "gccb_uniform", "seed": seed, "U": _m(U), "input": inp,
                    "eta": eta, "N": N, "samples": [[int(x) for x in s] for s in samples], "next_random": after})
    # binned input (multi-photon modes)
    U = unitary_group.rvs(5, random_state=55)
    np.random.seed(55)
    strat = GeneralizedCliffordsBUniformLossesSimulationStrategy(RyserPermanentCalculator(U), 0.8)
    samples = strat.simulate([2, 1, 1, 0, 0], 40)
    gcc.append({"kind": "gccb_uniform", "seed": 55, "U": _m(U), "input": [2, 1, 1, 0, 0], "eta": 0.8, "N": 40,
                "samples": [[int(x) for x in s] for s in samples], "next_random": float(np.random.random())})
    # non-uniform (network) losses: lossy matrix U diag(sqrt(t))
    for seed, m, n, N in [(56, 4, 2, 30), (57, 6, 3, 20)]:
        U = unitary_group.rvs(m, random_state=seed)
        t = np.random.default_rng(seed).uniform(0.3, 0.9, m)
        M = U @ np.diag(np.sqrt(t))
        calc = RyserPermanentCalculator(M.copy())
        strat = LossyNetworksGeneralizedCliffordsSimulationStrategy(calc)
        inp = [1] * n + [0] * (m - n)
        np.random.seed(seed)
        samples = strat.simulate(inp, N)
        gcc.append({"kind": "lossy_net", "seed": seed, "U": _m(M), "expanded": _m(calc.matrix), "input": inp,
                    "N": N, "samples": [[int(x) for x in s] for s in samples],
                    "next_random": float(np.random.random())})
    # plain (A-version) GCC
    for seed, m, n, N in [(58, 6, 3, 15)]:
        U = unitary_group.rvs(m, random_state=seed)
        inp = [1] * n + [0] * (m - n)
        np.random.seed(seed)
        strat = GeneralizedCliffordsSimulationStrategy(RyserPermanentCalculator(U))
        samples = strat.simulate(inp, N)
        gcc.append({"kind": "gcc", "seed": seed, "U": _m(U), "input": inp, "N": N,
                    "samples": [[int(x) for x in s] for s in samples],
                    "next_random": float(np.random.random())})
    with open(os.path.join(out_dir, "gcc_samples.json"), "w") as f:
        json.dump(gcc, f)

    # ---- exact uniform-loss distribution (the reference's known-answer test) ----
    P = np.array([[0, 0, 1, 0, 0], [1, 0, 0, 0, 0], [0, 0, 0, 1, 0], [0, 0, 0, 0, 1], [0, 1, 0, 0, 0]],
                 dtype=np.complex128)
    cfg = BosonSamplingExperimentConfiguration(
        interferometer_matrix=P, initial_state=[1, 1, 1, 0, 0], number_of_modes=5, initial_number_of_particles=3,
        number_of_particles_lost=2, number_of_particles_left=1, uniform_transmissivity=0.8)
    dist = BSDistributionCalculatorWithUniformLosses(cfg, ChinHuhPermanentCalculator(P)).calculate_distribution()
    U6 = unitary_group.rvs(4, random_state=61)
    cfg2 = BosonSamplingExperimentConfiguration(
        interferometer_matrix=U6, initial_state=[1, 1, 1, 0], number_of_modes=4, initial_number_of_particles=3,
        number_of_particles_lost=0, number_of_particles_left=3, uniform_transmissivity=0.6)
    dist2 = BSDistributionCalculatorWithUniformLosses(cfg2, ChinHuhPermanentCalculator(U6)).calculate_distribution()
    with open(os.path.join(out_dir, "distributions.json"), "w") as f:
        json.dump([{"U": _m(P), "input": [1, 1, 1, 0, 0], "eta": 0.8, "distribution": [float(x) for x in dist]},
                   {"U": _m(U6), "input": [1, 1, 1, 0], "eta": 0.6, "distribution": [float(x) for x in dist2]}], f)
    lossy_distributions(ref_root)
    mode_assignment_samples(ref_root)
    tvd_values(ref_root)
    bobs_samples(ref_root)
    gcc_uniform_losses_samples(ref_root)
    print("fixtures written to", out_dir)


def gcc_uniform_losses_samples(ref_root: str) -> None:
    """Seeded streams of theboss's A-version uniform-loss GCC
    (generalized_cliffords_uniform_losses_simulation_strategy.py:125-138): every
    photon survives when Python's random.random() < transmissivity, then numpy's
    random() picks its output.  Both generators are seeded; the value each one
    draws next is recorded, so the state theboss leaves behind is checked too."""
    import random

    sys.path.insert(0, ref_root)
    sys.dont_write_bytecode = True
    _install_gray_shim()
    from scipy.stats import unitary_group

    from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
        RyserPermanentCalculator,
    )
    from theboss.simulation_strategies.generalized_cliffords_uniform_losses_simulation_strategy import (
        GeneralizedCliffordsUniformLossesSimulationStrategy,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))
    recs = []
    for seed, py_seed, m, inp, eta, N in [(71, 171, 6, [1, 1, 1, 0, 0, 0], 0.6, 30),
                                          (72, 172, 8, [1, 1, 1, 1, 0, 0, 0, 0], 0.5, 25),
                                          (73, 173, 5, [2, 1, 0, 1, 0], 0.7, 25)]:
        U = unitary_group.rvs(m, random_state=seed)
        np.random.seed(seed)
        random.seed(py_seed)
        strat = GeneralizedCliffordsUniformLossesSimulationStrategy(RyserPermanentCalculator(U), eta)
        samples = strat.simulate(inp, N)
        recs.append({"kind": "gcc_uniform", "seed": seed, "py_seed": py_seed, "U": _m(U), "input": inp, "eta": eta,
                     "N": N, "samples": [[int(x) for x in s] for s in samples],
                     "dtypes": sorted({str(np.asarray(s).dtype) for s in samples}),
                     "next_random": float(np.random.random()), "next_py_random": random.random()})
    with open(os.path.join(out_dir, "gcc_uniform_losses_samples.json"), "w") as f:
        json.dump(recs, f)


def bobs_samples(ref_root: str) -> None:
    """Seeded streams of theboss's two BOBS strategies.  theboss's simulate() runs its
    per-sample loop (_simulate_in_parallel) in spawned worker processes whose
    generators cannot be seeded; the same loop is run here in this process after
    the same preparation simulate() does."""
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    from scipy.stats import unitary_group

    from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
        RyserPermanentCalculator,
    )
    from theboss.simulation_strategies.lossy_state_approximated_simulation_strategy import (
        LossyStateApproximationSimulationStrategy,
    )
    from theboss.simulation_strategies.nonuniform_losses_approximation_strategy import (
        NonuniformLossesApproximationStrategy,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))
    recs = []
    for seed, inp, eta, k, N in ((101, [1, 1, 1, 1, 0, 0], 0.6, 2, 40), (102, [1, 1, 1, 1, 1, 0, 0], 0.8, 3, 30),
                                 (103, [1, 1, 1, 0, 0], 0.5, 1, 30)):
        U = unitary_group.rvs(len(inp), random_state=seed)
        calc = RyserPermanentCalculator(U, input_state=inp)
        strat = LossyStateApproximationSimulationStrategy(calc, eta, k, threads_number=1)
        strat._prepare_not_approximated_lossy_mixed_state(inp[:k])
        strat._prepare_approximated_input_state(inp[k:])
        np.random.seed(seed)
        samples = strat._simulate_in_parallel(N)
        recs.append({"kind": "uniform_bobs", "seed": seed, "U": _m(U), "input": inp, "eta": eta, "k": k, "N": N,
                     "samples": [[int(x) for x in s] for s in samples], "next_random": float(np.random.random())})
    for seed, inp, ka, N in ((111, [1, 1, 1, 1, 0, 0], 2, 30), (112, [2, 1, 0, 1, 0], 3, 25)):
        m = len(inp)
        V = unitary_group.rvs(m, random_state=seed)
        t = np.random.default_rng(seed).uniform(0.4, 0.9, m)
        M = V @ np.diag(np.sqrt(t))
        calc = RyserPermanentCalculator(M, input_state=inp)
        strat = NonuniformLossesApproximationStrategy(calc, ka, threads_number=1)
        strat._state_without_approximated_modes = list(inp)
        for i in range(strat._approximated_modes_number):  # simulate()'s preparation
            strat._approximated_modes_particles_number += inp[i]
            strat._state_without_approximated_modes[i] = 0
        strat._binomial_weights = strat._compute_binomial_weights(
            max(max(inp), strat._approximated_modes_particles_number))
        np.random.seed(seed)
        samples = strat._simulate_in_parallel(N)
        recs.append({"kind": "nonuniform_bobs", "seed": seed, "U": _m(M), "input": inp, "k": ka, "N": N,
                     "samples": [[int(x) for x in s] for s in samples], "next_random": float(np.random.random())})
    with open(os.path.join(out_dir, "bobs_samples.json"), "w") as f:
        json.dump(recs, f)


def tvd_values(ref_root: str) -> None:
    """theboss's total-variation distances of seeded distributions (lists and dicts)."""
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    from theboss.quantum_computations_utilities import (
        count_total_variation_distance,
        count_total_variation_distance_dicts,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))
    rng = np.random.default_rng(91)
    recs = []
    for size in (1, 7, 1000, 3001):
        a, b = rng.random(size), rng.random(size)
        a, b = a / a.sum(), b / b.sum()
        recs.append({"kind": "list", "a": a.tolist(), "b": b.tolist(),
                     "tvd": float(count_total_variation_distance(list(a), list(b)))})
    for size in (5, 60, 400):
        d1, d2 = {}, {}
        for d in (d1, d2):
            for _ in range(size):
                d[tuple(int(v) for v in rng.integers(0, 4, 5))] = float(rng.random())
        recs.append({"kind": "dict", "d1": [[list(k), v] for k, v in d1.items()],
                     "d2": [[list(k), v] for k, v in d2.items()],
                     "tvd": float(count_total_variation_distance_dicts(d1, d2))})
    with open(os.path.join(out_dir, "tvd.json"), "w") as f:
        json.dump(recs, f)


def mode_assignment_samples(ref_root: str) -> None:
    """Seeded sample streams of theboss's mode-assignment generalized C&C."""
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    from scipy.stats import unitary_group

    from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
        RyserPermanentCalculator,
    )
    from theboss.simulation_strategies.mode_assignment_generalized_cliffords_simulation_strategy import (
        ModeAssignmentGeneralizedCliffordsSimulationStrategyInterface,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))
    recs = []
    for seed, inp, N in ((81, [1, 1, 1, 0, 0, 0], 30), (82, [2, 0, 1, 1, 0], 25)):
        U = unitary_group.rvs(len(inp), random_state=seed)
        np.random.seed(seed)
        strat = ModeAssignmentGeneralizedCliffordsSimulationStrategyInterface(RyserPermanentCalculator(U))
        samples = strat.simulate(inp, N)
        recs.append({"seed": seed, "U": _m(U), "input": inp, "N": N,
                     "samples": [[int(x) for x in s] for s in samples],
                     "r_sample": [int(x) for x in strat.r_sample],
                     "next_random": float(np.random.random())})
    with open(os.path.join(out_dir, "mode_assignment_samples.json"), "w") as f:
        json.dump(recs, f)


def lossy_distributions(ref_root: str) -> None:
    """Fixed- and uniform-loss exact distributions (standard and binned inputs, and
    one 11-particle case) computed by theboss's own calculators."""
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    from scipy.stats import unitary_group

    from theboss.boson_sampling_utilities.permanent_calculators.ryser_permanent_calculator import (
        RyserPermanentCalculator,
    )
    from theboss.boson_sampling_utilities.boson_sampling_utilities import generate_lossy_n_particle_input_states
    from theboss.distribution_calculators.bs_exact_distribution_with_uniform_losses import (
        BosonSamplingExperimentConfiguration,
        BSDistributionCalculatorWithFixedLosses,
        BSDistributionCalculatorWithUniformLosses,
    )

    out_dir = os.path.dirname(os.path.abspath(__file__))

    def cfg(U, inp, lost, eta=1.0):
        n = int(sum(inp))
        return BosonSamplingExperimentConfiguration(
            interferometer_matrix=U, initial_state=list(inp), initial_number_of_particles=n,
            number_of_modes=len(inp), number_of_particles_lost=lost, number_of_particles_left=n - lost,
            uniform_transmissivity=eta)

    cases = []
    U4 = unitary_group.rvs(4, random_state=71)
    for inp, lost in (([1, 1, 1, 0], 1), ([3, 1, 2, 0], 2)):
        c = BSDistributionCalculatorWithFixedLosses(cfg(U4, inp, lost), RyserPermanentCalculator(U4))
        cases.append({"kind": "fixed", "U": _m(U4), "input": inp, "lost": lost,
                      "outcomes": [[int(x) for x in o] for o in c.get_outcomes_in_proper_order()],
                      "probabilities": [float(x) for x in c.calculate_distribution()],
                      "lossy_inputs": [[int(x) for x in s]
                                       for s in generate_lossy_n_particle_input_states(inp, sum(inp) - lost)]})
    c = BSDistributionCalculatorWithUniformLosses(cfg(U4, [3, 1, 2, 0], 0, 0.5), RyserPermanentCalculator(U4))
    cases.append({"kind": "uniform", "U": _m(U4), "input": [3, 1, 2, 0], "lost": 0, "eta": 0.5,
                  "outcomes": [[int(x) for x in o] for o in c.get_outcomes_in_proper_order()],
                  "probabilities": [float(x) for x in c.calculate_distribution()]})
    U8 = unitary_group.rvs(8, random_state=72)
    c = BSDistributionCalculatorWithUniformLosses(cfg(U8, [1, 1, 1, 1, 1, 0, 0, 0], 0, 0.7), RyserPermanentCalculator(U8))
    outs = c.get_outcomes_in_proper_order()[::37]
    cases.append({"kind": "uniform", "U": _m(U8), "input": [1, 1, 1, 1, 1, 0, 0, 0], "lost": 0, "eta": 0.7,
                  "outcomes": [[int(x) for x in o] for o in outs],
                  "probabilities": [float(x) for x in c.calculate_probabilities_of_outcomes(outs)]})
    U12 = unitary_group.rvs(12, random_state=73)
    inp12 = [1] * 12
    c = BSDistributionCalculatorWithFixedLosses(cfg(U12, inp12, 1), RyserPermanentCalculator(U12))
    outs = [[1] * 11 + [0], [2, 0] + [1] * 9 + [0], [0, 3, 1, 1, 1, 1, 1, 1, 1, 0, 1, 0]]
    cases.append({"kind": "fixed", "U": _m(U12), "input": inp12, "lost": 1, "outcomes": outs,
                  "probabilities": [float(x) for x in c.calculate_probabilities_of_outcomes(outs)]})
    with open(os.path.join(out_dir, "lossy_distributions.json"), "w") as f:
        json.dump(cases, f)


if __name__ == "__main__":
    # python make_golden.py <theboss checkout> [--only lossy|mode_assignment|tvd|bobs|gcc_uniform]
    sections = {"lossy": lossy_distributions, "mode_assignment": mode_assignment_samples, "tvd": tvd_values,
                "bobs": bobs_samples, "gcc_uniform": gcc_uniform_losses_samples}
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <theboss checkout> [--only " + "|".join(sections) + "]")
    if len(sys.argv) > 3 and sys.argv[2] == "--only":
        sections[sys.argv[3]](sys.argv[1])
    else:
        main(sys.argv[1])
