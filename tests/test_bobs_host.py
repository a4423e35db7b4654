"""The BOBS strategies' random-number replays (no GPU) against numpy's own calls
in theboss's per-sample order (lossy_state_approximated_simulation_strategy.py:298-362,
nonuniform_losses_approximation_strategy.py:280-347, and the C&C-B steps of
generalized_cliffords_b_simulation_strategy.py:97-110)."""
import numpy as np
import pytest


def _gccb_steps(particles):
    ri, uu = [], []
    for left in range(particles, 0, -1):
        ri.append(np.random.randint(0, left))
        uu.append(np.random.random_sample())
    return ri, uu


@pytest.mark.parametrize("m,k,seed", [(6, 2, 1), (7, 3, 2), (5, 5, 3), (4, 0, 4)])
def test_uniform_bobs_replay_matches_numpy(m, k, seed):
    from theboss_gb300 import _native

    rng = np.random.default_rng(seed)
    exact = rng.integers(0, 3, (5, k))
    ew = rng.random(5)
    ew /= ew.sum()
    approx = np.zeros((4, m - k), dtype=int)
    if m > k:
        approx[:, 0] = np.arange(4)
    aw = np.array([0.1, 0.2, 0.3, 0.4])
    stride = int(exact.sum(axis=1).max() + approx.sum(axis=1).max())
    N = 50
    np.random.seed(seed)
    inputs, ph, perms, ri, uu = _native.bobs_uniform_predraw(N, m, k, exact, ew, approx, aw, stride)
    after = np.random.random()
    np.random.seed(seed)
    for s in range(N):
        ia = np.random.choice(range(len(aw)), p=aw)
        ie = np.random.choice(range(len(ew)), p=ew)
        inp = np.concatenate([exact[ie], approx[ia]])
        assert inputs[s].tolist() == inp.tolist()
        assert ph[s].tolist() == np.random.rand(m - k).tolist()
        perm = np.arange(m)
        np.random.shuffle(perm)
        assert perms[s].tolist() == perm.tolist()
        r, u = _gccb_steps(int(inp.sum()))
        assert ri[s, :len(r)].tolist() == r and uu[s, :len(u)].tolist() == u
    assert np.random.random() == after


@pytest.mark.parametrize("base,ka,na,lossy", [([0, 0, 1, 1, 0, 2], 2, 3, True), ([0, 0, 0, 1, 1], 3, 2, False),
                                              ([1, 0, 2], 0, 0, True)])
def test_nonuniform_bobs_replay_matches_numpy(base, ka, na, lossy):
    from scipy.special import binom

    from theboss_gb300 import _native

    top = max(max(base), na)
    eta = 0.7
    table = np.zeros((top + 1, top + 1))
    for n in range(1, top + 1):
        table[n, :n + 1] = [pow(eta, l) * binom(n, l) * pow(1 - eta, n - l) for l in range(n + 1)]
    stride = sum(base) + na
    N = 40
    np.random.seed(9)
    inputs, ph, ri, uu = _native.bobs_nonuniform_predraw(N, base, ka, na, table, lossy, stride)
    after = np.random.random()
    np.random.seed(9)
    for s in range(N):
        state = list(base)
        if ka > 0:
            state[np.random.randint(0, ka)] = na
        lossy_input = []
        for occ in state:
            if occ == 0 or not lossy:
                lossy_input.append(occ)
                continue
            acc, r = 0.0, np.random.random()
            for i in range(occ + 1):  # the strategy module's own choice()
                acc += table[occ][i]
                if acc > r:
                    lossy_input.append(i)
                    break
        assert inputs[s].tolist() == lossy_input
        assert ph[s].tolist() == np.random.rand(ka).tolist()
        r, u = _gccb_steps(sum(lossy_input))
        assert ri[s, :len(r)].tolist() == r and uu[s, :len(u)].tolist() == u
    assert np.random.random() == after
