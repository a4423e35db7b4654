"""Host-side parts of the batched sampler (no GPU): the MT19937 replay inside
libboss_gb300.so must draw exactly what numpy's global RandomState draws for
theboss's C&C-B samplers, and leave the generator in the same state."""
import numpy as np
import pytest


@pytest.mark.parametrize("inp,eta,N", [([1] * 6 + [0] * 4, 0.5, 200), ([2, 1, 1, 0, 0], 0.8, 100),
                                       ([1] * 20 + [0] * 20, None, 50), ([1] * 20 + [0] * 20, 0.5, 500),
                                       ([0, 0, 0], 0.3, 20), ([1], None, 30)])
def test_predraw_matches_numpy_replay(oracle, inp, eta, N):
    from theboss_gb300 import _native

    n = sum(inp)
    w = None if eta is None else oracle.binomial_weights(n, eta)
    np.random.seed(1234)
    L_ref, A_ref, U_ref = oracle.predraw_gccb(inp, N, w)
    after_ref = np.random.random()
    np.random.seed(1234)
    kept, popped, uni = _native.gccb_predraw(inp, w, N)
    after = np.random.random()
    assert after == after_ref
    assert kept.tolist() == L_ref.tolist()
    for s in range(N):
        l = kept[s]
        assert popped[s, :l].tolist() == A_ref[s, :l].tolist()
        assert uni[s, :l].tolist() == U_ref[s, :l].tolist()


def test_predraw_state_positions_across_twist(oracle):
    """Long streams cross many MT19937 regenerations (every 624 words)."""
    from theboss_gb300 import _native

    np.random.seed(7)
    for _ in range(3):
        np.random.random()
    st = np.random.get_state()
    inp = [1] * 12 + [0] * 12
    L_ref, A_ref, U_ref = oracle.predraw_gccb(inp, 400, None)
    ref_next = np.random.random()
    np.random.set_state(st)
    kept, popped, uni = _native.gccb_predraw(inp, None, 400)
    assert np.random.random() == ref_next
    assert (popped == A_ref).all() and (uni == U_ref).all()


def test_expanded_space_matrix_matches_reference():
    from conftest import as_matrix, load_golden
    from theboss_gb300.utilities import prepare_interferometer_matrix_in_expanded_space

    for rec in load_golden("gcc_samples.json"):
        if rec["kind"] != "lossy_net":
            continue
        M = as_matrix(rec["U"])
        got = prepare_interferometer_matrix_in_expanded_space(M)
        m = M.shape[0]
        if np.allclose(got, as_matrix(rec["expanded"]), rtol=0, atol=1e-13):
            continue  # same LAPACK build as the machine that made the fixture
        # Otherwise the SVD's phases may differ; check the phase-independent parts of
        # [[V S W, V L], [L W, S]] (L = sqrt(1 - S^2)).
        s = np.linalg.svd(M, compute_uv=False)
        loss = np.sqrt(np.clip(1 - s ** 2, 0, None))
        assert np.allclose(got[:m, :m], M, atol=1e-12)
        assert np.allclose(got[m:, m:], np.diag(s), atol=1e-12)
        assert np.allclose(np.linalg.norm(got[m:, :m], axis=1), loss, atol=1e-12)


@pytest.mark.parametrize("inp,eta,N,skip", [([1] * 20 + [0] * 20, 0.5, 10000, 0), ([1] * 20 + [0] * 20, 0.5, 4097, 313),
                                            ([1] * 12 + [0] * 12, None, 3000, 623), ([1] * 5 + [0] * 5, 0.9, 20000, 1),
                                            ([2, 1, 1, 0, 0], 0.8, 2048, 17), ([1], 0.5, 5000, 600)])
def test_parallel_replay_equals_numpy(oracle, inp, eta, N, skip):
    """From 1024 samples on the replay runs on several host threads, each parsing
    a slice of the word stream from a guessed start, stitched where the slices'
    parses meet the true one.  The draws, the zero tails of the rows and numpy's
    final state must be the sequential replay's, from any starting position in
    the generator's 624-word block."""
    from theboss_gb300 import _native

    n = sum(inp)
    w = None if eta is None else oracle.binomial_weights(n, eta)
    np.random.seed(99)
    np.random.random(skip)
    st = np.random.get_state()
    L_ref, A_ref, U_ref = oracle.predraw_gccb(inp, N, w)
    st_ref = np.random.get_state()
    np.random.set_state(st)
    kept, popped, uni = _native.gccb_predraw(inp, w, N)
    st_got = np.random.get_state()
    assert st_got[2] == st_ref[2] and np.array_equal(st_got[1], st_ref[1])
    assert np.array_equal(kept, L_ref)
    width = uni.shape[1]
    A = np.zeros((N, width), dtype=A_ref.dtype)
    Uu = np.zeros((N, width))
    A[:, :A_ref.shape[1]] = A_ref[:, :width]
    Uu[:, :U_ref.shape[1]] = U_ref[:, :width]
    mask = np.arange(width)[None, :] < kept[:, None]
    assert np.array_equal(np.where(mask, popped, 0), np.where(mask, A, 0))
    assert np.array_equal(uni, np.where(mask, Uu, 0.0))  # rows past the kept particles stay zero


def test_parallel_replay_across_growing_shapes(oracle):
    """The replay keeps its per-thread storage between calls; calls whose particle
    count grows must not write past what an earlier, smaller call sized."""
    from theboss_gb300 import _native

    for n, eta, N in [(1, 0.5, 9000), (5, 0.5, 20000), (12, None, 3000), (20, 0.5, 10000), (30, 0.7, 5000)]:
        inp = [1] * n + [0] * n
        w = None if eta is None else oracle.binomial_weights(n, eta)
        np.random.seed(n)
        L_ref, A_ref, U_ref = oracle.predraw_gccb(inp, N, w)
        after_ref = np.random.random()
        np.random.seed(n)
        kept, popped, uni = _native.gccb_predraw(inp, w, N)
        assert np.random.random() == after_ref
        assert np.array_equal(kept, L_ref)
        for s in range(0, N, 97):
            l = kept[s]
            assert popped[s, :l].tolist() == A_ref[s, :l].tolist()
            assert uni[s, :l].tolist() == U_ref[s, :l].tolist()


@pytest.mark.filterwarnings("ignore::DeprecationWarning")
def test_parallel_replay_in_a_forked_child(oracle):
    """A child forked after the replay's host threads started inherits none of
    them; its replay must still finish, with the parent's draws."""
    import os

    from theboss_gb300 import _native

    inp = [1] * 20 + [0] * 20
    w = oracle.binomial_weights(20, 0.5)
    np.random.seed(1)
    ref, _, _ = _native.gccb_predraw(inp, w, 5000)
    pid = os.fork()
    if pid == 0:  # the child: exit code 0 when its replay equals the parent's
        code = 1
        try:
            np.random.seed(1)
            got, _, _ = _native.gccb_predraw(inp, w, 5000)
            code = 0 if np.array_equal(got, ref) else 2
        finally:
            os._exit(code)
    _, status = os.waitpid(pid, 0)
    assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0
