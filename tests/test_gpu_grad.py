"""GPU parity of the adjoint: d perm(U[T,S]) / d U[j][i] = T_j S_i perm(U[T-e_j, S-e_i])
checked against minors from the oracle (theboss's all-minors algorithm), the
double-double oracle, and central finite differences through the Clements mesh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _patterns(m, n, count, seed, max_mult=2):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        v = np.zeros(m, dtype=np.int32)
        k = 0
        while k < n:
            i = int(rng.integers(0, m))
            if v[i] < max_mult:
                v[i] += 1
                k += 1
        out.append(v)
    return np.array(out, dtype=np.int32)


def _minor_grad(oracle, U, S, T):
    """T_j S_i perm(U[T - e_j, S - e_i]) from the oracle's all-minors (Ryser) sweeps."""
    m = len(S)
    g = np.zeros((m, m), dtype=complex)
    for j in range(m):
        if T[j] == 0:
            continue
        Tj = T.copy()
        Tj[j] -= 1
        if S.sum() == 1:
            sub = [complex(v) for v in S]
        else:
            sub = oracle.submatrices(U, list(S), list(Tj))
        for i in range(m):
            if S[i]:
                g[j, i] = T[j] * S[i] * sub[i]
    return g


@pytest.mark.parametrize("m,n,count,max_mult", [(12, 6, 6, 2), (10, 5, 4, 3), (24, 12, 3, 2)])
def test_gradients_match_oracle_minors(oracle, m, n, count, max_mult):
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    U = haar_unitary(m, m + n)
    S = _patterns(m, n, count, 1, max_mult)
    T = _patterns(m, n, count, 2, max_mult)
    perms, grads = _native.perm_grad_batch(U, S, T)
    ref_perms = _native.perm_batch(U, S, T, _native.GLYNN)
    for k in range(count):
        assert abs(perms[k] - ref_perms[k]) <= 1e-12 * abs(ref_perms[k])
        ref = _minor_grad(oracle, U, S[k], T[k])
        scale = np.abs(ref).max()
        assert np.abs(grads[k] - ref).max() <= 1e-11 * scale, (k, np.abs(grads[k] - ref).max() / scale)


@pytest.mark.parametrize("n,rows", [(16, 4), (24, 1)])
def test_gradients_against_double_double(oracle, n, rows):
    """Rows of d perm / dU against double-double all-minors (at n = 24 one row:
    the oracle's cost grows as 2^n: about a minute there on 16 Arm cores)."""
    from theboss_gb300 import _native
    from theboss_gb300.utilities import haar_unitary

    m = 2 * n
    U = haar_unitary(m, 5)
    S = np.zeros((1, m), dtype=np.int32)
    S[0, :n] = 1
    T = _patterns(m, n, 1, 9)
    _, grads = _native.perm_grad_batch(U, S, T)
    for j in np.nonzero(T[0])[0][:rows]:
        Tj = T[0].copy()
        Tj[j] -= 1
        ref = np.array(oracle.submatrices_dd(U, list(S[0]), list(Tj))) * T[0][j] * S[0]
        scale = np.abs(ref).max()
        assert np.abs(grads[0][j] - ref).max() <= 1e-10 * scale


def test_autograd_log_likelihood_matches_finite_differences():
    torch = pytest.importorskip("torch")
    from theboss_gb300.adjoint import clements_unitary, log_likelihood

    m, n = 8, 4
    g = torch.Generator().manual_seed(4)
    theta = (torch.rand(m * (m - 1) // 2, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    phi = (torch.rand(m * (m - 1) // 2, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    S = np.zeros((16, m), dtype=np.int32)
    S[:, :n] = 1
    T = _patterns(m, n, 16, 3)

    def loss(th, ph):
        return log_likelihood(clements_unitary(th, ph), S, T)

    L = loss(theta, phi)
    L.backward()
    h = 1e-6
    for which, param, grad in (("theta", theta, theta.grad), ("phi", phi, phi.grad)):
        for idx in (0, 5, 17, 27):
            with torch.no_grad():
                p = param.detach().clone()
                p[idx] += h
                lp = loss(p, phi.detach()) if which == "theta" else loss(theta.detach(), p)
                p[idx] -= 2 * h
                lm = loss(p, phi.detach()) if which == "theta" else loss(theta.detach(), p)
            fd = (lp - lm).item() / (2 * h)
            assert abs(fd - grad[idx].item()) <= 1e-6 * max(1.0, abs(fd)), (which, idx, fd, grad[idx].item())


def test_permanents_function_gradient_is_conjugate_derivative():
    torch = pytest.importorskip("torch")
    from theboss_gb300.adjoint import permanents
    from theboss_gb300.utilities import haar_unitary

    U0 = haar_unitary(6, 8)
    U = torch.tensor(U0, requires_grad=True)
    S = np.array([[1, 1, 1, 0, 0, 0]])
    T = np.array([[0, 1, 0, 2, 0, 0]])
    p = permanents(U, S, T)
    # L = Re(perm): dL/dU* convention gives grad = conj(d perm / dU) / 1 for the real part
    p.real.sum().backward()
    from theboss_gb300 import _native

    _, grads = _native.perm_grad_batch(U0, S.astype(np.int32), T.astype(np.int32))
    assert np.allclose(U.grad.numpy(), np.conj(grads[0]), atol=1e-13)


def test_clements_log_likelihood_gradient_at_benchmark_size(oracle):
    """The adjoint benchmark's own configuration: 256 seeded output patterns of
    n = 12 photons (doubles allowed) in m = 24 modes, a Clements mesh of 276
    (theta, phi) phases drawn uniformly.  The autograd gradient of the
    log-likelihood equals central finite differences (h = 1e-6) for a sample of
    the phases, within the differences' own rounding noise: each FP64 permanent
    perm_k is off its exact value by a relative e_k (measured here against the
    double-double oracle), so each log-probability by 2 e_k, and the difference
    quotient by up to sum_k 2 (2 e_k) / (2h); the bound takes twice that.  (The
    workload holds probabilities down to ~1e-27, permanents of ~1e-13 built from
    terms of order 2^-11, whose e_k approach 1e-10: theboss's float64 carries
    the same noise.)  d perm / dU of some patterns equals the oracle's minors of
    the mesh's unitary (theboss's all-minors algorithm)."""
    torch = pytest.importorskip("torch")
    from theboss_gb300 import _native
    from theboss_gb300.adjoint import clements_unitary, log_likelihood

    m, n, count = 24, 12, 256
    g = torch.Generator().manual_seed(2026)
    theta = (torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    phi = (torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi).requires_grad_(True)
    S = np.zeros((count, m), dtype=np.int32)
    S[:, :n] = 1
    T = _patterns(m, n, count, 2026)
    U = np.ascontiguousarray(clements_unitary(theta.detach(), phi.detach()).numpy())
    perms = _native.perm_batch(U, S, T, _native.GLYNN)
    e = 0.0
    for k in range(count):
        hi, lo = oracle.perm_dd(U, list(S[k]), list(T[k]))
        e += abs(perms[k] - (hi + lo)) / abs(hi + lo)
    h = 1e-6
    noise = 2 * (4 * e) / (2 * h)

    def loss(th, ph):
        return log_likelihood(clements_unitary(th, ph), S, T)

    loss(theta, phi).backward()
    picks = np.random.default_rng(7).choice(276, size=8, replace=False)
    for which, param, grad in (("theta", theta, theta.grad), ("phi", phi, phi.grad)):
        for idx in picks:
            with torch.no_grad():
                p = param.detach().clone()
                p[idx] += h
                lp = loss(p, phi.detach()) if which == "theta" else loss(theta.detach(), p)
                p[idx] -= 2 * h
                lm = loss(p, phi.detach()) if which == "theta" else loss(theta.detach(), p)
            fd = (lp - lm).item() / (2 * h)
            assert abs(fd - grad[idx].item()) <= 1e-6 * max(1.0, abs(fd)) + noise, \
                (which, idx, fd, grad[idx].item(), noise)
    _, grads = _native.perm_grad_batch(U, S[:4], T[:4])
    for k in range(4):
        ref = _minor_grad(oracle, U, S[k], T[k])
        scale = np.abs(ref).max()
        assert np.abs(grads[k] - ref).max() <= 1e-11 * scale
