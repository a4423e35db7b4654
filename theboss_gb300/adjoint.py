"""Differentiable permanents: output-pattern probabilities and log-likelihoods as
functions of the interferometer matrix or of its beam-splitter phases.

theboss has no derivatives.  d perm(U[T,S]) / d U[j][i] is T_j * S_i times the
(j, i) minor perm(U[T - e_j, S - e_i]); boss_perm_grad_batch returns all of them,
for every pattern, from one Glynn sweep per pattern (libboss_gb300.so).  Here
they back a torch.autograd.Function, and a Clements mesh (rectangular array of
m(m-1)/2 Mach-Zehnder interferometers, Clements et al., Optica 3, 1460 (2016))
maps phases to the unitary in torch so that gradients flow to the phases.
"""
from __future__ import annotations

import math
from typing import Sequence

import numpy as np
import torch

from . import _native


def _states(states, m: int) -> np.ndarray:
    a = np.asarray(states)
    if a.ndim == 1:
        a = a[None, :]
    if a.shape[1] != m:
        raise AttributeError("occupation vectors must have one entry per mode")
    return np.ascontiguousarray(np.rint(a).astype(np.int32))


class Permanents(torch.autograd.Function):
    """perms[k] = perm(U[T_k, S_k]); backward returns sum_k g_k * conj(d perm_k / dU),
    torch's convention for a holomorphic function of a complex tensor."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, input_states: np.ndarray, output_states: np.ndarray):
        Un = np.ascontiguousarray(U.detach().cpu().numpy().astype(np.complex128))
        perms = _native.perm_batch(Un, input_states, output_states, _native.GLYNN)
        ctx.save_for_backward(U)
        ctx.states = (input_states, output_states)
        return torch.from_numpy(perms).to(U.device)

    @staticmethod
    def backward(ctx, grad_perms: torch.Tensor):
        (U,) = ctx.saved_tensors
        S, T = ctx.states
        Un = np.ascontiguousarray(U.detach().cpu().numpy().astype(np.complex128))
        _, grads = _native.perm_grad_batch(Un, S, T)
        g = torch.from_numpy(grads).to(U.device)
        gU = torch.einsum("k,kji->ji", grad_perms.to(g.dtype), g.conj())
        return gU, None, None


def permanents(U: torch.Tensor, input_states, output_states) -> torch.Tensor:
    m = U.shape[0]
    return Permanents.apply(U, _states(input_states, m), _states(output_states, m))


def _norms(input_states: np.ndarray, output_states: np.ndarray) -> np.ndarray:
    f = np.vectorize(math.factorial)
    return np.prod(f(input_states), axis=1).astype(np.float64) * np.prod(f(output_states), axis=1).astype(np.float64)


def probabilities(U: torch.Tensor, input_states, output_states) -> torch.Tensor:
    """|perm(U[T,S])|^2 / (prod S! prod T!) for every pattern."""
    m = U.shape[0]
    S, T = _states(input_states, m), _states(output_states, m)
    p = Permanents.apply(U, S, T)
    return (p.real ** 2 + p.imag ** 2) / torch.from_numpy(_norms(S, T)).to(p.real.device)


def log_likelihood(U: torch.Tensor, input_states, output_states) -> torch.Tensor:
    return torch.log(probabilities(U, input_states, output_states)).sum()


def clements_layers(m: int):
    """Mode pairs (k, k+1) of each layer of the rectangular mesh: even layers start
    at mode 0, odd layers at mode 1; m layers give m(m-1)/2 interferometers."""
    out = []
    for layer in range(m):
        start = layer % 2
        out.append(np.arange(start, m - 1, 2))
    return out


def clements_unitary(theta: torch.Tensor, phi: torch.Tensor, output_phases: torch.Tensor = None) -> torch.Tensor:
    """U = D * T_L ... T_1 with T(theta, phi) on modes (k, k+1):
    [[e^{i phi} cos theta, -sin theta], [e^{i phi} sin theta, cos theta]]."""
    n_mzi = theta.shape[0]
    m = int(round((1 + math.sqrt(1 + 8 * n_mzi)) / 2))
    if m * (m - 1) // 2 != n_mzi or phi.shape[0] != n_mzi:
        raise ValueError("theta and phi need m(m-1)/2 entries each")
    ctype = torch.complex128
    M = torch.eye(m, dtype=ctype, device=theta.device)
    pos = 0
    for ks in clements_layers(m):
        k = torch.from_numpy(ks).to(theta.device)
        n = len(ks)
        th = theta[pos:pos + n]
        ep = torch.exp(1j * phi[pos:pos + n].to(ctype))
        pos += n
        c = torch.cos(th).to(ctype)
        s = torch.sin(th).to(ctype)
        top, bot = M[k], M[k + 1]
        new_top = (ep * c)[:, None] * top - s[:, None] * bot
        new_bot = (ep * s)[:, None] * top + c[:, None] * bot
        M = M.index_copy(0, k, new_top).index_copy(0, k + 1, new_bot)
    if output_phases is not None:
        M = torch.exp(1j * output_phases.to(ctype))[:, None] * M
    return M
