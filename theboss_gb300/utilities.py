"""Host-side helpers of the sampling path (numpy, no GPU work).

  mode_occupation_to_mode_assignment          boson_sampling_utilities.py:61-78
  mode_assignment_to_mode_occupation          boson_sampling_utilities.py:42-58
  generate_possible_states                    boson_sampling_utilities.py:81-155 (same
                                              order: per particle count, descending
                                              lexicographic)
  possible_states_array                       the same states as one int32 array
  generate_lossy_n_particle_input_states      boson_sampling_utilities.py:158-203 (same
                                              order: first occurrence over particle-index
                                              combinations)
  prepare_interferometer_matrix_in_expanded_space
                                              boson_sampling_utilities.py:264-342
  compute_qft_matrix                          quantum_computations_utilities.py:158-178
  generate_qft_matrix_for_first_m_modes       boson_sampling_utilities.py:505-521
  haar_unitary                                seeded Haar-random unitary (Mezzadri's
                                              QR of a complex Gaussian matrix with the
                                              phases of R's diagonal divided out)
"""
from __future__ import annotations

import itertools
from functools import lru_cache
from typing import List, Sequence, Tuple

import numpy as np


def mode_occupation_to_mode_assignment(mode_occupation: Sequence[int]) -> Tuple[int, ...]:
    out = []
    for i, v in enumerate(mode_occupation):
        out += [i] * int(v)
    return tuple(out)


def mode_assignment_to_mode_occupation(mode_assignment: Sequence[int], observed_modes_number: int = 0) -> Tuple[int, ...]:
    """Particle -> mode list to an occupation tuple of observed_modes_number entries
    (1 + the largest mode when 0)."""
    m = int(observed_modes_number) if observed_modes_number else max(mode_assignment) + 1
    occ = [0] * m
    for i in mode_assignment:
        occ[int(i)] += 1
    return tuple(occ)


@lru_cache(maxsize=None)
def _compositions(n: int, m: int) -> np.ndarray:
    """All m-mode n-particle occupations, descending lexicographic order."""
    if m == 1:
        return np.array([[n]], dtype=np.int32)
    parts = []
    for first in range(n, -1, -1):
        rest = _compositions(n - first, m - 1)
        block = np.empty((rest.shape[0], m), dtype=np.int32)
        block[:, 0] = first
        block[:, 1:] = rest
        parts.append(block)
    out = np.concatenate(parts)
    out.setflags(write=False)
    return out


@lru_cache(maxsize=8)
def possible_states_array(particles_number: int, modes_number: int, losses: bool = False) -> np.ndarray:
    """generate_possible_states as a read-only int32 array (rows in the same order)."""
    if particles_number < 0 or modes_number < 1:
        return np.zeros((0, max(modes_number, 0)), dtype=np.int32)
    first = 0 if losses else particles_number
    out = np.concatenate([_compositions(k, modes_number) for k in range(first, particles_number + 1)])
    out.setflags(write=False)
    return out


def generate_possible_states(particles_number: int, modes_number: int, losses: bool = False) -> List[Tuple[int, ...]]:
    """All m-mode states with n particles (or 0..n with losses), as tuples."""
    return [tuple(int(x) for x in row) for row in possible_states_array(particles_number, modes_number, losses)]


def generate_lossy_n_particle_input_states(initial_state: Sequence[int], number_of_particles_left: int) -> List[Tuple[int, ...]]:
    """Distinct sub-occupations of `initial_state` with the given particle count, in
    the order of their first appearance over combinations of particle indices."""
    m = len(initial_state)
    if sum(initial_state) == 0:
        return [tuple(initial_state)]
    x0 = mode_occupation_to_mode_assignment(initial_state)
    seen, out = set(), []
    for comb in itertools.combinations(range(len(x0)), number_of_particles_left):
        occ = [0] * m
        for c in comb:
            occ[x0[c]] += 1
        key = tuple(occ)
        if key not in seen:
            seen.add(key)
            out.append(key)
    return out


def compute_qft_matrix(n: int) -> np.ndarray:
    """n x n discrete Fourier matrix omega^(i j) / sqrt(n), omega = exp(2 pi i / n),
    with theboss's numpy expression (so the entries are the same doubles)."""
    if n == 0:
        return np.asarray([])
    omega = np.exp(2j * np.pi / n)
    horizontal = np.tile(range(n), n).reshape(n, n)
    return np.power(omega, horizontal * horizontal.transpose()) / np.sqrt(n)


def generate_qft_matrix_for_first_m_modes(m: int, all_modes_number: int) -> np.ndarray:
    """QFT on the first m modes, identity on the others."""
    qft = np.eye(all_modes_number, dtype=np.complex128)
    qft[0:m, 0:m] = compute_qft_matrix(m)
    return qft


def _loss_transfer_expansion(transmissivities: np.ndarray) -> np.ndarray:
    losses = 1.0 - transmissivities
    losses[losses < 0] = 0
    return np.diag(np.sqrt(losses))


def prepare_interferometer_matrix_in_expanded_space(interferometer_matrix) -> np.ndarray:
    """2m x 2m unitary dilation of a (lossy) m x m interferometer: its SVD V diag(s) W,
    with the lost amplitude sqrt(1 - s^2) routed into m extra modes."""
    v, s, w = np.linalg.svd(interferometer_matrix)
    zeros = np.zeros_like(v)
    eye = np.eye(len(v))
    expanded_v = np.block([[v, zeros], [zeros, eye]])
    expanded_w = np.block([[w, zeros], [zeros, eye]])
    t = np.array([x ** 2 for x in s])
    ext = _loss_transfer_expansion(t)
    sigma = np.block([[np.diag(s), ext], [ext, np.diag(s)]])
    return expanded_v @ sigma @ expanded_w


def haar_unitary(m: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return np.ascontiguousarray(q * (d / np.abs(d)), dtype=np.complex128)
