"""Host-side helpers of the sampling path (numpy, no GPU work).

  mode_occupation_to_mode_assignment          boson_sampling_utilities.py:61-78
  prepare_interferometer_matrix_in_expanded_space
                                              boson_sampling_utilities.py:264-342
  haar_unitary                                seeded Haar-random unitary (Mezzadri's
                                              QR of a complex Gaussian matrix with the
                                              phases of R's diagonal divided out)
"""
from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np


def mode_occupation_to_mode_assignment(mode_occupation: Sequence[int]) -> Tuple[int, ...]:
    out = []
    for i, v in enumerate(mode_occupation):
        out += [i] * int(v)
    return tuple(out)


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
