"""Clements mesh: m(m-1)/2 interferometers in m layers give a unitary (CPU only)."""
import numpy as np
import pytest


def test_clements_mesh_is_unitary_and_complete():
    torch = pytest.importorskip("torch")
    from theboss_gb300.adjoint import clements_layers, clements_unitary

    m = 24
    assert sum(len(l) for l in clements_layers(m)) == m * (m - 1) // 2 == 276
    g = torch.Generator().manual_seed(1)
    th = torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi
    ph = torch.rand(276, generator=g, dtype=torch.float64) * 2 * np.pi
    U = clements_unitary(th, ph).numpy()
    assert np.allclose(U.conj().T @ U, np.eye(m), atol=1e-13)
