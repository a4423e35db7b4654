"""The C-ABI library builds, loads and exports every entry point of include/boss.h (CPU only)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "boss.h")).read()
    return sorted(set(re.findall(r"BOSS_API\s+[\w\s\*]+?\b(boss_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from theboss_gb300 import _native

    lib = _native.load()
    names = _declared()
    assert "boss_perm_batch" in names and "boss_submatrices_batch" in names
    for name in names:
        assert hasattr(lib, name), name
    assert lib.boss_abi_version() == 1


def test_library_is_in_tree():
    from theboss_gb300 import _native

    path = _native.library_path()
    assert os.path.commonpath([os.path.realpath(path), os.path.realpath(ROOT)]) == os.path.realpath(ROOT)


def test_no_gpu_calls_fail_loudly_without_device():
    """Without a GPU the library reports it; it never computes on the host."""
    import numpy as np
    import pytest
    from theboss_gb300 import _native
    from theboss_gb300.permanent_calculators import RyserPermanentCalculator

    try:
        import torch  # noqa: F401

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(_native.GB300Error):
        RyserPermanentCalculator(np.eye(3, dtype=complex), [1, 1, 0], [1, 1, 0]).compute_permanent()


def test_arithmetic_switches_set_query_and_reject_bad_modes():
    """boss_minors_arithmetic / boss_perm_arithmetic only record the choice (no
    GPU needed): FP64 by default, float pairs on request, -1 queries."""
    import pytest
    from theboss_gb300 import _native

    for setter in (_native.minors_arithmetic, _native.perm_arithmetic):
        start = setter(-1)
        assert start in (_native.FLOAT_PAIRS, _native.FP64)
        try:
            assert setter(_native.FP64) == start
            assert setter(-1) == _native.FP64
            assert setter(_native.FLOAT_PAIRS) == _native.FP64
            assert setter(-1) == _native.FLOAT_PAIRS
            with pytest.raises(ValueError):  # BOSS_ERR_ARG
                setter(2)
            assert setter(-1) == _native.FLOAT_PAIRS
        finally:
            setter(start)
    assert _native.minors_arithmetic(-1) == _native.FP64  # the library's default
    assert _native.perm_arithmetic(-1) == _native.FP64
