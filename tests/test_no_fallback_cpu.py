"""The product path has no CPU fallback: without libdeo.so the package
raises, and on a machine without a GPU every apply raises a deo error from
the C ABI instead of computing anything on the host."""
import numpy as np
import pytest

import deo
from deo import _lib


def test_missing_library_raises(monkeypatch):
    monkeypatch.setattr(_lib, "LIB_PATH", "/nonexistent/libdeo.so")
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError, match="libdeo.so not found"):
        _lib.lib()


def test_applies_without_a_gpu_raise():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("checks the behaviour on a machine without a GPU")
    A = deo.CenteredDifference(2, 2, 0.1, 16) * deo.Dirichlet0BC(np.float64)
    with pytest.raises(deo.DeoError):
        A * np.zeros(16)                      # host buffers through deo_apply_host
    with pytest.raises(deo.DeoError, match="CUDA"):
        A * torch.zeros(16, dtype=torch.float64)  # the plan's tables need device memory
    with pytest.raises(deo.DeoArgError, match="CUDA tensor"):
        deo.CenteredDifference(2, 2, 0.1, 16) * torch.zeros(18, dtype=torch.float64)
