"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

from pyaxisymflow_gb300 import build as gbuild

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(REPO, "include", "axisym_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(axi_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = gbuild.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from pyaxisymflow_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES)
    lib = _native.lib()
    assert lib.axi_version() >= 100
    assert lib.axi_last_error() == b""


def test_no_cpu_fallback_for_cpu_tensors():
    import pytest
    import torch

    from pyaxisymflow_gb300.kernels.brinkmann_penalize import brinkmann_penalize
    t = torch.zeros((4, 4), dtype=torch.float64)
    with pytest.raises(ValueError, match="CUDA"):
        brinkmann_penalize(1.0, 1.0, t, 0.0, 0.0, t, t, t, t)
