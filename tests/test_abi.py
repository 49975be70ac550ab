"""The C-ABI library: it loads, exports every entry point include/mbx_gb300.h
declares, and (without a GPU) refuses to create a context instead of falling
back to the CPU. No compute calls here."""
import ctypes
import os
import re

import pytest

import mbx
from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "mbx_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mbx_[a-z_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert set(declared_functions()) == set(mbx.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = mbx.load_library()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.mbx_abi_version() == 1


def test_no_cpu_fallback_without_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        mbx.create_compute_backend("cuda")


def test_unknown_backend_name_rejected():
    with pytest.raises(ValueError):
        mbx.create_compute_backend("d3d11")
