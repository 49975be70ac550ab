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
    assert lib.mbx_abi_version() == 4


def test_no_cpu_fallback_without_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        mbx.create_compute_backend("cuda")


def test_unknown_backend_name_rejected():
    with pytest.raises(ValueError):
        mbx.create_compute_backend("d3d11")


@pytest.mark.parametrize("cname,pytype", [("mbx_request", "_Request"), ("mbx_stats", "Stats")])
def test_struct_layout_matches_header(tmp_path, cname, pytype):
    """The binding's struct mirrors have the header's sizes and field offsets."""
    cls = getattr(mbx, pytype)
    src = tmp_path / "layout.c"
    fields = [f for f, _ in cls._fields_]
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "mbx_gb300.h"\nint main(void){printf("%%zu", sizeof(%s));' % cname
                   + "".join('printf(" %%zu", offsetof(%s, %s));' % (cname, f) for f in fields) + "return 0;}\n")
    exe = tmp_path / "layout"
    import subprocess

    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    vals = [int(x) for x in subprocess.check_output([str(exe)], text=True).split()]
    assert vals[0] == ctypes.sizeof(cls)
    assert vals[1:] == [getattr(cls, f).offset for f in fields]
