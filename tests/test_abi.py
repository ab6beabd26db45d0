"""The C-ABI library builds, loads without a GPU, and exports every entry point
that include/*.h declares (no compute calls: this runs on CPU-only hosts)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ftgpu_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from femtech_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "ftgpu_get_force" in names and "ftgpu_run" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_without_gpu(libpath):
    lib = ctypes.CDLL(libpath)
    lib.ftgpu_status_string.restype = ctypes.c_char_p
    assert lib.ftgpu_status_string(-19) == b"time step below FailureTimeStep"
    assert lib.ftgpu_status_string(-1) == b"unknown material"


def test_create_fails_loudly_without_device(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from femtech_gb300 import Model, FtgpuError, meshgen as mg
    mesh = mg.hex_block(1, 1, 1, 1.0, 1.0, 1.0)
    with pytest.raises(FtgpuError) as ei:
        Model(mesh, mg.materials([(1, [1.0, 1.0, 1.0])]))
    assert ei.value.status == -32
