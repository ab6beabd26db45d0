"""The reference-side drop-in (femtech_gb300/dropin/ftgpu_dropin.cpp).

CPU: it links against the reference's own hot-path objects in place of the
files it replaces (symbol compatibility; needs the reference tree, skipped
otherwise).  GPU: an ex9-shaped C++ driver using it reproduces the reference
ex9 run (golden) in FP64 mode."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "femtech_gb300", "dropin", "ftgpu_dropin.cpp")
REPLACED = {"GetForce.o", "GetForce_3D.o", "CalculateAcclerations.o", "StableTimeStep.o",
            "Mass3D.o"}


def _lib():
    from femtech_gb300 import build
    return build.build()


def test_dropin_links_in_place_of_reference_sources(tmp_path):
    from oracle import oracle as orc
    if not orc.RefBuild.available():
        pytest.skip("reference tree not available in this checkout")
    lib = _lib()
    objdir = os.path.join(ROOT, "oracle", "_ref", "obj")
    objs = []
    for d, _, files in os.walk(objdir):
        for f in files:
            if f.endswith(".o") and f not in REPLACED:
                objs.append(os.path.join(d, f))
    dobj = str(tmp_path / "dropin.o")
    subprocess.run(["g++", "-O2", "-fPIC", "-I", os.path.join(ROOT, "include"), "-c", DROPIN,
                    "-o", dobj], check=True)
    out = subprocess.run(["g++", "-shared", "-Wl,--no-undefined", "-o", str(tmp_path / "x.so"),
                          *objs, dobj, lib, "-lm"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-2000:]


@pytest.mark.gpu
def test_dropin_ex9_driver_matches_reference(golden, tmp_path):
    lib = _lib()
    exe = str(tmp_path / "ex9_gpu")
    subprocess.run(["g++", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin", "ex9_dropin_driver.cpp"), DROPIN,
                    lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    traj = str(tmp_path / "u.bin")
    out = subprocess.run([exe, traj], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    g = golden["ref_ex9"]
    u = np.fromfile(traj, dtype=np.float64).reshape(-1, 24)
    assert len(u) == int(g["steps"])
    err = np.linalg.norm(u - g["u_out"]) / np.linalg.norm(g["u_out"])
    assert err < 1e-5
