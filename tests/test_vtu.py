"""Output steps: the reference's ASCII VTU / PVTU / PVD files.

CPU: the engine's writer (host code) produces the reference writer's bytes
(tests/golden/ref_vtu.npz: WriteVTU + WritePVD of the reference on a mixed
mesh and a seeded state).  GPU: the model-level writer writes the device
state and the device-computed averaged strain."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden as mk  # noqa: E402


@pytest.fixture(scope="module")
def golden_vtu():
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                "ref_vtu.npz"))


@pytest.mark.parametrize("i", [0, 1])
def test_vtu_files_match_reference_bytes(golden_vtu, tmp_path, i):
    from femtech_gb300 import meshio
    g = golden_vtu
    name = str(g["vtu_name_%d" % i])
    mesh = mk.vtu_mesh()
    u, a, b, E, cells = mk.vtu_state(mesh)
    meshio.write_vtu_arrays(tmp_path, name, 3, mesh, u, a, b, E, cells)
    meshio.write_pvd(tmp_path, name, 3, g["vtu_times"])
    base = name.rsplit(".", 1)[0]
    for key, rel in (("vtu", "results/vtu/%s.vtu.0003.0000" % name),
                     ("pvtu", "results/%s.0003.pvtu" % name), ("pvd", base + ".pvd")):
        got = open(os.path.join(tmp_path, rel)).read()
        assert got == str(g["vtu_%s_%d" % (key, i)]), (name, key)


def _data_array(text, name):
    tag = 'Name="%s"' % name
    start = text.index(">", text.index(tag)) + 1
    return np.array(text[start:text.index("</DataArray>", start)].split(), np.float64)


@pytest.mark.gpu
def test_model_writes_device_state(tmp_path):
    import femtech_gb300 as ft
    from femtech_gb300 import meshgen as mg, meshio
    mesh, mats, loads = mg.cube_tension_case(n=6)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    m.init_explicit(0.9, 0.0, 0.01)
    m.run(150)
    st = m.state()
    E9 = m.element_strain()[0].ravel()
    flags = {"Flag": (np.arange(m.nE) % 3 == 0).astype(np.int32)}
    m.write_vtu(tmp_path / "a", "cube", 2, flags)
    meshio.write_vtu_arrays(tmp_path / "b", "cube", 2, mesh, st["u"], st["a"], loads.boundary,
                            E9, flags)
    fa = open(tmp_path / "a" / "results" / "vtu" / "cube.vtu.0002.0000").read()
    fb = open(tmp_path / "b" / "results" / "vtu" / "cube.vtu.0002.0000").read()
    assert fa == fb
    np.testing.assert_allclose(_data_array(fa, "Displacements"), st["u"], rtol=1e-8, atol=1e-20)
    np.testing.assert_allclose(_data_array(fa, "AvgStrain"), E9, rtol=1e-8, atol=1e-20)
    assert open(tmp_path / "a" / "results" / "cube.0002.pvtu").read() == \
        open(tmp_path / "b" / "results" / "cube.0002.pvtu").read()
    m.close()
