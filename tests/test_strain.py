"""Element strain (CalculateStrain / CalculateMaximumPrincipalStrain) on the GPU
against the reference's own values (tests/golden/ref_force.npz, material 1)."""
import numpy as np
import pytest

from helpers import MATS, golden_mesh
from femtech_gb300 import meshgen as mg


def _gpu_strain(ft, mesh, u, precision):
    m = ft.Model(mesh, mg.materials([(1, MATS[1])]), precision=precision)
    m.set_state(u=u)
    E9, mx, mn, sh = m.element_strain()
    m.close()
    return np.concatenate([E9, mx[:, None], mn[:, None], sh[:, None]], 1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hex", "tet"])
def test_fp64_element_strain_matches_reference(golden, name):
    import femtech_gb300 as ft
    f = golden["ref_force"]
    mesh = golden_mesh(golden, name)
    for k in range(3):
        got = _gpu_strain(ft, mesh, f[name + "_u"][k], ft.FP64)
        ref = f[name + "_strain"][k]
        scale = np.abs(ref[:, :9]).max()
        assert np.abs(got[:, :9] - ref[:, :9]).max() <= 1e-12 * scale
        assert np.abs(got[:, 9:] - ref[:, 9:]).max() <= 1e-10 * scale


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hex", "tet"])
def test_mixed_element_strain_within_fp32(golden, name):
    import femtech_gb300 as ft
    f = golden["ref_force"]
    mesh = golden_mesh(golden, name)
    got = _gpu_strain(ft, mesh, f[name + "_u"][0], ft.MIXED)
    ref = f[name + "_strain"][0]
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_element_strain_after_device_loop_matches_oracle(oracle_lib):
    import femtech_gb300 as ft
    mesh, mats, loads = mg.cube_tension_case(n=6)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    m.init_explicit(0.9, 0.0, 0.01)
    m.run(150)
    u = m.state()["u"]
    E9, mx, mn, sh = m.element_strain()
    m.close()
    o = oracle_lib.Oracle(mesh, mats)
    o.get_force(u, 0.0)
    rE9, rmx, rmn, rsh = o.element_strain()
    s = np.abs(rE9).max()
    assert s > 1e-4  # the loop has strained the cube
    assert np.abs(E9 - rE9).max() <= 1e-12 * s
    for a, b in ((mx, rmx), (mn, rmn), (sh, rsh)):
        assert np.abs(a - b).max() <= 1e-10 * s
