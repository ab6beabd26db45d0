"""Pin the FP64 oracle to the reference's own outputs (tests/golden, produced by
the reference sources compiled unmodified; see tests/golden/make_golden.py)."""
import numpy as np
import pytest

from helpers import MATS, ex9_mesh_loads, golden_mesh, rel
from femtech_gb300 import meshgen as mg


@pytest.mark.parametrize("name", ["hex", "tet"])
@pytest.mark.parametrize("mid", [1, 2, 3, 4, 5])
def test_force_mass_dt_pk2_match_reference(oracle_lib, golden, name, mid):
    f = golden["ref_force"]
    mesh = golden_mesh(golden, name)
    o = oracle_lib.Oracle(mesh, mg.materials([(mid, MATS[mid])]))
    np.testing.assert_allclose(o.mass, f["%s_m%d_mass" % (name, mid)], rtol=1e-14, atol=0)
    u = f[name + "_u"]
    b = np.zeros(3 * o.nNodes, np.int32)
    for k in range(3):  # consecutive calls: viscoelastic history must advance identically
        fi = o.get_force(u[k], 1.0e-6)
        ref = f["%s_m%d_fi" % (name, mid)][k]
        assert rel(fi, ref) < 1e-13
        pk2 = o.gp_arrays()[2]
        assert rel(pk2, f["%s_m%d_pk2" % (name, mid)][k]) < 1e-13
        assert o.stable_time_step(u[k], b) == pytest.approx(f["%s_m%d_dt" % (name, mid)][k],
                                                            rel=1e-14)


@pytest.mark.parametrize("name", ["hex", "tet"])
def test_element_strain_matches_reference(oracle_lib, golden, name):
    """CalculateMaximumPrincipalStrain (CalculateStrain.cpp:8-75) on three states."""
    f = golden["ref_force"]
    mesh = golden_mesh(golden, name)
    o = oracle_lib.Oracle(mesh, mg.materials([(1, MATS[1])]))
    for k in range(3):
        o.get_force(f[name + "_u"][k], 1.0e-6)
        E9, mx, mn, sh = o.element_strain()
        got = np.concatenate([E9, mx[:, None], mn[:, None], sh[:, None]], 1)
        np.testing.assert_array_equal(got, f[name + "_strain"][k])


def test_percentile95_matches_reference(oracle_lib, golden):
    """compute95thPercentileValue(BruteForce) of math.cpp, incl. ties and n = 20, 21."""
    f = golden["ref_force"]
    i = 0
    while "pct_data_%d" % i in f.files:
        assert oracle_lib.percentile95(f["pct_data_%d" % i]) == float(f["pct_ref_%d" % i])
        i += 1
    assert i == 5


def test_ex9_loop_matches_reference_and_abaqus(oracle_lib, golden):
    g = golden["ref_ex9"]
    mesh, mats, loads = ex9_mesh_loads()
    o = oracle_lib.Oracle(mesh, mats)
    res = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.8, max_steps=100000,
                         out_every=1)
    assert res["steps"] == int(g["steps"])
    assert rel(res["u_out"], g["u_out"]) < 1e-12
    # the reference CI check (examples/ex9/compareResults.py:14-25): node
    # (0.005,0.005,0.005) within 5 % of Abaqus, final time within 1 %
    abq = g["abaqus_last"]
    assert abs(res["time"] - abq[0]) / abq[0] < 0.01
    u8 = res["u"][21:24]
    assert np.max(np.abs((u8 - abq[1:]) / abq[1:])) < 0.05


def test_cube_tension_matches_reference(oracle_lib, golden):
    g = golden["ref_cube"]
    mesh, mats, loads = mg.cube_tension_case(n=10)
    o = oracle_lib.Oracle(mesh, mats, threads=4)
    res = o.explicit_run(loads.dof_fn, loads.fns, tmax=0.01, reduction=0.9, max_steps=100000,
                         out_every=100, energy=True)
    assert res["steps"] == int(g["steps"])
    np.testing.assert_allclose(res["t_out"], g["t_out"], rtol=1e-14)
    assert rel(res["u_out"], g["u_out"]) < 1e-12
    # CheckEnergy every step: internal work, external work, kinetic energy
    assert res["energy"].shape == g["energy"].shape
    assert rel(res["energy"], g["energy"]) < 1e-12
