"""GPU parity of the per-call primitives (GetForce, mass, StableTimeStep,
Gauss-point stress) against the reference's own outputs (golden) and the FP64
oracle.  Tolerances: FP64 mode 1e-10 relative (reassociation only); mixed mode
(FP32 element kinematics) 2e-4 relative on nodal forces."""
import numpy as np
import pytest

import femtech_gb300 as ft
from femtech_gb300 import meshgen as mg
from helpers import MATS, golden_mesh, random_fibers, rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 2e-4


@pytest.mark.parametrize("name", ["hex", "tet"])
@pytest.mark.parametrize("mid", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("prec", [ft.FP64, ft.MIXED])
def test_force_matches_reference(golden, name, mid, prec):
    f = golden["ref_force"]
    mesh = golden_mesh(golden, name)
    m = ft.Model(mesh, mg.materials([(mid, MATS[mid])]), precision=prec)
    tol = FP64_TOL if prec == ft.FP64 else MIXED_TOL
    np.testing.assert_allclose(m.mass, f["%s_m%d_mass" % (name, mid)], rtol=1e-12)
    u = f[name + "_u"]
    for k in range(3):  # consecutive calls (material 5 history advances per call)
        fi = m.GetForce(u[k], 1.0e-6)
        assert rel(fi, f["%s_m%d_fi" % (name, mid)][k]) < tol
        pk2 = m.gauss_points()[2]
        assert rel(pk2, f["%s_m%d_pk2" % (name, mid)][k]) < (tol if mid != 3 else 10 * tol)
        dt = m.StableTimeStep(u[k])
        assert dt == pytest.approx(f["%s_m%d_dt" % (name, mid)][k],
                                   rel=1e-12 if prec == ft.FP64 else 1e-5)
    m.close()


@pytest.mark.parametrize("name", ["hex", "tet"])
@pytest.mark.parametrize("mid", [6, 7])
@pytest.mark.parametrize("prec", [ft.FP64, ft.MIXED])
def test_new_materials_match_oracle(oracle_lib, golden, name, mid, prec):
    f = golden["ref_force"]
    mesh = dict(golden_mesh(golden, name))
    E = len(mesh["etype"])
    mesh["fiber"] = random_fibers(E, seed=3)
    mats = mg.materials([(mid, MATS[mid])])
    o = oracle_lib.Oracle(mesh, mats)
    m = ft.Model(mesh, mats, precision=prec)
    u = f[name + "_u"]
    tol = FP64_TOL * 100 if prec == ft.FP64 else MIXED_TOL
    for k in range(3):
        fo = o.get_force(u[k], 2.0e-6)
        fg = m.GetForce(u[k], 2.0e-6)
        assert rel(fg, fo) < tol
    m.close()


def test_mixed_force_on_jittered_block_vs_oracle(oracle_lib):
    mesh = mg.hex_block(12, 10, 8, 0.012, 0.010, 0.008, jitter=0.1, seed=2)
    mats = mg.materials([(6, MATS[6])])
    rng = np.random.default_rng(0)
    u = rng.normal(0, 2e-6, 3 * len(mesh["coordinates"]))
    o = oracle_lib.Oracle(mesh, mats, threads=4)
    m = ft.Model(mesh, mats, precision=ft.MIXED)
    assert rel(m.GetForce(u), o.get_force(u, 0.0)) < MIXED_TOL
    b = np.zeros(len(u), np.int32)
    assert m.StableTimeStep(u) == pytest.approx(o.stable_time_step(u, b), rel=1e-5)


def test_patch_sizes_agree(oracle_lib):
    mesh = mg.hex_block(9, 7, 5, 0.009, 0.007, 0.005, jitter=0.1, seed=4)
    mats = mg.materials([(1, MATS[1])])
    u = np.random.default_rng(1).normal(0, 1e-6, 3 * len(mesh["coordinates"]))
    ref = oracle_lib.Oracle(mesh, mats).get_force(u, 0.0)
    for pe in (32, 64, 128, 256):
        m = ft.Model(mesh, mats, precision=ft.FP64 if pe <= 128 else ft.MIXED, patch_size=pe)
        assert rel(m.GetForce(u), ref) < (FP64_TOL if pe <= 128 else MIXED_TOL)
        m.close()


def test_mixed_hex_tet_mesh(oracle_lib):
    hexm = mg.hex_block(3, 3, 3, 0.003, 0.003, 0.003, jitter=0.1, seed=8)
    tetm = mg.tet_ellipsoid(0.002, 0.002, 0.002, 0.0008, seed=9)
    n1 = len(hexm["coordinates"])
    tet_conn = tetm["connectivity"] + n1
    mesh = dict(coordinates=np.concatenate([hexm["coordinates"], tetm["coordinates"] + 0.01]),
                eptr=np.concatenate([hexm["eptr"], hexm["eptr"][-1] + tetm["eptr"][1:]]).astype(np.int32),
                connectivity=np.concatenate([hexm["connectivity"], tet_conn]).astype(np.int32),
                etype=np.concatenate([hexm["etype"], tetm["etype"]]),
                pid=np.concatenate([np.zeros(len(hexm["etype"]), np.int32),
                                    np.ones(len(tetm["etype"]), np.int32)]))
    mats = mg.materials([(1, MATS[1]), (4, MATS[4])])
    u = np.random.default_rng(2).normal(0, 1e-6, 3 * len(mesh["coordinates"]))
    ref = oracle_lib.Oracle(mesh, mats).get_force(u, 0.0)
    m = ft.Model(mesh, mats, precision=ft.FP64)
    assert rel(m.GetForce(u), ref) < FP64_TOL
    F, J, S = m.gauss_points()
    assert F.shape[0] == 8 * 27 + len(tetm["etype"])


def test_rigid_motion_gives_no_force():
    mesh = mg.hex_block(4, 4, 4, 0.004, 0.004, 0.004, jitter=0.1, seed=3)
    X = mesh["coordinates"]
    th = 0.3
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    u = (X @ R.T - X + np.array([1e-3, -2e-3, 5e-4])).ravel()
    for mid in (1, 4, 6):
        m = ft.Model(mesh, mg.materials([(mid, MATS[mid])]), precision=ft.FP64)
        fi = m.GetForce(u)
        scale = MATS[mid][1] * 0.004 ** 2
        assert np.abs(fi).max() < 1e-9 * scale
        m.close()


@pytest.mark.parametrize("alpha", [5.0, -5.0, 0.2])
@pytest.mark.parametrize("g", [0.02, 0.06, 0.12, 0.2])
def test_mixed_ogden_finite_strain_vs_oracle(oracle_lib, alpha, g):
    """FP32 Ogden (series below its alpha-dependent bound, eigen-decomposition
    above it) against the FP64 oracle on a finitely strained jittered block:
    an affine stretch / shear of size g plus noise."""
    mesh = mg.hex_block(6, 5, 4, 0.006, 0.005, 0.004, jitter=0.1, seed=7)
    mats = mg.materials([(6, [1040.0, 1.5e3, 2.0e7, alpha])])
    X = mesh["coordinates"]
    rng = np.random.default_rng(int(100 * g) + int(abs(alpha) * 10))
    G = g * rng.normal(size=(3, 3)) / 2
    u = (X @ G.T + rng.normal(0, 1e-3 * g * 1e-3, X.shape)).ravel()
    o = oracle_lib.Oracle(mesh, mats)
    m = ft.Model(mesh, mats, precision=ft.MIXED)
    assert rel(m.GetForce(u), o.get_force(u, 0.0)) < MIXED_TOL
    m.close()
