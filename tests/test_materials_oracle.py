"""Known-answer tests of the oracle's material laws, in particular the two laws
the reference does not have (6: Ogden, 7: anisotropic GOH + 1-term Prony),
which are pinned through reductions to reference laws and energy checks."""
import numpy as np
import pytest

from oracle.oracle import material_stress


def rand_F(rng, scale=0.15):
    F = np.eye(3) + rng.uniform(-scale, scale, (3, 3))
    if np.linalg.det(F) < 0.3:
        F = np.eye(3) + 0.3 * (F - np.eye(3))
    return F


def colmaj(F):
    return np.asarray(F).ravel(order="F")


def voigt_to_full(s):
    return np.array([[s[0], s[5], s[4]], [s[5], s[1], s[3]], [s[4], s[3], s[2]]])


def ogden_energy(F, mu, lam, alpha):
    K = lam + 2 * mu / 3
    J = np.linalg.det(F)
    Cb = J ** (-2 / 3) * F.T @ F
    w = np.linalg.eigvalsh(Cb)
    return 2 * mu / alpha ** 2 * np.sum(w ** (alpha / 2) - 1) + 0.5 * K * ((J * J - 1) / 2 - np.log(J))


@pytest.mark.parametrize("seed", range(5))
def test_ogden_alpha2_equals_reference_hgo_with_k1_zero(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    F = rand_F(rng)
    mu, lam = 1.5e3, 2.0e7
    s_og = material_stress(6, [1040, mu, lam, 2.0], colmaj(F))
    s_hgo = material_stress(4, [1040, mu, lam, 0.0, 10.0], colmaj(F))
    np.testing.assert_allclose(s_og, s_hgo, rtol=1e-9, atol=1e-9 * np.abs(s_hgo).max())


@pytest.mark.parametrize("alpha", [5.0, -3.0, 8.0, 0.5])
def test_ogden_stress_is_energy_derivative(oracle_lib, alpha):
    rng = np.random.default_rng(7)
    F = rand_F(rng, 0.1)
    mu, lam = 1.5e3, 5.0e4
    S = voigt_to_full(material_stress(6, [1040, mu, lam, alpha], colmaj(F)))
    # S = 2 dW/dC ; P = F S = dW/dF, checked by central differences
    P = F @ S
    h = 1e-6
    Pfd = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            Fp, Fm = F.copy(), F.copy()
            Fp[i, j] += h
            Fm[i, j] -= h
            Pfd[i, j] = (ogden_energy(Fp, mu, lam, alpha) - ogden_energy(Fm, mu, lam, alpha)) / (2 * h)
    np.testing.assert_allclose(P, Pfd, rtol=1e-5, atol=1e-5 * np.abs(Pfd).max())


def test_ogden_undeformed_and_degenerate(oracle_lib):
    s = material_stress(6, [1040, 1.5e3, 2.0e7, 5.0], colmaj(np.eye(3)))
    assert np.abs(s).max() < 1e-9
    # equal principal stretches (pure dilatation): deviatoric part vanishes
    F = 1.01 * np.eye(3)
    s = material_stress(6, [1040, 1.5e3, 2.0e7, 5.0], colmaj(F))
    assert abs(s[0] - s[1]) < 1e-9 * abs(s[0]) and abs(s[3]) < 1e-9 * abs(s[0])


@pytest.mark.parametrize("seed", range(3))
def test_ogden_objectivity(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    F = rand_F(rng)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    p = [1040, 1.5e3, 2.0e7, 5.0]
    np.testing.assert_allclose(material_stress(6, p, colmaj(q @ F)), material_stress(6, p, colmaj(F)),
                               rtol=1e-8, atol=1e-8)


@pytest.mark.parametrize("seed", range(4))
def test_goh_kappa_third_equals_reference_visco_with_one_term(oracle_lib, seed):
    rng = np.random.default_rng(seed)
    a0 = rng.normal(size=3)
    a0 /= np.linalg.norm(a0)
    p7 = [1040, 1.0e3, 2.19e5, 5.0e3, 10.0, 0.6, 6e-3, 1.0 / 3.0]
    p5 = [1040, 1.0e3, 2.19e5, 5.0e3, 10.0, 0.6, 6e-3, 0.0, 1.0]
    h7, h5 = np.zeros(27), np.zeros(27)
    for k in range(4):  # a short deformation path: history must evolve identically
        F = rand_F(rng, 0.12)
        s7 = material_stress(7, p7, colmaj(F), a0=a0, dt=1e-4, hist=h7)
        s5 = material_stress(5, p5, colmaj(F), dt=1e-4, hist=h5)
        np.testing.assert_allclose(s7, s5, rtol=1e-10, atol=1e-10 * np.abs(s5).max())


def test_goh_fiber_stiffens_along_fiber(oracle_lib):
    # stretch along the fibre: kappa = 0 (aligned) is stiffer than kappa = 1/3 (isotropic)
    F = np.diag([1.1, 1 / np.sqrt(1.1), 1 / np.sqrt(1.1)])
    a0 = np.array([1.0, 0.0, 0.0])
    base = [1040, 1.0e3, 2.19e5, 5.0e3, 10.0, 0.0, 1.0]
    s_al = material_stress(7, base + [0.0], colmaj(F), a0=a0, dt=1e-4, hist=np.zeros(27))
    s_iso = material_stress(7, base + [1 / 3], colmaj(F), a0=a0, dt=1e-4, hist=np.zeros(27))
    assert s_al[0] - s_al[1] > s_iso[0] - s_iso[1] > 0


def test_rotation_bc_closed_form(oracle_lib):
    """The oracle's driver-side rigid rotation (half-sine angular acceleration
    about a fixed axis) against Rodrigues' formula at times inside and after
    the pulse."""
    import ctypes as C
    from femtech_gb300 import meshgen as mg
    mesh = mg.hex_block(2, 2, 2, 0.02, 0.02, 0.02)
    X = mesh["coordinates"]
    o = oracle_lib.Oracle(mesh, mg.materials([(1, [1000.0, 1e3, 1e5])]))
    loads = mg.Loads(len(X))
    ax = np.array([0.2, 0.5, 1.0])
    c = np.array([0.01, 0.0, -0.01])
    loads.rotation(np.arange(len(X)), ax, c, 6e3, 0.01)
    k = ax / np.linalg.norm(ax)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    tab = oracle_lib.bc_table(loads.fns)
    L = oracle_lib.Oracle.lib()
    L.or_apply_bc.argtypes = [C.POINTER(oracle_lib._Model), oracle_lib._ip, C.c_void_p,
                              C.c_double, oracle_lib._dp, oracle_lib._dp, oracle_lib._dp]
    for t in (0.004, 0.01, 0.015):
        u, v, a = np.zeros(3 * len(X)), np.zeros(3 * len(X)), np.ones(3 * len(X))
        L.or_apply_bc(C.byref(o.m), loads.dof_fn, C.cast(tab, C.c_void_p), t, u, v, a)
        a0, T = 6e3, 0.01
        if t <= T:
            th = a0 * T / np.pi * (t - T / np.pi * np.sin(np.pi * t / T))
            om = a0 * T / np.pi * (1 - np.cos(np.pi * t / T))
        else:
            om = 2 * a0 * T / np.pi
            th = a0 * T * T / np.pi + om * (t - T)
        R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
        rr = X - c
        np.testing.assert_allclose(u.reshape(-1, 3), rr @ R.T - rr, atol=1e-15)
        np.testing.assert_allclose(v.reshape(-1, 3), om * np.cross(k, rr @ R.T), atol=1e-12)
        assert np.all(a == 0)
