"""The learned constitutive surrogate (material 7).

CPU: the FP64 MLP checker (oracle/mlp_oracle.py) against finite differences.
GPU: the BF16 tensor-core forward/backward against that checker, the training
data against the plain law, and what the trained network gains over the
method without it (the law's first-order model S_lin)."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

PROPS7 = [1040.0, 1.0e3, 2.19e8, 5.0e3, 10.0, 0.6, 6.0e-3, 0.1]


def rand_params(rng, scale=0.3):
    p = rng.normal(0.0, scale, mo.NPARAMS)
    w = p.copy()
    for k in ("W0", "W1", "W2", "W3"):
        a, b = mo.OFF[k]
        fan_in = mo.NI if k == "W0" else mo.NH
        w[a:b] /= np.sqrt(fan_in) / 2
    return w


def rand_batch(rng, n):
    x = np.zeros((n, mo.NI))
    x[:, :9] = rng.uniform(-1, 1, (n, 9))
    t = np.zeros((n, mo.NO))
    t[:, :6] = rng.normal(0, 1, (n, 6))
    return x, t


def test_fp64_mlp_checker_gradient_by_finite_differences():
    rng = np.random.default_rng(0)
    p = rand_params(rng)
    x, t = rand_batch(rng, 16)
    loss, g = mo.loss_and_grad(p, x, t, quantize=False)
    for idx in rng.choice(mo.NPARAMS, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (mo.loss_and_grad(pp, x, t, quantize=False)[0] -
              mo.loss_and_grad(pm, x, t, quantize=False)[0]) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)), idx


def goh_iso_fp64(U, a0):
    """Isochoric PK2 of the plain material-7 law (oracle), Voigt."""
    from oracle.oracle import material_stress
    mu, lam = PROPS7[1], PROPS7[2]
    K = lam + 2 * mu / 3
    S = material_stress(7, PROPS7[:5] + [0.0, 1.0, PROPS7[7]], U.ravel(order="F"), a0=a0, dt=1e-4,
                        hist=np.zeros(27))
    J = np.linalg.det(U)
    Ci = np.linalg.inv(U.T @ U)
    Sv = 0.5 * K * (J * J - 1) * Ci
    return S - np.array([Sv[0, 0], Sv[1, 1], Sv[2, 2], Sv[1, 2], Sv[0, 2], Sv[0, 1]])


def held_out_states(rng, n, lo=0.7, hi=1.4):
    Es, As, Ss = [], [], []
    for _ in range(n):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        U = Q @ np.diag(rng.uniform(lo, hi, 3)) @ Q.T
        a0 = rng.normal(size=3)
        a0 /= np.linalg.norm(a0)
        E = 0.5 * (U.T @ U - np.eye(3))
        Es.append([E[0, 0], E[1, 1], E[2, 2], E[1, 2], E[0, 2], E[0, 1]])
        As.append(a0)
        Ss.append(goh_iso_fp64(U, a0))
    return np.array(Es), np.array(As), np.array(Ss)


def test_fibre_strain_mirror_matches_invariants():
    from femtech_gb300.surrogate import fibre_strain
    rng = np.random.default_rng(3)
    kappa = PROPS7[7]
    for _ in range(50):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        U = Q @ np.diag(rng.uniform(0.8, 1.2, 3)) @ Q.T
        a0 = rng.normal(size=3)
        a0 /= np.linalg.norm(a0)
        C = U.T @ U
        E = 0.5 * (C - np.eye(3))
        Ev = np.array([[E[0, 0], E[1, 1], E[2, 2], E[1, 2], E[0, 2], E[0, 1]]])
        j23 = np.linalg.det(C) ** (-1.0 / 3.0)
        want = kappa * (j23 * np.trace(C) - 3) + (1 - 3 * kappa) * (j23 * a0 @ C @ a0 - 1)
        assert abs(fibre_strain(Ev, a0[None], kappa)[0] - want) <= 1e-12


def test_first_order_model_residual_is_second_order():
    """(S_iso - S_lin) / |E|^2 stays bounded as the strain shrinks: the network
    only has to carry an O(|E|^2) correction (plain law from the oracle)."""
    from femtech_gb300.surrogate import linear_part, e2_of
    rng = np.random.default_rng(4)
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    d = np.array([0.7, -0.2, 0.4])
    a0 = np.array([0.6, 0.0, 0.8])
    ratios = []
    for eps in (1e-1, 1e-2, 1e-3):
        U = Q @ np.diag(1 + eps * d) @ Q.T
        E = 0.5 * (U.T @ U - np.eye(3))
        Ev = np.array([[E[0, 0], E[1, 1], E[2, 2], E[1, 2], E[0, 2], E[0, 1]]])
        r = goh_iso_fp64(U, a0) - linear_part(Ev, a0[None], PROPS7[1], PROPS7[3], PROPS7[7])[0]
        ratios.append(np.linalg.norm(r) / e2_of(Ev)[0])
    assert max(ratios) < 10 * (PROPS7[1] + PROPS7[3]), ratios
    assert ratios[2] < 2 * ratios[1] + 1.0, ratios


@pytest.mark.gpu
def test_tensor_core_gradient_matches_fp64_checker():
    from femtech_gb300.surrogate import Surrogate
    s = Surrogate(PROPS7, seed=3)
    rng = np.random.default_rng(1)
    s.params = rand_params(rng).astype(np.float32)
    p = s.params.astype(np.float64)
    x, t = rand_batch(rng, 1024)
    g_gpu, l_gpu = s.gradient(x, t)
    l_ref, g_ref = mo.loss_and_grad(p, x, t, quantize=True)
    assert abs(l_gpu - l_ref) <= 2e-3 * l_ref
    for k, (a, b) in mo.OFF.items():
        err = np.linalg.norm(g_gpu[a:b] - g_ref[a:b]) / max(np.linalg.norm(g_ref[a:b]), 1e-30)
        assert err < 2e-2, (k, err)
    y_gpu = s.forward(x)
    y_ref, _ = mo.forward(p, x, quantize=True)
    assert np.abs(y_gpu - y_ref).max() <= 1e-2 * np.abs(y_ref).max()
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [100, 3001])
def test_tcgen05_training_gemms_match_mma_sync(n):
    """Forward, dX and dW on tcgen05 (TMEM accumulators, weight gradients
    split over K) against the warp-level mma.sync kernels: a batch below one
    128-row tile and a ragged one over 12 K slices."""
    from femtech_gb300.surrogate import Surrogate
    s = Surrogate(PROPS7, seed=3)
    rng = np.random.default_rng(7)
    s.params = rand_params(rng).astype(np.float32)
    x, t = rand_batch(rng, n)
    out = {}
    for tc in (True, False):
        s.gemm_path(tc)
        g, loss = s.gradient(x, t)
        out[tc] = (g, loss, s.forward(x))
    s.close()
    (g1, l1, y1), (g0, l0, y0) = out[True], out[False]
    assert abs(l1 - l0) <= 1e-4 * l0
    assert np.abs(y1 - y0).max() <= 2e-3 * np.abs(y0).max()
    for k, (a, b) in mo.OFF.items():
        err = np.linalg.norm(g1[a:b] - g0[a:b]) / max(np.linalg.norm(g0[a:b]), 1e-30)
        assert err < 5e-3, (k, err)


@pytest.mark.gpu
def test_training_samples_follow_the_plain_law():
    from femtech_gb300 import surrogate as sg
    s = sg.Surrogate(PROPS7, seed=4)
    s.generate(4096, seed=9)
    x, t = s.samples(64)
    assert np.all(np.isfinite(t)) and np.all(t[:, 6:] == 0)
    # rebuild the strain from the (BF16) features and check the residual target
    E = sg.strain_of(x)
    a0 = x[:, 7:10].astype(np.float64)
    a0 /= np.linalg.norm(a0, axis=1, keepdims=True)
    assert s.out_scale > 0
    errs = []
    for i in range(len(E)):
        Em = np.array([[E[i, 0], E[i, 5], E[i, 4]], [E[i, 5], E[i, 1], E[i, 3]],
                       [E[i, 4], E[i, 3], E[i, 2]]])
        w, V = np.linalg.eigh(np.eye(3) + 2 * Em)
        U = V @ np.diag(np.sqrt(w)) @ V.T
        S = goh_iso_fp64(U, a0[i])
        r = (S - sg.linear_part(E[i:i + 1], a0[i:i + 1], s.mu, s.k1, s.kappa)[0]) / (
            s.s0 * s.out_scale * sg.e2_of(E[i:i + 1])[0])
        errs.append(np.abs(r - t[i, :6]).max() / max(np.abs(t[i, :6]).max(), 1e-3))
    assert np.median(errs) < 0.05  # features are BF16-rounded strains
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [5, 3001, 70000])
def test_tensor_core_inference_matches_mma_and_training_forward(n):
    """tcgen05 inference (TMEM accumulators) against the warp-level mma.sync
    kernel and the training forward: fewer rows than one 128-row tile, a
    ragged last tile, and many tiles per CTA."""
    from femtech_gb300.surrogate import Surrogate
    import ctypes as C
    s = Surrogate(PROPS7, seed=6)
    rng = np.random.default_rng(2)
    s.params = rand_params(rng).astype(np.float32)
    x, _ = rand_batch(rng, n)
    x = x.astype(np.float32)
    y_gen = s.forward(x)
    out = {}
    for name in ("ftgpu_surrogate_infer", "ftgpu_surrogate_infer_mma"):
        f = getattr(s.L, name)
        f.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
        y = np.zeros_like(y_gen)
        assert f(s.h, len(x), x.ctypes.data, y.ctypes.data) == 0, name
        out[name] = y
    scale = np.abs(y_gen).max()
    e_tc = np.abs(out["ftgpu_surrogate_infer"] - y_gen).max() / scale
    e_mma = np.abs(out["ftgpu_surrogate_infer_mma"] - y_gen).max() / scale
    print("n=%d: tcgen05 %.2e, mma.sync %.2e (max error / max |y|)" % (n, e_tc, e_mma))
    assert np.abs(out["ftgpu_surrogate_infer"] - y_gen).max() <= 1e-2 * scale
    assert np.abs(out["ftgpu_surrogate_infer_mma"] - y_gen).max() <= 1e-2 * scale
    assert np.abs(out["ftgpu_surrogate_infer"] - out["ftgpu_surrogate_infer_mma"]).max() <= 1e-2 * scale
    s.close()


@pytest.mark.gpu
def test_surrogate_outside_trust_region_equals_plain_path():
    import femtech_gb300 as ft
    from femtech_gb300 import meshgen as mg
    from femtech_gb300.surrogate import Surrogate
    mesh, mats, loads = mg.head_case(target_elements=8_000, seed=2)
    s = Surrogate(PROPS7, seed=1)  # untrained: every Gauss point must fall back
    out = []
    for use in (False, True):
        m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
        if use:
            m.set_surrogate(s, trust_e2=-1.0)
        m.init_explicit(0.9, 0.0, 1.0)
        m.run(120)
        out.append(m.state()["u"])
        m.close()
    assert np.array_equal(out[0], out[1])
    s.close()


@pytest.mark.gpu
def test_trained_network_gains_over_the_linearised_law():
    from femtech_gb300.surrogate import Surrogate, linear_part
    s = Surrogate(PROPS7, seed=5)
    s.generate(4_000_000, seed=11)
    loss = s.train(epochs=4, batch=4096, lr=2e-3)
    assert np.isfinite(loss)
    # held-out states inside the sampled box (stretches 0.85..1.15, |E|_F^2 < 0.06);
    # the method without the network is the law's linearisation S_lin
    rng = np.random.default_rng(12)
    E, A, S = held_out_states(rng, 400, 0.85, 1.15)
    pred = s.predict(E, A)
    lin = linear_part(E, A, s.mu, s.k1, s.kappa)
    err_nn = np.linalg.norm(pred - S) / np.linalg.norm(S)
    err_lin = np.linalg.norm(lin - S) / np.linalg.norm(S)
    print("held-out relative stress error: network %.4f, linearisation %.4f" % (err_nn, err_lin))
    assert err_nn < 0.05 and err_nn < err_lin / 5, (err_nn, err_lin)
    s.close()
