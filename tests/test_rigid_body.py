"""Rigid-body motion from sampled accelerations (the brain drivers' skull
boundary condition, examples/ex5/ex5.cpp:339-392 and 976-1020).

CPU: the oracle's interpolateLinear and per-node kinematics against the
reference's own math.cpp (tests/golden/ref_rigid.npz); its Dormand-Prince
step against closed forms and an independent quaternion integration.
GPU: the device loop against the oracle (integrator state, displacements,
energy), chunking, several instances, and the sampled drive against the
closed-form rotation it samples."""
import numpy as np
import pytest

from femtech_gb300 import meshgen as mg


def _zero():
    return (np.array([0.0, 1.0]), np.array([0.0, 0.0]))


def test_interp_linear_matches_reference(golden, oracle_lib):
    g = golden["ref_rigid"]
    for i in range(3):
        x, y, q = g["interp_x_%d" % i], g["interp_y_%d" % i], g["interp_q_%d" % i]
        got = np.array([oracle_lib.interp_linear(x, y, v) for v in q])
        assert np.array_equal(got, g["interp_ref_%d" % i]), i


def test_rigid_point_kinematics_match_reference(golden, oracle_lib):
    g = golden["ref_rigid"]
    rb = oracle_lib.RigidBody([_zero()] * 6)
    for y, yd, ref in zip(g["rigid_y"], g["rigid_yd"], g["rigid_uva"]):
        rb.set_state(y, yd)
        got = rb.point(g["rigid_X"])
        scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
        assert np.abs(got - ref).max() <= 1e-14 * scale.max(), np.abs(got - ref).max()


def test_integrator_exact_for_cubic_motion(oracle_lib):
    """a_cm = c t and alpha = b t (zero at t = 0, so the zero starting
    derivative of the drivers is exact): the fifth-order step reproduces the
    polynomial motion to rounding."""
    T = np.array([0.0, 1.0])
    c = np.array([3.0, -2.0, 5.0])
    rb = oracle_lib.RigidBody([_zero(), _zero(), _zero()] +
                              [(T, np.array([0.0, ck])) for ck in c])
    t, h = 0.0, 1.0e-3
    for _ in range(250):
        rb.step(t, h)
        t += h
    y = rb.y
    np.testing.assert_allclose(y[6:9], c * t * t / 2, rtol=1e-12)
    np.testing.assert_allclose(y[9:12], c * t ** 3 / 6, rtol=1e-12)
    np.testing.assert_allclose(rb.yd[6:9], c * t, rtol=1e-12)


def test_rotation_generator_rate_matches_quaternion_kinematics(oracle_lib):
    """Boyle's rate of the rotation generator (ex5.cpp:1001-1018) against an
    independent integration of dq/dt = [0, omega] q / 2 (spatial angular
    velocity) for an angular velocity that turns in space."""
    from scipy.integrate import solve_ivp
    T = np.linspace(0.0, 0.02, 81)
    chans = [(T, 3000.0 * np.sin(400.0 * T)), (T, 2000.0 * np.sin(300.0 * T)),
             (T, 1500.0 * T / 0.02)]
    rb = oracle_lib.RigidBody(chans + [_zero()] * 3)
    # the samples fall on step boundaries: within a step the accelerations
    # are linear, so the steps are exact up to the rotation's own truncation
    t, h = 0.0, 2.5e-5
    for _ in range(800):
        rb.step(t, h)
        t += h

    def alpha(s):
        return np.array([np.interp(s, *c) for c in chans])

    def qmul(p, q):
        return np.concatenate([[p[0] * q[0] - p[1:] @ q[1:]],
                               p[0] * q[1:] + q[0] * p[1:] + np.cross(p[1:], q[1:])])

    def f(s, z):
        return np.concatenate([alpha(s), 0.5 * qmul(np.concatenate([[0.0], z[:3]]), z[3:])])

    sol = solve_ivp(f, (0.0, t), np.array([0, 0, 0, 1.0, 0, 0, 0]), rtol=1e-12, atol=1e-14,
                    max_step=2.5e-5, t_eval=[t])
    r = rb.y[3:6]
    rm = np.linalg.norm(r)
    q = np.concatenate([[np.cos(rm)], np.sin(rm) / rm * r])
    np.testing.assert_allclose(rb.y[:3], sol.y[:3, -1], rtol=1e-9, atol=1e-9)
    assert np.abs(q - sol.y[3:, -1]).max() <= 1e-9


def test_sampled_fixed_axis_rotation_matches_closed_form(oracle_lib):
    """A half-sine angular acceleration about a fixed axis, sampled at 100 kHz,
    against the closed-form rotation of the same pulse (the engine's
    FTGPU_BCK_ROT function): the sampling error is O(dt_s^2)."""
    axis = np.array([0.3, -0.5, 0.8])
    axis /= np.linalg.norm(axis)
    a0, P = 6.0e3, 0.01
    ts = np.arange(0.0, 0.0200001, 1.0e-5)
    ang = a0 * np.where(ts <= P, np.sin(np.pi * ts / P), 0.0)
    rb = oracle_lib.RigidBody([(ts, ang * axis[k]) for k in range(3)] + [_zero()] * 3)
    X = np.array([[0.05, 0.02, -0.03], [-0.04, 0.06, 0.01]])
    t, h = 0.0, 1.0e-6
    for _ in range(15000):
        rb.step(t, h)
        t += h
    u, v, _ = rb.point(X)
    if t <= P:
        om = a0 * P / np.pi * (1 - np.cos(np.pi * t / P))
        th = a0 * P / np.pi * (t - P / np.pi * np.sin(np.pi * t / P))
    else:
        om = 2 * a0 * P / np.pi
        th = a0 * P * P / np.pi + om * (t - P)
    for i, x in enumerate(X):
        kx = np.cross(axis, x)
        Rx = x * np.cos(th) + kx * np.sin(th) + axis * (axis @ x) * (1 - np.cos(th))
        np.testing.assert_allclose(u[i], Rx - x, atol=1e-6 * np.linalg.norm(x))
        np.testing.assert_allclose(v[i], om * np.cross(axis, Rx), atol=1e-5 * om * np.linalg.norm(x))


# ------------------------------------------------------------------ GPU

def _case(n=4_000, seed=5):
    mesh, mats, loads, rec = mg.head_impact_case(target_elements=n, seed=seed)
    return mesh, mats, loads, rec


def _oracle_run(oracle_lib, mesh, mats, loads, rec, steps, energy=False):
    o = oracle_lib.Oracle(mesh, mats, threads=8)
    rb = oracle_lib.RigidBody(rec)
    res = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=steps,
                         out_every=steps, energy=energy, rigid=rb)
    return res, rb


def _model(ft, mesh, mats, loads, rec, precision, energy=False):
    m = ft.Model(mesh, mats, precision=precision, loads=loads)
    m.set_rigid_body(rec)
    if energy:
        m.set_energy(True)
    m.init_explicit(0.9, 0.0, 1.0)
    return m


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
def test_fp64_rigid_drive_matches_oracle(oracle_lib):
    import femtech_gb300 as ft
    mesh, mats, loads, rec = _case()
    steps = 300
    res, rb = _oracle_run(oracle_lib, mesh, mats, loads, rec, steps)
    m = _model(ft, mesh, mats, loads, rec, ft.FP64)
    assert m.run(steps) == steps
    y, yd = m.rigid_body()
    np.testing.assert_allclose(y, rb.y, rtol=1e-9, atol=1e-12 * np.abs(rb.y).max())
    np.testing.assert_allclose(yd, rb.yd, rtol=1e-9, atol=1e-12 * np.abs(rb.yd).max())
    st = m.state()
    print("u rel err %.2e, v %.2e, a(rigid) %.2e" % (
        _rel(st["u"], res["u"]), _rel(st["v"], res["v"]), _rel(st["a"], res["a"])))
    assert _rel(st["u"], res["u"]) <= 1e-5
    assert _rel(st["v"], res["v"]) <= 1e-5
    rig = np.repeat(mg.rigid_nodes(mesh, mats), 3) * 3 + np.tile([0, 1, 2],
                                                                len(mg.rigid_nodes(mesh, mats)))
    assert _rel(st["a"][rig], res["a"][rig]) <= 1e-8
    assert np.abs(res["u"][rig]).max() > 0
    m.close()


@pytest.mark.gpu
def test_mixed_rigid_drive_within_mixed_tolerance(oracle_lib):
    import femtech_gb300 as ft
    mesh, mats, loads, rec = _case()
    steps = 300
    res, rb = _oracle_run(oracle_lib, mesh, mats, loads, rec, steps)
    m = _model(ft, mesh, mats, loads, rec, ft.MIXED)
    assert m.run(steps) == steps
    y, _ = m.rigid_body()
    # the mixed loop's dt comes from FP32 element geometry: the state follows
    # the oracle's to the dt difference
    np.testing.assert_allclose(y, rb.y, rtol=1e-4, atol=1e-4 * np.abs(rb.y).max())
    assert _rel(m.state()["u"], res["u"]) <= 1e-3
    m.close()


@pytest.mark.gpu
def test_rigid_drive_chunked_equals_continuous():
    """Each step integrates the body once, whether it starts a chunk (its own
    kernel before the begin pass) or is fused into the previous step's end."""
    import femtech_gb300 as ft
    mesh, mats, loads, rec = _case(n=2_000)
    outs = []
    for chunks in ((120,), (7, 13, 16, 84)):
        m = _model(ft, mesh, mats, loads, rec, ft.FP64)
        for c in chunks:
            assert m.run(c) == c
        outs.append((m.state()["u"], m.rigid_body()[0]))
        m.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.gpu
def test_rigid_drive_energy_matches_oracle(oracle_lib):
    """CheckEnergy's reaction work m (a + a_prev) du on the driven DOFs."""
    import femtech_gb300 as ft
    mesh, mats, loads, rec = _case(n=3_000)
    steps = 120
    res, _ = _oracle_run(oracle_lib, mesh, mats, loads, rec, steps, energy=True)
    m = _model(ft, mesh, mats, loads, rec, ft.FP64, energy=True)
    assert m.run(steps) == steps
    e = m.energy()
    got = np.array([e["internal_work"], e["external_work"], e["kinetic"]])
    ref = res["energy"][-1]
    assert abs(ref[1]) > 0
    np.testing.assert_allclose(got, ref, rtol=1e-7, atol=1e-10 * np.abs(ref).max())
    m.close()


@pytest.mark.gpu
def test_two_instances_follow_their_own_records():
    import femtech_gb300 as ft
    mesh, mats, loads, _ = _case(n=1_500)
    recs = [mg.pulse_records(seed=11), mg.pulse_records(seed=12, peak_ang=3.0e3)]
    single = []
    for rec in recs:
        m = _model(ft, mesh, mats, loads, rec, ft.FP64)
        assert m.run(80) == 80
        single.append(m.state()["u"])
        m.close()
    # the same mesh twice as two instances of one model
    nN = len(mesh["coordinates"])
    nE = len(mesh["eptr"]) - 1
    two = dict(coordinates=np.concatenate([mesh["coordinates"]] * 2),
               eptr=np.concatenate([mesh["eptr"][:-1], mesh["eptr"] + mesh["eptr"][-1]]),
               connectivity=np.concatenate([mesh["connectivity"], mesh["connectivity"] + nN]),
               etype=np.concatenate([mesh["etype"]] * 2),
               pid=np.concatenate([mesh["pid"]] * 2),
               fiber=np.concatenate([mesh["fiber"]] * 2))
    l2 = mg.Loads(2 * nN)
    l2.rigid(np.concatenate([mg.rigid_nodes(mesh, mats), mg.rigid_nodes(mesh, mats) + nN]))
    inst = dict(node_offset=np.array([0, nN, 2 * nN]), tmax=np.array([1.0, 1.0]),
                reduction=np.array([0.9, 0.9]))
    m = ft.Model(two, mats, precision=ft.FP64, loads=l2, instances=inst)
    for i, rec in enumerate(recs):
        m.set_rigid_body(rec, inst=i)
    m.init_explicit(0.9, 0.0, 1.0)
    m.run(80)
    u = m.state()["u"]
    assert nE > 0
    for i in range(2):
        np.testing.assert_allclose(u[3 * nN * i:3 * nN * (i + 1)], single[i], rtol=0,
                                   atol=1e-12 * np.abs(single[i]).max())
    y0, _ = m.rigid_body(0)
    y1, _ = m.rigid_body(1)
    assert not np.allclose(y0, y1)
    m.close()


@pytest.mark.gpu
def test_sampled_drive_matches_closed_form_rotation_drive():
    """The same half-sine rotation as FTGPU_BCK_ROT (closed form) and as
    sampled angular-acceleration records through the rigid-body integrator."""
    import femtech_gb300 as ft
    mesh, mats, loads, _ = _case(n=3_000)
    nodes = mg.rigid_nodes(mesh, mats)
    axis = np.array([0.2, 0.9, -0.4])
    axis /= np.linalg.norm(axis)
    a0, P = 6.0e3, 0.01
    ts = np.arange(0.0, 0.0200001, 1.0e-5)
    ang = a0 * np.where(ts <= P, np.sin(np.pi * ts / P), 0.0)
    rec = [(ts, ang * axis[k]) for k in range(3)] + [(ts, 0.0 * ts)] * 3
    lr = mg.Loads(len(mesh["coordinates"]))
    lr.rotation(nodes, axis, [0.0, 0.0, 0.0], a0, P)
    us = []
    for kind in ("rot", "rigid"):
        m = ft.Model(mesh, mats, precision=ft.FP64, loads=lr if kind == "rot" else loads)
        if kind == "rigid":
            m.set_rigid_body(rec)
        m.init_explicit(0.9, 0.0, 1.0)
        assert m.run(400) == 400
        us.append(m.state()["u"])
        m.close()
    # the drivers start the integrator from a zero derivative: the first step
    # lags by h b1 alpha(0) = 0, so only the sampling error remains
    assert _rel(us[1], us[0]) <= 1e-4, _rel(us[1], us[0])


@pytest.mark.gpu
def test_rigid_inputs_are_checked():
    import femtech_gb300 as ft
    mesh, mats, loads, rec = _case(n=1_000)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    with pytest.raises(RuntimeError):
        m.init_explicit(0.9, 0.0, 1.0)  # rigid DOFs without records
    bad = list(rec)
    bad[2] = (bad[2][0][::-1].copy(), bad[2][1])
    with pytest.raises(RuntimeError):
        m.set_rigid_body(bad)
    with pytest.raises(RuntimeError):
        m.set_rigid_body([(np.zeros(0), np.zeros(0))] * 6)
    m.set_rigid_body(rec)
    m.init_explicit(0.9, 0.0, 1.0)
    assert m.run(5) == 5
    m.close()
