"""GPU parity of the device-resident explicit loop (central difference,
boundary conditions, stable dt, CUDA-graph chunks) against the reference loop
(golden) and the FP64 oracle; determinism; batched instances.

Tolerances (relative nodal-displacement error, max over output steps):
FP64 mode 1e-5, mixed mode (FP32 element kernels, FP64 nodal state) 1e-3."""
import numpy as np
import pytest

import femtech_gb300 as ft
from femtech_gb300 import meshgen as mg
from helpers import MATS, ex9_mesh_loads, rel, run_to

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(ft.FP64, 1e-5), (ft.MIXED, 1e-3)])
def test_ex9_against_reference_loop_and_abaqus(golden, prec, tol):
    g = golden["ref_ex9"]
    mesh, mats, loads = ex9_mesh_loads()
    m = ft.Model(mesh, mats, precision=prec, loads=loads)
    us, ts, steps, st = run_to(m, 1.0, 0.8, 1)
    if prec == ft.FP64:
        assert steps == int(g["steps"])
    n = min(len(us), len(g["u_out"]))
    err = max(rel(us[i], g["u_out"][i]) for i in range(5, n))
    assert err < tol
    abq = g["abaqus_last"]
    u8 = st["u"][21:24]
    assert np.max(np.abs((u8 - abq[1:]) / abq[1:])) < 0.05  # compareResults.py:14-25


@pytest.mark.parametrize("prec,tol", [(ft.FP64, 1e-5), (ft.MIXED, 1e-3)])
def test_cube_tension_against_reference(golden, prec, tol):
    g = golden["ref_cube"]
    mesh, mats, loads = mg.cube_tension_case(n=10)
    m = ft.Model(mesh, mats, precision=prec, loads=loads)
    us, ts, steps, st = run_to(m, 0.01, 0.9, 100)
    assert abs(steps - int(g["steps"])) <= (0 if prec == ft.FP64 else 1)
    err = max(rel(us[i], g["u_out"][i]) for i in range(len(g["u_out"])))
    assert err < tol
    if prec == ft.FP64:
        np.testing.assert_allclose(ts, g["t_out"], rtol=1e-12)


def test_runs_are_bitwise_reproducible():
    mesh, mats, loads = mg.ogden_block_case(nx=12, ny=10, nz=8, lx=0.012, ly=0.01, lz=0.008)
    out = []
    for _ in range(2):
        m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
        m.init_explicit(0.9, 0.0, 1.0)
        m.run(200)
        out.append(m.state()["u"])
        m.close()
    assert np.array_equal(out[0], out[1])


# runs of 5 steps; and lengths that end in every tail graph (2 to 14 steps,
# odd lengths with one step past the limit) and in whole 16-step chunks
@pytest.mark.parametrize("lengths", [[5] * 20, [1, 2, 3, 14, 15, 17, 16, 32]])
def test_chunked_equals_continuous(lengths):
    assert sum(lengths) == 100
    mesh, mats, loads = mg.cube_tension_case(n=6)
    a = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    a.init_explicit(0.9, 0.0, 1.0)
    a.run(100)
    b = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    b.init_explicit(0.9, 0.0, 1.0)
    for k in lengths:
        assert b.run(k) == k
    sa, sb = a.state(), b.state()
    assert sa["step"] == sb["step"] == 100
    assert np.array_equal(sa["u"], sb["u"]) and np.array_equal(sa["v"], sb["v"])


def test_ogden_block_mixed_vs_oracle(oracle_lib):
    mesh, mats, loads = mg.ogden_block_case(nx=10, ny=10, nz=6, lx=0.01, ly=0.01, lz=0.006,
                                            amp=1e-4, freq=200.0)
    o = oracle_lib.Oracle(mesh, mats, threads=4)
    ref = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=300,
                         out_every=100)
    m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
    us, ts, steps, st = run_to(m, 1.0, 0.9, 100, max_steps=300)
    assert steps == 300
    err = max(rel(us[i], ref["u_out"][i]) for i in range(3))
    assert err < 1e-3


@pytest.mark.parametrize("prec,tol", [(ft.FP64, 1e-7), (ft.MIXED, 1e-3)])
def test_three_element_groups_side_by_side_vs_oracle(oracle_lib, prec, tol):
    """Three parts (Neo-Hookean, HGO, Ogden layers) make three element groups,
    whose passes run on alternating streams of the step graph: the loop still
    matches the oracle and repeats bitwise."""
    mesh, mats, loads = mg.ogden_block_case(nx=8, ny=8, nz=6, lx=0.008, ly=0.008, lz=0.006,
                                            amp=1e-4, freq=200.0)
    X = mesh["coordinates"]
    conn = np.asarray(mesh["connectivity"]).reshape(-1, 8)
    zc = X[conn, 2].mean(axis=1)
    mesh["pid"] = np.digitize(zc, [0.002, 0.004]).astype(np.int32)
    mats = mg.materials([(1, MATS[1]), (4, MATS[4]), (6, MATS[6])])
    o = oracle_lib.Oracle(mesh, mats, threads=4)
    ref = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=200,
                         out_every=100)
    out = []
    for _ in range(2):
        m = ft.Model(mesh, mats, precision=prec, loads=loads)
        us, ts, steps, st = run_to(m, 1.0, 0.9, 100, max_steps=200)
        assert steps == 200
        assert max(rel(us[i], ref["u_out"][i]) for i in range(2)) < tol
        out.append(us[-1])
        m.close()
    assert np.array_equal(out[0], out[1])


def test_batched_instances_equal_separate_runs():
    cases = [mg.cube_tension_case(n=n, mu=mu) for n, mu in ((4, 3400.0), (5, 5000.0), (3, 2000.0))]
    Xs, conns, eptrs, pids, fns, dofs = [], [], [], [], [], []
    noff, eoff, parts = [0], 0, []
    for i, (mesh, mats, loads) in enumerate(cases):
        Xs.append(mesh["coordinates"])
        conns.append(mesh["connectivity"] + noff[-1])
        pids.append(np.full(len(mesh["etype"]), i, np.int32))
        parts.append((1, list(mats["properties"][:3])))
        d = loads.dof_fn.copy()
        d[d >= 0] += len(fns)
        dofs.append(d)
        fns += loads.fns
        noff.append(noff[-1] + len(mesh["coordinates"]))
    E = sum(len(c) // 8 for c in conns)
    big = dict(coordinates=np.concatenate(Xs), connectivity=np.concatenate(conns).astype(np.int32),
               eptr=np.arange(0, 8 * E + 1, 8, dtype=np.int32), etype=np.zeros(E, np.int32),
               pid=np.concatenate(pids))
    bl = mg.Loads(noff[-1])
    bl.dof_fn = np.concatenate(dofs)
    bl.fns = fns
    inst = dict(node_offset=np.array(noff, np.int32), tmax=np.array([1e-3, 2e-3, 1.5e-3]),
                reduction=np.array([0.9, 0.8, 0.9]))
    mb = ft.Model(big, mg.materials(parts), precision=ft.FP64, loads=bl, instances=inst)
    mb.init_explicit()
    mb.run(10**6)
    ub = mb.state()["u"]
    clk = mb.instance_clocks()
    for i, (mesh, mats, loads) in enumerate(cases):
        m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
        m.init_explicit(inst["reduction"][i], 0.0, inst["tmax"][i])
        m.run(10**6)
        s = m.state()
        # same dt sequence (exact minima); patch order may differ -> rounding only
        assert clk["step"][i] == s["step"] and clk["time"][i] == s["time"]
        assert rel(ub[3 * noff[i]:3 * noff[i + 1]], s["u"]) < 1e-12


def test_rotation_bc_against_oracle(oracle_lib):
    """Surface nodes driven by the half-sine rigid rotation; interior free."""
    mesh = mg.tet_ellipsoid(0.01, 0.008, 0.007, 0.002, seed=1)
    X = mesh["coordinates"]
    r = np.sqrt((X[:, 0] / 0.01) ** 2 + (X[:, 1] / 0.008) ** 2 + (X[:, 2] / 0.007) ** 2)
    surf = np.where(r > 0.8)[0]
    mats = mg.materials([(1, [1000.0, 3.4e3, 2.0e5])])
    loads = mg.Loads(len(X))
    loads.rotation(surf, [0.2, 0.5, 1.0], [0.0, 0.0, 0.0], 6e3, 0.01)
    o = oracle_lib.Oracle(mesh, mats)
    ref = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=200,
                         out_every=50)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    us, ts, steps, st = run_to(m, 1.0, 0.9, 50, max_steps=200)
    assert steps == 200
    assert max(rel(us[i], ref["u_out"][i]) for i in range(4)) < 1e-8
    np.testing.assert_allclose(ts, ref["t_out"], rtol=1e-13)


def test_errors_are_status_codes():
    mesh, mats, loads = mg.cube_tension_case(n=3)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    with pytest.raises(ft.FtgpuError) as ei:
        m.init_explicit(0.9, 1.0, 1.0)  # FailureTimeStep larger than any dt
    assert ei.value.status == ft.ERR_DT
    # inverted element: push one interior node through its neighbour
    u = np.zeros(3 * len(mesh["coordinates"]))
    u[3 * 21 + 2] = -0.02
    with pytest.raises(ft.FtgpuError) as ei:
        m.GetForce(u)
    assert ei.value.status == ft.ERR_INVERTED
    bad = mg.materials([(9, [1.0, 1.0, 1.0])])
    with pytest.raises(ft.FtgpuError) as ei:
        ft.Model(mesh, bad)
    assert ei.value.status == ft.ERR_MATERIAL


def test_state_transfer_pinned_and_pageable_agree():
    """set_state / get_state move the reference-layout arrays exactly, whether
    the host arrays are page-locked (read and written in place by the
    transpose kernels) or pageable (staged copies)."""
    import torch
    mesh, mats, loads = mg.cube_tension_case(n=5)
    m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
    n = 3 * len(mesh["coordinates"])
    rng = np.random.default_rng(3)
    u, v, a = (rng.normal(size=n) for _ in range(3))
    pin = {k: torch.tensor(x).pin_memory().numpy() for k, x in zip("uva", (u, v, a))}
    out = {k: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for k in "uva"}
    for src in (pin, dict(u=u, v=v, a=a)):
        m.set_state(src["u"], src["v"], src["a"], 0.0)
        s1 = m.state()  # pageable destination
        s2 = m.state(out=out)  # page-locked destination
        for k, x in zip("uva", (u, v, a)):
            assert np.array_equal(s1[k], x) and np.array_equal(s2[k], x), k
    m.close()
