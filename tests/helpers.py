"""Shared builders for the parity tests (same meshes as tests/golden/make_golden.py)."""
import numpy as np

from femtech_gb300 import meshgen as mg

MATS = {
    1: [1000.0, 3400.0, 2.0e6],
    2: [1000.0, 3400.0, 2.0e6],
    3: [1000.0, 3400.0, 2.0e6],
    4: [1040.0, 1.0e3, 2.0e6, 5.0e3, 10.0],
    5: [1040.0, 1.0e3, 2.0e6, 5.0e3, 10.0, 0.6, 6.0e-3, 0.2, 2.0e-3],
    6: [1040.0, 1.5e3, 2.0e7 - 1.0e3, 5.0],
    7: [1040.0, 1.0e3, 2.19e8, 5.0e3, 10.0, 0.6, 6.0e-3, 0.1],
}


def golden_mesh(golden, name):
    f = golden["ref_force"]
    X = f[name + "_X"]
    conn = f[name + "_conn"]
    et = f[name + "_etype"]
    nc = 8 if et[0] == 0 else 4
    E = len(et)
    return dict(coordinates=X, eptr=np.arange(0, nc * E + 1, nc, dtype=np.int32),
                connectivity=conn.astype(np.int32), etype=et.astype(np.int32),
                pid=np.zeros(E, np.int32))


def ex9_mesh_loads():
    X = np.array([[0, 0, 0], [0.005, 0, 0], [0, 0.005, 0], [0.005, 0.005, 0],
                  [0, 0, 0.005], [0.005, 0, 0.005], [0, 0.005, 0.005], [0.005, 0.005, 0.005]],
                 np.float64)
    conn = np.array([0, 1, 3, 2, 4, 5, 7, 6], np.int32)
    mesh = dict(coordinates=X, eptr=np.array([0, 8], np.int32), connectivity=conn,
                etype=np.array([0], np.int32), pid=np.array([0], np.int32))
    mats = mg.materials([(1, [1040.0, 100.0, 100.0])])
    tol = 1e-5
    loads = mg.Loads(8)
    loads.fix(np.where(np.abs(X[:, 0]) < tol)[0], dofs=(0,))
    loads.fix(np.where(np.abs(X[:, 1]) < tol)[0], dofs=(1,))
    loads.fix(np.where(np.abs(X[:, 2]) < tol)[0], dofs=(2,))
    loads.ramp(np.where(np.abs(X[:, 1] - 0.005) < tol)[0], 1, 0.007)
    return mesh, mats, loads


def random_fibers(E, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(E, 3))
    return a / np.linalg.norm(a, axis=1, keepdims=True)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_to(m, tmax, reduction, out_every, max_steps=10**7):
    """Run a model's device loop, pausing every out_every steps to record u;
    returns (u at each full pause, their times, steps run, final state)."""
    m.init_explicit(reduction=reduction, failure_dt=0.0, tmax=tmax)
    us, ts = [], []
    total = 0
    while total < max_steps:
        k = m.run(min(out_every, max_steps - total))
        total += k
        s = m.state()
        if k == out_every:
            us.append(s["u"])
            ts.append(s["time"])
        if k < out_every:
            break
    return np.array(us), np.array(ts), total, m.state()
