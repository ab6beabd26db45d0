"""The learned surrogate inside the explicit loop, where the network matters.

A 10x10x10 C3D8 block of the GOH + 1-term Prony law (material 7, the
head-like mesh's core: mu 1 kPa, k1 5 kPa, k2 10, kappa 0.1, lambda 2.19e8,
g1 0.6, tau1 6 ms, seeded random fibres), base fixed, top face pulled
sideways at 0.6 m/s.  The shear wave behind the top face carries the Green
strain to |E|_F^2 = 0.01-0.04 over most elements within 2000 steps, inside
the trust region (|E|_F^2 <= 0.04), where the network's correction to the
linearised law is not small.  Three mixed-precision runs are compared with
the FP64 oracle (plain law, HGOIsotropicViscoelastic.cpp:27-168 generalised
to the fibre term): the plain law, the trained surrogate, and the method
without the network (its output held at zero: the linearised law S_lin).
"""
import numpy as np
import pytest

import femtech_gb300 as ft
from femtech_gb300 import meshgen as mg
from helpers import rel, run_to

pytestmark = pytest.mark.gpu

PROPS7 = [1040.0, 1.0e3, 2.19e8, 5.0e3, 10.0, 0.6, 6.0e-3, 0.1]
STEPS, EVERY = 2000, 200


def strained_block():
    n, h = 10, 1e-3
    mesh = mg.hex_block(n, n, n, n * h, n * h, n * h, jitter=0.1, seed=31)
    E = len(mesh["etype"])
    rng = np.random.default_rng(32)
    a = rng.normal(size=(E, 3))
    mesh["fiber"] = a / np.linalg.norm(a, axis=1, keepdims=True)
    mats = mg.materials([(7, PROPS7)])
    X = mesh["coordinates"]
    loads = mg.Loads(len(X))
    loads.fix(np.where(np.abs(X[:, 2]) < 1e-9)[0])
    top = np.where(np.abs(X[:, 2] - n * h) < 1e-9)[0]
    loads.ramp(top, 0, 0.6)
    loads.fix(top, dofs=(1, 2))
    return mesh, mats, loads


@pytest.fixture(scope="module")
def reference(oracle_lib):
    mesh, mats, loads = strained_block()
    o = oracle_lib.Oracle(mesh, mats, threads=4)
    return o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=STEPS,
                          out_every=EVERY)


@pytest.fixture(scope="module")
def trained():
    from femtech_gb300.surrogate import Surrogate
    s = Surrogate(PROPS7, seed=5)
    s.generate(10_000_000, seed=11)
    s.train(epochs=4, batch=8192, lr=2e-3)
    yield s
    s.close()


def run(mesh, mats, loads, surrogate=None):
    m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
    if surrogate is not None:
        m.set_surrogate(surrogate, trust_e2=0.04)
    us, ts, steps, st = run_to(m, 1.0, 0.9, EVERY, max_steps=STEPS)
    e9 = m.element_strain()[0]
    m.close()
    assert steps == STEPS
    return us, e9


def test_surrogate_in_loop_at_finite_strain(reference, trained):
    from femtech_gb300.surrogate import Surrogate
    mesh, mats, loads = strained_block()
    ref = reference["u_out"]
    out = {}
    us, e9 = run(mesh, mats, loads)
    out["plain"] = us
    out["surrogate"] = run(mesh, mats, loads, trained)[0]
    zero = Surrogate(PROPS7, seed=5)
    zero.generate(4096, seed=11)  # the output scale; weights zeroed below
    zero.params = np.zeros_like(zero.params)
    out["linearised"] = run(mesh, mats, loads, zero)[0]
    zero.close()
    err = {k: max(rel(v[i], ref[i]) for i in range(len(ref))) for k, v in out.items()}
    # the regime: averaged Green strain per element, |E|_F^2
    e2 = (e9 ** 2).sum(axis=1)
    active = float(((e2 > 0.01) & (e2 <= 0.04)).mean())
    print("max rel. displacement error vs FP64 oracle: plain %.2e, surrogate %.2e, "
          "linearised %.2e; elements with 0.01 < |E|^2 <= 0.04: %.1f %%, above 0.04: %.1f %%"
          % (err["plain"], err["surrogate"], err["linearised"], 100 * active,
             100 * float((e2 > 0.04).mean())))
    assert active > 0.05  # the network carries a non-small part of the stress
    assert err["plain"] < 1e-3
    assert err["surrogate"] < 1e-3
    assert err["surrogate"] < err["linearised"]  # what the network gains in the loop
