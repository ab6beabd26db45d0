"""Energy balance of the device loop against the reference's CheckEnergy.

tests/golden/ref_cube.npz holds, per step of the CPU-runnable cube run, the
cumulative internal and external work and the kinetic energy that the
reference's own CheckEnergy (src/fem/SolidMechanics/CheckEnergy.cpp) logged;
the oracle reproduces them bitwise (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from femtech_gb300 import meshgen as mg


def _cube(ft, precision):
    mesh, mats, loads = mg.cube_tension_case(n=10)
    m = ft.Model(mesh, mats, precision=precision, loads=loads)
    m.set_energy(True)
    m.init_explicit(0.9, 0.0, 0.01)
    return m


def _e(m):
    e = m.energy()
    return np.array([e["internal_work"], e["external_work"], e["kinetic"]]), e


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [37, 100, 516])
def test_fp64_energy_matches_reference_checkenergy(golden, steps):
    import femtech_gb300 as ft
    g = golden["ref_cube"]["energy"]
    m = _cube(ft, ft.FP64)
    assert m.run(steps) == steps
    got, e = _e(m)
    ref = g[steps - 1]
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())
    m.close()


@pytest.mark.gpu
def test_fp64_energy_whole_run_and_violation_count(golden):
    import femtech_gb300 as ft
    g = golden["ref_cube"]["energy"]
    m = _cube(ft, ft.FP64)
    n = m.run(100000)
    assert n == len(g)
    got, e = _e(m)
    np.testing.assert_allclose(got, g[-1], rtol=1e-9)
    # the reference's own balance check, step by step from the golden history
    tot = np.abs(g[:, 2] + g[:, 0] - g[:, 1])
    mx = np.maximum(np.abs(g).max(axis=1), 1e-300)
    assert e["violations"] == int(np.sum(tot > 0.01 * np.abs(g).max(axis=1)))
    assert abs(e["max_violation"] - (tot / mx).max()) <= 1e-9
    m.close()


@pytest.mark.gpu
def test_mixed_energy_within_mixed_tolerance(golden):
    import femtech_gb300 as ft
    g = golden["ref_cube"]["energy"]
    m = _cube(ft, ft.MIXED)
    n = m.run(100000)
    assert abs(n - len(g)) <= 1
    got, _ = _e(m)
    ref = g[min(n, len(g)) - 1]
    assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max()
    m.close()


@pytest.mark.gpu
def test_energy_chunked_equals_continuous():
    import femtech_gb300 as ft
    outs = []
    for chunks in ((200,), (60, 60, 80)):
        m = _cube(ft, ft.FP64)
        for c in chunks:
            m.run(c)
        outs.append(_e(m)[0])
        m.close()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.gpu
def test_energy_off_leaves_the_loop_unchanged():
    import femtech_gb300 as ft
    us = []
    for on in (False, True):
        mesh, mats, loads = mg.cube_tension_case(n=6)
        m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads)
        m.set_energy(on)
        m.init_explicit(0.9, 0.0, 0.01)
        m.run(150)
        us.append(m.state()["u"])
        m.close()
    assert np.array_equal(us[0], us[1])


@pytest.mark.gpu
def test_head_rotation_energy_matches_oracle(oracle_lib):
    """Rigid-rotation drive, shell + GOH/Prony core: FP64 device loop against
    the oracle's CheckEnergy restatement."""
    import femtech_gb300 as ft
    mesh, mats, loads = mg.head_case(target_elements=6_000, seed=3)
    o = oracle_lib.Oracle(mesh, mats, threads=8)
    res = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=60,
                         out_every=60, energy=True)
    m = ft.Model(mesh, mats, precision=ft.FP64, loads=loads)
    m.set_energy(True)
    m.init_explicit(0.9, 0.0, 1.0)
    assert m.run(60) == 60
    got, _ = _e(m)
    ref = res["energy"][-1]
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-12 * np.abs(ref).max())
    m.close()
