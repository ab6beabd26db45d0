"""Per-step injury criteria (ex5's CalculateInjuryCriterions) in the device loop
against the oracle's restatement (whose parts, the element strain and the 95th
percentile, are pinned bitwise to the reference: tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from femtech_gb300 import meshgen as mg

SCALARS = ("max_strain", "max_strain_time", "min_strain", "min_strain_time", "max_shear",
           "max_shear_time", "max_psxsr", "max_psxsr_time", "mps95", "mps95_time", "mpsxsr95",
           "mpsxsr95_time")
ELEMS = ("max_strain_elem", "min_strain_elem", "max_shear_elem", "max_psxsr_elem",
         "mps95_count", "mpsxsr95_count")
BITS = (("mps15", 1), ("mps30", 2), ("psr120", 4), ("psxsr28", 8), ("in_mps95", 16),
        ("in_mpsxsr95", 32))


def _case():
    """The cube tension case on a jittered lattice: without jitter, mirror-image
    elements tie exactly and the element named for an extreme would be decided
    by the last bit of rounding."""
    mesh, mats, loads = mg.cube_tension_case(n=6)
    jm = mg.hex_block(6, 6, 6, 0.01, 0.01, 0.01, jitter=0.1, seed=7)
    mesh = dict(mesh, coordinates=jm["coordinates"])
    return mesh, mats, loads


def _run_gpu(ft, precision, ids, steps, chunks=None):
    mesh, mats, loads = _case()
    m = ft.Model(mesh, mats, precision=precision, loads=loads)
    m.set_injury(ids)
    m.init_explicit(0.9, 0.0, 0.01)
    for c in (chunks or (steps,)):
        m.run(c)
    out = m.injury()
    m.close()
    return out


def _run_oracle(orc, ids, steps):
    mesh, mats, loads = _case()
    o = orc.Oracle(mesh, mats)
    res = o.explicit_run(loads.dof_fn, loads.fns, 0.01, 0.9, steps, steps, injury_ids=ids)
    return res["injury"]


@pytest.mark.gpu
@pytest.mark.parametrize("subset", [False, True])
def test_fp64_injury_criteria_match_oracle(oracle_lib, subset):
    import femtech_gb300 as ft
    nE = len(mg.cube_tension_case(n=6)[0]["etype"])
    ids = np.arange(nE)[::-1][::2].copy() if subset else np.arange(nE)
    g = _run_gpu(ft, ft.FP64, ids, 300)
    r = _run_oracle(oracle_lib, ids, 300)
    assert g["steps"] == 300
    assert r["max_strain"] > 0.1  # the run strains the cube into the criteria's range
    for k in SCALARS:
        assert g[k] == pytest.approx(r[k], rel=1e-9, abs=1e-15), k
    for k in ELEMS:
        assert g[k] == r[k], k
    for k, b in BITS:
        np.testing.assert_array_equal((g["flags"] & b) != 0, r[k] != 0, err_msg=k)
    np.testing.assert_allclose(g["ps"], r["ps_old"], rtol=1e-9, atol=1e-15)


@pytest.mark.gpu
def test_mixed_injury_criteria_within_fp32(oracle_lib):
    import femtech_gb300 as ft
    nE = len(mg.cube_tension_case(n=6)[0]["etype"])
    ids = np.arange(nE)
    g = _run_gpu(ft, ft.MIXED, ids, 300)
    r = _run_oracle(oracle_lib, ids, 300)
    for k in ("max_strain", "min_strain", "max_shear", "mps95"):
        assert g[k] == pytest.approx(r[k], rel=1e-3), k
    assert np.abs(g["ps"] - r["ps_old"]).max() <= 1e-3 * np.abs(r["ps_old"]).max()
    assert np.mean(((g["flags"] & 1) != 0) != (r["mps15"] != 0)) <= 0.02


@pytest.mark.gpu
def test_injury_chunked_equals_continuous():
    import femtech_gb300 as ft
    nE = len(mg.cube_tension_case(n=6)[0]["etype"])
    ids = np.arange(nE)
    a = _run_gpu(ft, ft.FP64, ids, 250)
    b = _run_gpu(ft, ft.FP64, ids, 250, chunks=(90, 70, 90))
    for k in SCALARS + ELEMS:
        assert a[k] == b[k], k
    np.testing.assert_array_equal(a["flags"], b["flags"])
