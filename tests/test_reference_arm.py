"""The CPU reference arm of bench.py (`--impl reference`): where the reference
compiles here, its own explicit loop (with the oracle's Ogden law plugged into
its material switch) must agree with the FP64 oracle port that stands in for it
elsewhere, and the arm's bounded rate sample must run."""
import os
import sys

import numpy as np
import pytest

from femtech_gb300 import meshgen as mg
from helpers import rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_build_loop_matches_port(oracle_lib):
    if not oracle_lib.RefBuild.available():
        pytest.skip("reference build not present")
    mesh, mats, loads = mg.ogden_block_case(nx=6, ny=5, nz=4, lx=0.006, ly=0.005, lz=0.004,
                                            jitter=0.1, seed=0)
    kw = dict(tmax=1.0, reduction=0.9, max_steps=30, out_every=0)
    a = oracle_lib.RefBuild(mesh, mats).explicit_run(loads.dof_fn, loads.fns, **kw)
    b = oracle_lib.Oracle(mesh, mats).explicit_run(loads.dof_fn, loads.fns, **kw)
    assert a["steps"] == b["steps"] == 30
    assert np.abs(b["u"]).max() > 0
    assert rel(a["u"], b["u"]) < 1e-9
    assert a["time"] == pytest.approx(b["time"], rel=1e-12)


@pytest.mark.parametrize("kind", ["port", "reference"])
def test_reference_arm_rate_sample(kind):
    sys.path.insert(0, ROOT)
    import bench
    r = bench.cpu_reference_rate(threads=2, target_s=0.2, kind=kind)
    assert r["value"] > 0 and r["unit"] == "element-updates/s"
    assert r["kind"] in ("port", "reference")
    assert "sub-block" in r["sample"]
