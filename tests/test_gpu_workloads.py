"""GPU parity of the benchmark workload families at small sizes against the
FP64 oracle: the head-like C3D4 ellipsoid (Neo-Hookean shell, anisotropic GOH
+ Prony core with a fibre field, rigid-rotation drive) and the batched Ogden
ensemble.  Mixed precision, tolerance 1e-3 relative nodal displacement."""
import numpy as np
import pytest

import femtech_gb300 as ft
from femtech_gb300 import meshgen as mg
from helpers import rel

pytestmark = pytest.mark.gpu


_HEAD = {}


def _head_small(oracle_lib):
    """The small head case and its FP64 oracle run (computed once per module)."""
    if not _HEAD:
        mesh, mats, loads = mg.head_case(target_elements=12_000, seed=4)
        o = oracle_lib.Oracle(mesh, mats, threads=4)
        ref = o.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=300,
                             out_every=100)
        _HEAD.update(mesh=mesh, mats=mats, loads=loads, ref=ref)
    return _HEAD["mesh"], _HEAD["mats"], _HEAD["loads"], _HEAD["ref"]


# patch size 0 (default 128): most nodes in one to eight patches (eight-slot
# node records); 32: many nodes in more than eight (the CSR path of the
# node step)
@pytest.mark.parametrize("patch", [0, 32])
def test_head_case_small_vs_oracle(oracle_lib, patch):
    mesh, mats, loads, ref = _head_small(oracle_lib)
    m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads, patch_size=patch)
    m.init_explicit(0.9, 0.0, 1.0)
    us = []
    for _ in range(3):
        assert m.run(100) == 100
        us.append(m.state()["u"])
    err = max(rel(us[i], ref["u_out"][i]) for i in range(3))
    assert err < 1e-3
    assert np.abs(ref["u_out"][-1]).max() > 0  # the drive actually moved the body


def test_ensemble_small_vs_separate_oracle_runs(oracle_lib):
    mesh, mats, loads, off = mg.ensemble_case(n_instances=3, e_min=300, e_max=1500, seed=7)
    inst = dict(node_offset=off, tmax=np.full(3, 1e300), reduction=np.full(3, 0.9))
    m = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads, instances=inst)
    m.init_explicit()
    assert m.run(150) == 150
    u = m.state()["u"]
    clk = m.instance_clocks()
    eptr = mesh["eptr"]
    conn = mesh["connectivity"].reshape(-1, 8)
    for i in range(3):
        n0, n1 = off[i], off[i + 1]
        sel = np.where((conn[:, 0] >= n0) & (conn[:, 0] < n1))[0]
        sub = dict(coordinates=mesh["coordinates"][n0:n1], connectivity=(conn[sel] - n0).ravel(),
                   eptr=np.arange(0, 8 * len(sel) + 1, 8, dtype=np.int32),
                   etype=np.zeros(len(sel), np.int32), pid=np.zeros(len(sel), np.int32))
        smats = mg.materials([(6, mats["properties"].reshape(-1, 9)[i][:4])])
        dof = loads.dof_fn[3 * n0:3 * n1]
        used = sorted(set(int(x) for x in dof if x >= 0))
        remap = {f: k for k, f in enumerate(used)}
        sdof = np.array([remap[x] if x >= 0 else x for x in dof], np.int32)
        sfns = [loads.fns[f] for f in used]
        o = oracle_lib.Oracle(sub, smats, threads=2)
        ref = o.explicit_run(sdof, sfns, tmax=1e300, reduction=0.9, max_steps=150, out_every=150)
        assert ref["steps"] == 150 and clk["step"][i] >= 150
        assert rel(u[3 * n0:3 * n1], ref["u"]) < 1e-3
        assert clk["time"][i] == pytest.approx(ref["time"], rel=1e-5)
    del eptr
