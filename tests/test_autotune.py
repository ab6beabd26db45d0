"""Autotuner: bucket keys, cache round trip and candidate selection (CPU, with
an injected timer); on the GPU a real tuning run on a small batch."""
import numpy as np
import pytest

from femtech_gb300 import autotune as at
from femtech_gb300 import meshgen as mg


def test_bucket_and_selection(tmp_path, monkeypatch):
    monkeypatch.setenv("FTGPU_TUNING_CACHE", str(tmp_path / "t.json"))
    mesh, mats, loads = mg.cube_tension_case(n=4)
    k = at.bucket(mesh, mats, 1)
    assert k == "et0|mat1|p1|E2^6|I2^0"
    cost = {64: 3.0, 96: 2.0, 128: 1.5, 192: 1.7, 256: 2.5}
    calls = []

    def timer(p, t, s):
        calls.append((p, t, s))
        return cost[p] + {128: 0.3, 256: 0.0, 512: 0.1}[t] + {1: 0.05, 0: 0.0}[s]

    out = at.tune(mesh, mats, loads, timer=timer)
    assert out["patch"] == 128 and out["node_threads"] == 256 and out["split"] == 0
    assert at.load_cache()[k]["patch"] == 128
    # every candidate timed once: 5 patch sizes, 2 more nodal blocks, 1 more split
    assert len(calls) == len(set(calls)) == 8
    # FP64 mode never tries patches above 128 elements, nor the mixed-only split
    calls.clear()
    at.tune(mesh, mats, loads, precision=0, timer=timer, cache=False)
    assert max(p for p, _, _ in calls) == 128 and {s for _, _, s in calls} == {1}


@pytest.mark.gpu
def test_tuned_model_runs_and_matches_default(tmp_path, monkeypatch):
    import femtech_gb300 as ft
    monkeypatch.setenv("FTGPU_TUNING_CACHE", str(tmp_path / "t.json"))
    mesh, mats, loads, off = mg.ensemble_case(n_instances=4, e_min=500, e_max=3000, seed=3)
    inst = dict(node_offset=off, tmax=np.full(4, 1e300), reduction=np.full(4, 0.9))
    m = at.tuned_model(mesh, mats, loads, inst, precision=ft.MIXED, steps=5,
                       patch_candidates=(64, 128), node_candidates=(128, 256))
    assert m.tuning["patch"] in (64, 128) and m.tuning["split"] in (0, 1)
    assert len(m.tuning["ms"]) == 4
    m.init_explicit(0.9, 0.0, 1e300)
    m.run(50)
    u_t = m.state()["u"]
    d = ft.Model(mesh, mats, precision=ft.MIXED, loads=loads, instances=inst)
    d.init_explicit(0.9, 0.0, 1e300)
    d.run(50)
    u_d = d.state()["u"]
    assert np.linalg.norm(u_t - u_d) <= 1e-5 * np.linalg.norm(u_d)
