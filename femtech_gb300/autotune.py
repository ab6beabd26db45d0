"""Autotuner for the engine's launch shapes.

Three choices decide how a mesh maps onto the GPU and are tuned per *shape
bucket* (element types, materials, precision, element count rounded to a power
of two, instance count rounded likewise):

* elements per patch = threads per block of the element kernel (64..256):
  larger patches replicate fewer nodes (less slot traffic) but occupy more
  shared memory and registers per block;
* threads per block of the nodal kernels (128 / 256 / 512);
* the nodal pass split (mixed precision): a lean kernel over the free and
  function-driven nodes plus the general kernel over the rest, or the general
  kernel over every node (meshes where most nodes carry rigid-rotation or
  rigid-body drives gain nothing from the split).

`tune()` times the candidates on the actual model for a few steps (device
time with CUDA events, after warm-up) -- the patch size first, then the nodal
block size, then the split -- keeps the fastest and stores it in a JSON cache
(``$FTGPU_TUNING_CACHE``, default ``~/.cache/femtech_gb300/tuning.json``).
`tuned_model()` builds a Model with the cached choice, tuning first on a miss.
"""
import ctypes as C
import json
import math
import os

import numpy as np

PATCH_CANDIDATES = (64, 96, 128, 192, 256)
NODE_CANDIDATES = (128, 256, 512)
SPLIT_CANDIDATES = (1, 0)


def cache_path():
    return os.environ.get("FTGPU_TUNING_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "femtech_gb300",
                                       "tuning.json"))


def bucket(mesh, mats, precision, instances=None):
    """Cache key: element types, material IDs, precision, log2 sizes."""
    et = sorted(set(int(x) for x in np.unique(mesh["etype"])))
    mids = sorted(set(int(x) for x in np.unique(np.asarray(mats["materialID"]))))
    E = len(mesh["etype"])
    ni = 1 if instances is None else len(instances["node_offset"]) - 1
    return "et%s|mat%s|p%d|E2^%d|I2^%d" % ("".join(map(str, et)), "".join(map(str, mids)),
                                          int(precision), round(math.log2(max(E, 1))),
                                          round(math.log2(max(ni, 1))))


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply_choice(m, node_threads, split):
    """Set the nodal knobs of a Model (before or after setup)."""
    import femtech_gb300 as ft
    L = ft.lib()
    L.ftgpu_set_node_split.argtypes = [C.c_void_p, C.c_int]
    ft._check(L.ftgpu_set_node_threads(m.h, int(node_threads)))
    ft._check(L.ftgpu_set_node_split(m.h, int(split)))


def time_config(mesh, mats, loads, instances, precision, patch, node_threads, split=1,
                steps=20, warmup=5, device=0):
    """Device milliseconds per step of one configuration."""
    import femtech_gb300 as ft
    m = ft.Model(mesh, mats, precision=precision, device=device, loads=loads,
                 patch_size=patch, instances=instances, setup=False)
    apply_choice(m, node_threads, split)
    m.setup()
    m.init_explicit(0.9, 0.0, 1e300)
    m.run(warmup)
    sd, ms = C.c_int(), C.c_double()
    ft._check(ft.lib().ftgpu_run_timed(m.h, int(steps), C.byref(sd), C.byref(ms)))
    m.close()
    return ms.value / max(sd.value, 1)


def tune(mesh, mats, loads=None, instances=None, precision=1, steps=20, device=0,
         patch_candidates=PATCH_CANDIDATES, node_candidates=NODE_CANDIDATES,
         split_candidates=SPLIT_CANDIDATES, timer=None, cache=True):
    """Time the candidates, return {'patch': p, 'node_threads': t, 'split': s,
    'ms': {config: ms per step}} (timer(p, t, s) -> ms, injectable for tests)."""
    timer = timer or (lambda p, t, s: time_config(mesh, mats, loads, instances, precision, p,
                                                  t, s, steps=steps, device=device))
    pcs = [p for p in patch_candidates if not (precision == 0 and p > 128)]
    scs = [s for s in split_candidates if not (precision == 0 and s == 0)] or [1]
    res = {}

    def run(p, t, s):
        k = "p%d_t%d_s%d" % (p, t, s)
        if k not in res:
            res[k] = timer(p, t, s)
        return res[k]

    s0 = scs[0]
    for p in pcs:  # patch size first, at the default nodal block
        run(p, 128, s0)
    best_p = min(pcs, key=lambda p: run(p, 128, s0))
    best_t = min(node_candidates, key=lambda t: run(best_p, t, s0))
    best_s = min(scs, key=lambda s: run(best_p, best_t, s))
    out = {"patch": best_p, "node_threads": best_t, "split": best_s, "ms": res}
    if cache:
        c = load_cache()
        c[bucket(mesh, mats, precision, instances)] = out
        save_cache(c)
    return out


def tuned_model(mesh, mats, loads=None, instances=None, precision=1, device=0, retune=False,
                **kw):
    """A Model built with the cached launch shapes of its bucket (tuning on a miss)."""
    import femtech_gb300 as ft
    key = bucket(mesh, mats, precision, instances)
    c = load_cache()
    choice = None if retune else c.get(key)
    if choice is None:
        choice = tune(mesh, mats, loads, instances, precision, device=device, **kw)
    m = ft.Model(mesh, mats, precision=precision, device=device, loads=loads,
                 patch_size=choice["patch"], instances=instances, setup=False)
    apply_choice(m, choice["node_threads"], choice.get("split", 1))
    m.setup()
    m.tuning = choice
    return m
