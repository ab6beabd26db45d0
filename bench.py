#!/usr/bin/env python
"""Element-updates/s of FemTech's explicit hot path on GB300.

Default workload (the headline configuration that fits one GPU): the
200x200x100 C3D8 block (4,000,000 elements, 4,080,501 nodes, 0.2x0.2x0.1 m),
nodes jittered +-10 % of the edge length (seeded; faces kept planar), 1-term
Ogden (mu 1.5 kPa, alpha 5, K 20 MPa, rho 1040), base fixed, top face
sinusoidal shear 1 mm at 50 Hz, dt = 0.9 x stable dt; FP32 element kernels,
FP64 nodal state and dt.  One step = one central-difference step of every
element (force, stress, stable dt, assembly, nodal update), i.e. one
element-update per element.  Inputs are synthetic (seeded), generated in the
run.

Reported (one JSON line from rank 0):
  value       element-updates/s, device time of the timed steps (CUDA events
              on the engine's stream, device synchronised on both sides)
  e2e         the same metric through the public C ABI with host buffers:
              initial state uploaded from host, displacements read back every
              100 steps, setup of the loop included
  roofline    dominant kernel (element pass): the algorithmic bytes of one
              element-update (32 B per element + 116 B per node) over its
              time against the measured HBM bandwidth, its FP32 rate against
              the measured FMA rate of this GPU, and which of the two roofs
              binds
  rel_disp_err_vs_fp64  mixed path against the FP64 path over the
              configuration's 5000 steps on a 40x40x20 sub-block
  cpu_baseline the FP64 oracle (OpenMP port of the reference algorithm) on
              the host cores, on a bounded sub-block of the same workload

--impl reference times the reference algorithm on the host CPU (the oracle
port on all host threads; the reference's own sources where they were
compiled in this checkout) on the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# Workload
NX, NY, NZ = 200, 200, 100
LX, LY, LZ = 0.2, 0.2, 0.1
WORKLOAD = "ogden_hex8_block_200x200x100_jitter10_sine50Hz"

# Algorithmic (compulsory) bytes of one element-update at the stated
# precisions, whole step: per element the connectivity 8 x 4 B; per node
# (x nodes / elements) X f32 12 B + u f64 24 B + v_half f64 24 B + mass f64
# 8 B read and u, v_half (48 B) written = 116 B.  For the 4M block:
# 32 + 116 x 4,080,501 / 4,000,000 = 150.3 B.  Everything else the kernels
# move is overhead of this design, not algorithmic: the Gauss-point geometry
# table of the FP32 C3D8 kernels (320 B per element), the patch-local slot
# replicas of u and of the partial forces, the f32 force hand-off between the
# passes.  The measured DRAM bytes of the element pass (profiles/) carry it.
ALG_BYTES_PER_EL_C3D8 = 32.0
ALG_BYTES_PER_NODE = 116.0
# design overheads per element of the FP32 C3D8 path (for the line's notes)
GEO_TABLE_BYTES_PER_EL = 320.0
# nodal pass alone: u, v_half, mass f64 read, u, v_half written, force f32 read
NODE_BYTES_PER_NODE = 116.0
# FP32 operations of one C3D8 Ogden element-update in this formulation
# (small-strain series path), counted from the kernel source (ft_elem.cuh /
# ft_materials.cuh), FMA = 2: per Gauss point displacement-gradient columns
# 54, D = H A^-T 45, J - 1 27, Ogden series law 291 (2E 40, norm 11, M^2 30,
# invariants 21, eight Cayley-Hamilton steps of the I / M / M^2 coefficients
# of the A series 88, tr B from A 16, exact (I + M)^-1 7, coefficients of S
# 15, J^-alpha/3 5, S 21, volumetric 37), det A S 6, P = S + D S 54, P A^-1
# 45, moments 63 -> 585 per Gauss point, 4680 for 8; Hadamard transform of u
# 75, face areas 540, inverse transform 90.  (A^-1 and det A of the reference
# geometry are read from the set-up table, not recomputed.)  ncu counts
# 1858 FFMA + 795 FADD + 844 FMUL = 5355 per element on this path.
FLOP_PER_EL_OGDEN = 4680 + 75 + 540 + 90


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max_sum(vals, world, backend_device=None):
    """Max of times and sum of work over ranks (torch.distributed when world > 1)."""
    if world == 1:
        return vals
    import torch
    import torch.distributed as dist
    t = torch.tensor(vals, dtype=torch.float64, device=backend_device or "cpu")
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    return mx.tolist()


def build_workload(nx=NX, ny=NY, nz=NZ, lx=LX, ly=LY, lz=LZ):
    from femtech_gb300 import meshgen as mg
    return mg.ogden_block_case(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, jitter=0.1, seed=0)


def host_cpu():
    """The host CPU's model name (lscpu), else the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


def cpu_reference_rate(threads, target_s=12.0, kind="port"):
    """Element-updates/s of the FP64 reference algorithm on host cores, on a
    bounded sub-block (40x40x20 of the same spacing, jitter, law and loads)."""
    from oracle import oracle as orc
    sub = (40, 40, 20)
    mesh, mats, loads = build_workload(sub[0], sub[1], sub[2], LX * sub[0] / NX, LY * sub[1] / NY,
                                       LZ * sub[2] / NZ)
    E = len(mesh["etype"])
    if kind == "reference" and orc.RefBuild.available():
        runner = orc.RefBuild(mesh, mats)
        threads = 1
    else:
        kind = "port"
        runner = orc.Oracle(mesh, mats, threads=threads)
    t = time.perf_counter()
    runner.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=2, out_every=0)
    per = (time.perf_counter() - t) / 3.0
    steps = max(2, int(target_s / max(per, 1e-6)))
    t = time.perf_counter()
    res = runner.explicit_run(loads.dof_fn, loads.fns, tmax=1.0, reduction=0.9, max_steps=steps,
                              out_every=0)
    dt = time.perf_counter() - t
    rate = E * res["steps"] / dt
    return dict(value=rate, unit="element-updates/s", cores=threads, kind=kind, cpu=host_cpu(),
                sample="%dx%dx%d sub-block (%d C3D8, same spacing/jitter/law/loads), FP64, %d steps "
                       "incl. initial force and dt, %.1f s" % (sub + (E, res["steps"], dt)))


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle as orc
    if not os.path.exists(orc.LIB):
        orc.build()
    kind = "reference" if orc.RefBuild.available() else "port"
    # bounded samples (each a few seconds of every host thread): up to two
    # short warm-up samples, then up to three timed ones; value = their mean
    warm = min(max(args.warmup, 0), 2)
    rates = []
    for i in range(warm + max(1, min(args.steps, 3))):
        r = cpu_reference_rate(threads, target_s=8.0 if i >= warm else 2.0, kind=kind)
        if i >= warm:
            rates.append(r)
    v = float(np.mean([r["value"] for r in rates]))
    base = rates[-1]
    base["value"] = v
    line = {"metric": "element-updates/s", "value": v, "unit": "element-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "impl": "reference", "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample": base["sample"]},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "element-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def make_workload(name, size=None):
    """Mesh, materials, loads, instances and the traffic / flop model of one
    benchmark configuration."""
    from femtech_gb300 import meshgen as mg
    if name == "block":
        nx, ny, nz = NX, NY, NZ
        if size:
            nx, ny, nz = (int(x) for x in size.split(","))
        mesh, mats, loads = build_workload(nx, ny, nz, LX * nx / NX, LY * ny / NY, LZ * nz / NZ)
        E, N = len(mesh["etype"]), len(mesh["coordinates"])
        return dict(mesh=mesh, mats=mats, loads=loads, instances=None,
                    label=WORKLOAD if not size else "ogden_hex8_block_%dx%dx%d" % (nx, ny, nz),
                    alg_bytes=E * ALG_BYTES_PER_EL_C3D8 + N * ALG_BYTES_PER_NODE,
                    flop=FLOP_PER_EL_OGDEN * E, kernel="k_elem<float,C3D8,Ogden>",
                    material="ogden mu=1.5e3 alpha=5 K=2e7 rho=1040")
    if name == "head":
        target = int(size) if size else 2_000_000
        mesh, mats, loads = mg.head_case(target_elements=target)
        E, N = len(mesh["etype"]), len(mesh["coordinates"])
        inner = int((mesh["pid"] == 1).sum())
        # C3D4: connectivity 16 B + part 4 B per element; interior fibre 12 B and
        # Prony history (H, S0: 12 f32) read + written 96 B; nodes as above
        eb = E * (16 + 4) + inner * (12 + 96) + N * ALG_BYTES_PER_NODE
        return dict(mesh=mesh, mats=mats, loads=loads, instances=None,
                    label="head_tet4_ellipsoid_%dk_shell_NH_core_GOH_prony_rotation" % (E // 1000),
                    alg_bytes=eb, flop=None, kernel="k_elem<float,C3D4,NH|GOH+Prony>",
                    material="shell NH E=6GPa nu=0.3; core GOH mu=1kPa k1=5kPa k2=10 kappa=0.1 "
                             "lambda=2.19e8 + Prony g1=0.6 tau1=6ms")
    if name == "head-impact":
        # the brain drivers' set-up: rigid skull (material 0) moved by sampled
        # angular and linear accelerations, integrated on the device each step
        target = int(size) if size else 2_000_000
        mesh, mats, loads, rec = mg.head_impact_case(target_elements=target)
        E, N = len(mesh["etype"]), len(mesh["coordinates"])
        inner = int((mesh["pid"] == 1).sum())
        eb = E * (16 + 4) + inner * (12 + 96) + N * ALG_BYTES_PER_NODE
        return dict(mesh=mesh, mats=mats, loads=loads, instances=None, rigid=rec,
                    label="head_tet4_ellipsoid_%dk_rigid_skull_GOH_prony_sampled_accelerations"
                          % (E // 1000),
                    alg_bytes=eb, flop=None, kernel="k_elem<float,C3D4,GOH+Prony>",
                    material="shell rigid (material 0); core GOH mu=1kPa k1=5kPa k2=10 "
                             "kappa=0.1 lambda=2.19e8 + Prony g1=0.6 tau1=6ms; 6 records at 10 kHz")
    if name == "ensemble":
        n = int(size) if size else 256
        mesh, mats, loads, off = mg.ensemble_case(n_instances=n)
        E, N = len(mesh["etype"]), len(mesh["coordinates"])
        inst = dict(node_offset=off, tmax=np.full(n, 1e300), reduction=np.full(n, 0.9))
        return dict(mesh=mesh, mats=mats, loads=loads, instances=inst,
                    label="ensemble_%d_ogden_hex8_blocks_4k_250k" % n,
                    alg_bytes=E * ALG_BYTES_PER_EL_C3D8 + N * ALG_BYTES_PER_NODE,
                    flop=FLOP_PER_EL_OGDEN * E, kernel="k_elem<float,C3D8,Ogden> (all instances)",
                    material="ogden per instance mu~U[0.5,5]kPa alpha~U[-5,8] K~U[2,50]MPa")
    raise SystemExit("unknown workload " + name)


def surrogate_summary(dev, size=None, steps=1000, warmup=20, samples=10_000_000, epochs=3,
                      trust_e2=0.04):
    """Head-like mesh: plain mixed path vs the learned surrogate for the GOH +
    Prony core, same steps, both against an FP64 run of the plain path (the
    FP64 GPU path matches the CPU oracle to ~1e-13 in the parity tests).
    The network is trained on the GPU first (its time is reported, not timed
    in the rates)."""
    import torch
    import femtech_gb300 as ft
    from femtech_gb300.surrogate import Surrogate
    wl = make_workload("head", size)
    mesh, mats, loads = wl["mesh"], wl["mats"], wl["loads"]
    E = len(mesh["etype"])
    props7 = list(mats["properties"].reshape(-1, 9)[1])
    t0 = time.perf_counter()
    s = Surrogate(props7, device=dev, seed=1)
    s.generate(samples, seed=2)
    loss = s.train(epochs=epochs, batch=8192, lr=2e-3)
    torch.cuda.synchronize(dev)
    t_train = time.perf_counter() - t0
    res = {}
    for name in ("plain", "surrogate", "fp64"):
        m = ft.Model(mesh, mats, precision=ft.FP64 if name == "fp64" else ft.MIXED, device=dev,
                     loads=loads)
        if name == "surrogate":
            m.set_surrogate(s, trust_e2=trust_e2)
        m.init_explicit(0.9, 0.0, 1e300)
        m.run(warmup)
        k, ms = timed_run(m, steps)
        res[name] = dict(steps=k, ms=ms, u=m.state()["u"], value=E * k / (ms / 1e3))
        m.close()
    s.close()
    ref = res["fp64"]["u"]

    def rel(a):
        return float(np.linalg.norm(a - ref) / max(np.linalg.norm(ref), 1e-300))

    return {"workload": wl["label"], "elements": E, "steps": steps, "warmup": warmup,
            "value": res["surrogate"]["value"], "unit": "element-updates/s",
            "ms_per_step": res["surrogate"]["ms"] / max(steps, 1),
            "plain_value": res["plain"]["value"],
            "speedup_vs_plain": res["surrogate"]["value"] / res["plain"]["value"],
            "rel_disp_err_vs_fp64": rel(res["surrogate"]["u"]),
            "plain_mixed_rel_disp_err_vs_fp64": rel(res["plain"]["u"]),
            "fp64_value": res["fp64"]["value"], "trust_e2": trust_e2,
            "train_samples": samples, "epochs": epochs, "final_batch_mse": loss,
            "train_s": t_train}


def surrogate_compare(args, dev):
    r = surrogate_summary(dev, args.size, args.steps, args.warmup, args.train_samples,
                          args.train_epochs, args.trust_e2)
    line = {
        "metric": "element-updates/s", "value": r["value"], "unit": "element-updates/s",
        "n_gpus": 1, "steps": r["steps"], "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 surrogate MLP (fp32 accumulate) / f32 element kernels / f64 nodal state",
        "data": "synthetic (seeded, generated in-run)",
        "config": {"workload": r["workload"] + "_surrogate", "elements": r["elements"],
                   "total_steps": args.warmup + args.steps, "trust_e2": args.trust_e2},
        "surrogate": r,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="block",
                    choices=["block", "head", "head-impact", "ensemble"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="ensemble: default launch shapes instead of the autotuned ones")
    ap.add_argument("--retune", action="store_true",
                    help="ensemble: tune again even when the cache holds this shape bucket")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the mixed-vs-FP64 displacement error of the block workload")
    ap.add_argument("--size", default=None,
                    help="block: nx,ny,nz; head: target elements; ensemble: instances")
    ap.add_argument("--injury", action="store_true",
                    help="per-step injury criteria over the elements of part 1 and above "
                         "(the brain drivers exclude the skull parts)")
    ap.add_argument("--energy", action="store_true",
                    help="track the energy balance (CheckEnergy) in the loop (single instance)")
    ap.add_argument("--surrogate", action="store_true",
                    help="head workload: plain vs learned surrogate vs FP64")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="block workload: skip the surrogate arm (head-like mesh) of the line")
    ap.add_argument("--train-samples", type=int, default=10_000_000)
    ap.add_argument("--train-epochs", type=int, default=3)
    ap.add_argument("--trust-e2", type=float, default=0.04)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps are required")

    import torch
    import femtech_gb300 as ft

    if args.surrogate:
        if rank == 0:
            surrogate_compare(args, local)
        return

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    t0 = time.perf_counter()
    wl = make_workload(args.workload, args.size)
    mesh, mats, loads = wl["mesh"], wl["mats"], wl["loads"]
    E = len(mesh["etype"])
    N = len(mesh["coordinates"])
    tuning = None
    if args.workload == "ensemble" and not args.no_tune:
        # the batched ensemble through the autotuner: its launch shapes are
        # tuned on this model (cached per shape bucket) and reported
        from femtech_gb300 import autotune as at
        model = at.tuned_model(mesh, mats, loads, wl["instances"], precision=ft.MIXED, device=dev,
                               retune=args.retune, steps=20)
        ch = model.tuning
        d_ms = ch["ms"].get("p128_t128_s1")
        b_ms = min(ch["ms"].values())
        tuning = {"patch": ch["patch"], "node_threads": ch["node_threads"],
                  "split": ch.get("split", 1), "default_ms_per_step": d_ms,
                  "tuned_ms_per_step": b_ms, "gain": (d_ms / b_ms) if d_ms else None,
                  "candidates_ms_per_step": ch["ms"]}
        wl["tuning"] = ch
    else:
        model = ft.Model(mesh, mats, precision=ft.MIXED, device=dev, loads=loads,
                         instances=wl["instances"])
    log("setup %.1f s (%d elements, %d nodes)" % (time.perf_counter() - t0, E, N))
    if wl.get("rigid") is not None:
        model.set_rigid_body(wl["rigid"])
    if args.energy:
        model.set_energy(True)
    if args.injury:
        model.set_injury(np.nonzero(np.asarray(mesh["pid"]) >= 1)[0])
    model.init_explicit(reduction=0.9, failure_dt=0.0, tmax=1e300)
    model.run(args.warmup)
    torch.cuda.synchronize(dev)

    # ---- timed region: device time of K steps ----
    sampler = ClockSampler(dev)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    steps, dev_ms = timed_run(model, args.steps)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = reduce_max_sum([dev_ms], world, "cuda:%d" % dev)[0]
    value = E * steps * world / (ms / 1000.0)
    # every step's kernels, plus the run's opening half-step (k_node; and
    # k_rigid_begin where acceleration records drive a rigid body)
    launches = model.launches_per_step() * steps + (2 if wl.get("rigid") is not None else 1)

    # ---- per-kernel times (events around every pass) for the roofline ----
    kp = min(args.steps, 400)
    pk = ft.lib()
    import ctypes as C
    sd, em, nm = C.c_int(), C.c_double(), C.c_double()
    ft._check(pk.ftgpu_run_profiled(model.h, kp, C.byref(sd), C.byref(em), C.byref(nm)))
    elem_ms = em.value / max(sd.value, 1)
    node_ms = nm.value / max(sd.value, 1)
    hbm, peak_kind = peaks()
    alg_bytes = wl["alg_bytes"]  # one step = one launch of each pass
    node_bytes = N * NODE_BYTES_PER_NODE
    if elem_ms >= node_ms:
        dom, dom_ms = wl["kernel"] + " (one element pass)", elem_ms
        traffic = load_traffic(args.workload, E)
    else:
        dom, dom_ms, traffic = "k_node_step<float> fused update", node_ms, None
    # the per-element-update algorithmic bytes over the dominant pass's time
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    fp32 = None
    binding = "hbm"
    if wl["flop"]:
        fp32_peak, fp32_src = fp32_peak_tflops(dev)
        fp32_ach = wl["flop"] / (elem_ms / 1e3) / 1e12
        fp32 = {"achieved": fp32_ach, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": fp32_ach / fp32_peak, "peak_source": fp32_src,
                "flop_per_element": wl["flop"] / E}
        # the roof that binds: the larger of the two lower bounds on time
        t_hbm = alg_bytes / (hbm * 1e9)
        t_fp32 = wl["flop"] / (fp32_peak * 1e12)
        binding = "fp32" if t_fp32 > t_hbm else "hbm"
        fp32["roof_ms"] = t_fp32 * 1e3
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                "algorithmic_bytes_per_element_update": alg_bytes / E,
                "launch_ms": dom_ms, "hbm_roof_ms": alg_bytes / (hbm * 1e9) * 1e3,
                "binding_roof": binding,
                "elem_pass_ms": elem_ms, "node_pass_ms": node_ms,
                "node_pass_algorithmic_gbs": node_bytes / (node_ms / 1e3) / 1e9,
                "node_pass_frac": node_bytes / (node_ms / 1e3) / 1e9 / hbm,
                "step_algorithmic_gbs": alg_bytes / (ms / max(steps, 1) / 1e3) / 1e9,
                "fp32": fp32}
    if traffic is not None and "C3D8" in wl["kernel"]:
        roofline["traffic_note"] = (
            "measured DRAM bytes of one element pass (ncu, scaled per element); they include "
            "the %d B/element Gauss-point geometry table and the slot replicas, which are "
            "overheads of this design, not algorithmic bytes" % GEO_TABLE_BYTES_PER_EL)

    # ---- end to end through the C ABI with host buffers ----
    if world > 1:
        torch.distributed.barrier()
    e2e = end_to_end(ft, wl, dev, args.steps, E, N)
    # whole job: every rank's element-updates over the slowest rank's time
    el_max = reduce_max_sum([e2e.pop("_elapsed_s")], world, "cuda:%d" % dev)[0]
    e2e["value"] = E * e2e.pop("_steps") * world / el_max

    line = {
        "metric": "element-updates/s", "value": value, "unit": "element-updates/s",
        "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms / max(steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 element kernels / f64 nodal state",
        "data": "synthetic (seeded, generated in-run)",
        "config": {"workload": wl["label"] + ("_energy_balance" if args.energy else "")
                   + ("_injury_criteria" if args.injury else ""),
                   "elements": E, "nodes": N,
                   "material": wl["material"], "precision": "mixed",
                   # device bytes from the set-up allocations: per C3D8 element 36 B
                   # + the 320 B geometry table, per C3D4 element about 80 B (with
                   # history and fibre), per node about 285 B with its slots
                   "l2": "inputs larger than L2 (about %.2f GB resident)" % (
                       (E * (356 if "C3D8" in wl["kernel"] else 80) + N * 285) / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": roofline,
        "e2e": e2e,
    }
    if rank == 0 and args.workload == "block" and not args.no_accuracy:
        acc = accuracy_vs_fp64(dev)
        line["rel_disp_err_vs_fp64"] = acc["rel_disp_err"]
        line["accuracy"] = acc
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.workload == "block":
        line["cpu_baseline"] = cpu_reference_rate(os.cpu_count() or 1)
    if rank == 0 and world == 1 and args.workload == "block" and not args.no_surrogate:
        # the metric's second arm: the learned surrogate on the head-like mesh
        line["surrogate"] = surrogate_summary(dev, steps=1000, warmup=20)
    if tuning is not None:
        line["tuning"] = tuning
    if args.energy:
        line["energy"] = model.energy()
    if args.injury:
        inj = model.injury()
        line["injury"] = {k: inj[k] for k in ("max_strain", "max_strain_elem", "mps95",
                                              "mps95_count", "steps")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    model.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def fp32_peak_tflops(dev):
    """Measured FP32 FMA rate of this GPU (the library's FMA-chain probe,
    CUDA events, best of five launches)."""
    import ctypes as C
    import femtech_gb300 as ft
    L = ft.lib()
    L.ftgpu_fp32_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    tf, msb = C.c_double(), C.c_double()
    ft._check(L.ftgpu_fp32_fma_peak(int(dev), C.byref(tf), C.byref(msb)))
    return tf.value, "measured (ftgpu_fp32_fma_peak: FMA chains on every SM, CUDA events)"


def accuracy_vs_fp64(dev, steps=5000, every=100):
    """Relative nodal-displacement error of the mixed path against the FP64
    path, max over outputs every `every` steps, on a 40x40x20 sub-block of the
    block workload (same spacing, jitter, law and loads) for the
    configuration's full 5000 steps.  The FP64 GPU path matches the CPU
    oracle on this sub-block to <= 1e-5 over 2000 steps
    (tests/test_gpu_scale_accuracy.py)."""
    import femtech_gb300 as ft
    sub = (40, 40, 20)
    mesh, mats, loads = build_workload(sub[0], sub[1], sub[2], LX * sub[0] / NX,
                                       LY * sub[1] / NY, LZ * sub[2] / NZ)
    outs = {}
    for name, prec in (("mixed", ft.MIXED), ("fp64", ft.FP64)):
        m = ft.Model(mesh, mats, precision=prec, device=dev, loads=loads)
        m.init_explicit(reduction=0.9, failure_dt=0.0, tmax=1e300)
        us = []
        for _ in range(steps // every):
            m.run(every)
            us.append(m.state()["u"])
        if name == "mixed":
            e9 = m.element_strain()[0]
            two_e = 2.0 * np.linalg.norm(e9, axis=1)
        outs[name] = us
        m.close()
    errs = [float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
            for a, b in zip(outs["mixed"], outs["fp64"])]
    k = int(np.argmax(errs))
    return {"rel_disp_err": max(errs), "at_step": (k + 1) * every, "final": errs[-1],
            "case": "%dx%dx%d sub-block (%d C3D8, same spacing/jitter/law/loads), mixed vs FP64 "
                    "on the GPU, %d steps, u every %d" % (sub + (len(mesh["etype"]), steps, every)),
            "share_2E_above_0.04": float((two_e > 0.04).mean()),
            "share_2E_above_0.2": float((two_e > 0.2).mean())}


def timed_run(model, steps):
    import ctypes as C
    import femtech_gb300 as ft
    sd, ms = C.c_int(), C.c_double()
    ft._check(ft.lib().ftgpu_run_timed(model.h, int(steps), C.byref(sd), C.byref(ms)))
    return sd.value, ms.value


def end_to_end(ft, wl, dev, steps, E, N):
    """Public-API run with host buffers: upload the initial state from host
    memory, run the loop, read all displacements back every 100 steps."""
    import torch
    ch = wl.get("tuning")
    model = ft.Model(wl["mesh"], wl["mats"], precision=ft.MIXED, device=dev, loads=wl["loads"],
                     instances=wl["instances"], patch_size=ch["patch"] if ch else 0,
                     setup=ch is None)
    if ch:
        from femtech_gb300 import autotune as at
        at.apply_choice(model, ch["node_threads"], ch.get("split", 1))
        model.setup()
    u0 = torch.zeros(3 * N, dtype=torch.float64).pin_memory().numpy()
    v0 = torch.zeros(3 * N, dtype=torch.float64).pin_memory().numpy()
    a0 = torch.zeros(3 * N, dtype=torch.float64).pin_memory().numpy()
    # pinned host arrays the state is read back into
    out = {k: torch.empty(3 * N, dtype=torch.float64).pin_memory().numpy() for k in "uva"}
    every = 100
    outs = 0
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    model.set_state(u0, v0, a0, 0.0)
    if wl.get("rigid") is not None:
        model.set_rigid_body(wl["rigid"])
    model.init_explicit(reduction=0.9, failure_dt=0.0, tmax=1e300)
    done = 0
    while done < steps:
        k = model.run(min(every, steps - done))
        done += k
        u = model.state(out=out)["u"]
        outs += 1
        if k == 0:
            break
    torch.cuda.synchronize(dev)
    el = time.perf_counter() - t
    model.close()
    del u
    h2d = 3 * 3 * N * 8
    d2h = outs * 3 * 3 * N * 8
    return {"value": E * done / el, "unit": "element-updates/s",
            "h2d_bytes_per_step": h2d / max(done, 1), "d2h_bytes_per_step": d2h / max(done, 1),
            "what": "set_state from pinned host arrays + init_explicit + run, full u/v/a read "
                    "back into pinned host arrays every %d steps" % every,
            "_elapsed_s": el, "_steps": done}


def load_traffic(workload, E):
    """DRAM bytes of one element pass from the committed ncu summary
    (profiles/traffic.json, bytes per element of a smaller capture of the same
    kernel), scaled by the element count: traffic grows in proportion to the
    elements processed."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    b = d.get(workload, {}).get("elem_pass_dram_bytes_per_element")
    return None if b is None else b * E


if __name__ == "__main__":
    main()
