#!/usr/bin/env python3
"""Throughput of the GB300 tracer-advection step (tracer-cell updates/s).

Default workload: the precision form at scale -- 2048x2048 nodes doubly
periodic (dx = 1 km), 64 layers stretched 5 m -> 250 m, 4 tracers (T, S, two
passive blobs), MUSCL horizontal + PPM vertical + FCT, FP32 form; the plain
FP64 path is timed on the same workload beside it. A step is one
do_oce_adv_tra for every tracer plus the tendency update, inputs resident in
HBM (they are far larger than the 129 MB L2, so no flush is needed).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the CPU implementation of the path

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tracer-cell updates/s (MUSCL+FCT): FP32/batched vs plain FP64; % HBM roofline"
UNIT = "tracer-cell updates/s"

WORKLOADS = {
    # BASELINE configuration 4: the precision form at scale.
    "precision_2048": dict(nx=2049, ny=2049, L=2048e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=400.0,
                           precision="fp32", compare_fp64=True),
    # Same configuration on a 512x512 grid (profiling case: a few hundred MB).
    "precision_512": dict(nx=513, ny=513, L=512e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=400.0,
                          precision="fp32", compare_fp64=False),
    # BASELINE configuration 2: the plain FP64 drop-in, MUSCL-FCT + QR4C.
    "fp64_512": dict(nx=513, ny=513, L=512e3, nz=48, K=2, hor="MUSCL", ver="QR4C", lim="FCT", dt=400.0,
                     precision="fp64", compare_fp64=False),
}


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------------------
# Clocks during the timed region
# ---------------------------------------------------------------------------
def _smi_id(local):
    """nvidia-smi id of the CUDA device (PCI bus id; CUDA_VISIBLE_DEVICES does not apply to nvidia-smi)."""
    try:
        import torch

        p = torch.cuda.get_device_properties(local)
        return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
    except Exception:
        return str(local)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = _smi_id(gpu_index)
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


# ---------------------------------------------------------------------------
# Algorithmic bytes per launch of each stage: per tracer-cell update, the
# tracer arrays an FCT step must move (A_t passes of s bytes: stage 1 reads T
# and writes adf_h (E/N = 3 per node), LO and adf_v; stage 2 reads LO, T,
# adf_h, adf_v and writes R+, R-; stage 3 reads adf_h, R+-, adf_v, LO and T
# and writes T: 23 passes, +1 per stage-1 read of a separate T_AB) plus the
# shared fields read once per step (A_s / K: uv 4, helem 2, w, area, hnode,
# hnode_new, areasvol 1 each, +2 for QR4C's Z and zbar). Without a limiter a
# fused gather pass needs A_t = 2 (+1 for T_AB) and A_s = 10. Split over this
# library's kernels as written below; intermediates the kernels add (the
# edge volume fluxes, repeated geometry reads) are not algorithmic.
# ---------------------------------------------------------------------------
def stage_bytes(m, K, s, ver, fct=True, copy_ab=True):
    cells = m.N * m.nz  # node-layers; x K tracer-cells
    ta = 0 if copy_ab else 1
    e = 3
    qr = 2 if ver == "QR4C" else 0
    b = {"vflux": cells * s * 6}                                   # uv (2 comps x 2 elements), helem
    if fct:
        b["hflux"] = cells * s * K * (1 + ta + e)                  # T (+T_AB) -> adf_h
        b["lo"] = cells * s * (5 + qr + K * 2)                      # w, area, hnode, hnode_new, areasvol -> LO, adf_v
        b["ratio"] = cells * s * K * (1 + 1 + e + 1 + 2)           # LO, T, adf_h, adf_v -> R+, R-
        b["update"] = cells * s * K * (e + 2 + 1 + 1 + 2)          # adf_h, R+-, adf_v, LO, T -> T
    else:
        b["hflux"] = cells * s * K * (1 + ta)                      # T (+T_AB)
        b["update"] = cells * s * (4 + qr + K * 1)                 # w_e, area, hnode_new, areasvol -> T
    return b


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload):
    """Per-launch DRAM bytes of each stage from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"dram_traffic_{workload}.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            f = line.split()
            if len(f) == 2 and not line.startswith("#"):
                try:
                    out[f[0]] = float(f[1])
                except ValueError:
                    pass
    return out


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def build_case(cfg, precision, device, seed=20260301):
    import numpy as np
    import torch

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    zb = synthetic.stretched_zbar(cfg["nz"], 5.0, 250.0)
    m = Mesh(cfg["nx"], cfg["ny"], cfg["nz"] + 1, Lx=cfg["L"], Ly=cfg["L"], depth=-zb[-1], periodic=True,
             orient_left=True, zbar=zb)
    dtype = torch.float32 if precision == "fp32" else torch.float64
    rng = np.random.default_rng(seed)
    vel, w = synthetic.flat_streamfunction_device(m, rng, cfg["dt"], dtype, device, cfl=0.4)
    T0 = synthetic.tracers_device(m, cfg["K"], seed, dtype, device)
    eng = TracerAdvection(m, cfg["K"], precision, cfg["hor"], cfg["ver"], cfg["lim"], copy_ab=True, device=device)
    eng.load_padded(T=T0, vel=vel, w=w)
    del T0
    return m, eng, eng.T.clone()  # initial values in the engine's tracer layout


def time_engine(eng, T0, dt, steps, warmup, dist_barrier, per_stage=True):
    import torch

    from fesom2_tracer_dwarf_gb300 import _lib

    stages = [_lib.STAGE_VFLUX, _lib.STAGE_HFLUX, _lib.STAGE_LO, _lib.STAGE_RATIO, _lib.STAGE_UPDATE]
    names = ["vflux", "hflux", "lo", "ratio", "update"]
    if eng.lim != "FCT":
        stages = [_lib.STAGE_VFLUX, _lib.STAGE_HFLUX, _lib.STAGE_UPDATE]
        names = ["vflux", "hflux", "update"]
    for _ in range(warmup):
        eng.step(dt)
    eng.T.copy_(T0)
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = eng.launches
    dist_barrier()
    torch.cuda.synchronize()
    start.record()
    for k in range(steps):
        ev[k][0].record()
        for i, st in enumerate(stages):
            eng.step(dt, stages=st)
            ev[k][i + 1].record()
    end.record()
    torch.cuda.synchronize()
    dist_barrier()
    total_ms = start.elapsed_time(end)
    per = {n: statistics.mean(ev[k][i].elapsed_time(ev[k][i + 1]) for k in range(steps)) for i, n in enumerate(names)}
    return total_ms, per, eng.launches - launches0


def time_e2e(eng, T0, dt, steps, dist_barrier):
    """Same step through the public API with host buffers: H2D of the tracer
    fields from pinned memory, the step, D2H of the result, every step."""
    import torch

    host_in = torch.empty(T0.shape, dtype=T0.dtype, pin_memory=True)
    host_in.copy_(T0.cpu())
    host_out = torch.empty_like(host_in).pin_memory()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_barrier()
    start.record()
    for _ in range(steps):
        eng.T.copy_(host_in, non_blocking=True)
        eng.step(dt)
        host_out.copy_(eng.T, non_blocking=True)
    end.record()
    torch.cuda.synchronize()
    dist_barrier()
    nbytes = host_in.numel() * host_in.element_size()
    return start.elapsed_time(end), nbytes, nbytes


def cpu_sample(seconds=12.0, nx=129, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=400.0, seed=7):
    """The oracle (single-threaded C restatement) on a bounded sample of the
    same workload: same schemes, layers and resolution on a smaller domain."""
    import numpy as np

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh
    from oracle import oracle as O

    O.build()
    zb = synthetic.stretched_zbar(nz, 5.0, 250.0)
    L = (nx - 1) * 1000.0
    om = O.Mesh(nx, nx, nz + 1, Lx=L, Ly=L, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb)
    hm = Mesh(nx, nx, nz + 1, Lx=L, Ly=L, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb, upload=False)
    rng = np.random.default_rng(seed)
    vel, w = synthetic.streamfunction_flow(hm, rng, dt, cfl=0.4)
    T = np.ascontiguousarray(np.stack([synthetic.gaussian_T(hm, rng), synthetic.salinity(hm, rng)] +
                                      [synthetic.passive_blob(hm, rng) for _ in range(K - 2)]))
    vab = T.copy()
    W = O.Work(om)
    cells = om.nod2D * nz * K
    t0 = time.perf_counter()
    n = 0
    while True:
        O.analytic_step(om, W, dt, vel, w, T, vab, [(hor, ver, lim)] * K, copy_ab=True)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return cells * n / el, f"{nx - 1}x{nx - 1} periodic, {nz} layers, {K} tracers, {hor}/{ver}/{lim}, {n} step(s), {el:.1f} s"


def run_gpu(args):
    import torch

    rank, world, local = _env_rank()
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    from fesom2_tracer_dwarf_gb300 import _lib

    _lib.load()
    cfg = WORKLOADS[args.workload]
    m, eng, T0 = build_case(cfg, cfg["precision"], device)
    cells = m.N * m.nz * cfg["K"]
    tuned = None
    if not args.no_tune:
        from fesom2_tracer_dwarf_gb300 import autotune

        tuned = autotune.tune(eng, cfg["dt"], reps=3)
    with ClockSampler(local) as clk:
        total_ms, per, launches = time_engine(eng, T0, cfg["dt"], args.steps, args.warmup, barrier)
    clocks = clk.summary()
    ms = total_ms / args.steps
    t_max = ms
    if dist is not None:
        tt = torch.tensor([ms], device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = cells * world / (t_max / 1e3)
    # roofline of the dominant stage
    s = 4 if cfg["precision"] == "fp32" else 8
    sb = stage_bytes(m, cfg["K"], s, cfg["ver"], fct=cfg["lim"] == "FCT")
    dom = max(per, key=per.get)
    peak, peak_kind = load_peaks()
    achieved = sb[dom] / (per[dom] / 1e3) / 1e9
    traffic = load_traffic(args.workload).get(dom)
    step_bytes = sum(sb.values())
    # e2e through the public API with host buffers
    e2e_steps = max(2, min(args.steps, 10))
    e2e_ms, h2d, d2h = time_e2e(eng, T0, cfg["dt"], e2e_steps, barrier)
    e2e_value = cells * world / (e2e_ms / e2e_steps / 1e3)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if cfg["precision"] == "fp32" else "f64", "data": "synthetic",
        "config": {"workload": args.workload,
                   "mesh": f"{cfg['nx'] - 1}x{cfg['ny'] - 1} doubly periodic analytic grid, dx=1 km, "
                           f"{cfg['nz']} layers 5->250 m",
                   "nodes": m.N, "edges": m.E, "elements": m.M, "tracers": cfg["K"],
                   "schemes": f"{cfg['hor']}/{cfg['ver']}/{cfg['lim']}", "form": cfg["precision"], "dt_s": cfg["dt"],
                   "tracer_cells_per_step": cells, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{world}",
                   "launch_cfg": tuned["cfg"] if tuned else "default"},
        "stage_ms": {k: round(v, 4) for k, v in per.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": sb[dom]},
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "achieved_gbs": step_bytes / (ms / 1e3) / 1e9,
                          "frac": step_bytes / (ms / 1e3) / 1e9 / peak},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "ms_per_step": e2e_ms / e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if cfg.get("compare_fp64") and not args.no_fp64:
        del eng, T0
        torch.cuda.empty_cache()
        m64, e64, T64 = build_case(cfg, "fp64", device)
        if not args.no_tune:
            autotune.tune(e64, cfg["dt"], reps=1)
        n64 = max(2, min(args.steps, args.fp64_steps))
        tot64, per64, l64 = time_engine(e64, T64, cfg["dt"], n64, min(args.warmup, 2), barrier)
        ms64 = tot64 / n64
        result["fp64"] = {"value": cells * world / (ms64 / 1e3), "ms_per_step": ms64, "steps": n64,
                          "stage_ms": {k: round(v, 3) for k, v in per64.items()}}
        result["fp32_over_fp64"] = value / result["fp64"]["value"]
        result["gpu_launches"] += l64
        del e64
    if rank == 0 and not args.no_cpu:
        v, sample = cpu_sample(seconds=args.cpu_seconds, K=cfg["K"], nz=cfg["nz"], hor=cfg["hor"], ver=cfg["ver"],
                               lim=cfg["lim"], dt=cfg["dt"])
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Reference arm: the CPU implementation of the path on all host cores
# ---------------------------------------------------------------------------
def _ref_worker(args):
    seconds, nx, nz, K, hor, ver, lim, dt, seed = args
    sys.path.insert(0, ROOT)
    return cpu_sample(seconds=seconds, nx=nx, nz=nz, K=K, hor=hor, ver=ver, lim=lim, dt=dt, seed=seed)


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    import multiprocessing as mp

    cfg = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    from oracle import oracle as O

    O.build()
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_ref_worker, [(args.cpu_seconds, 65, cfg["nz"], cfg["K"], cfg["hor"], cfg["ver"],
                                      cfg["lim"], cfg["dt"], 100 + i) for i in range(cores)])
        el = time.perf_counter() - t0
    value = sum(r[0] for r in res)
    sample = (f"{cores} concurrent processes of the single-threaded C restatement (the Fortran reference has no "
              f"compiler on this machine), each: {res[0][1]}")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload, "schemes": f"{cfg['hor']}/{cfg['ver']}/{cfg['lim']}",
                      "layers": cfg["nz"], "tracers": cfg["K"], "wall_s": el},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="precision_2048", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="use the default launch configuration")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
