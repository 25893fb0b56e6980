#!/usr/bin/env python3
"""Throughput of the GB300 tracer-advection step (tracer-cell updates/s).

Default workload: the precision form at scale -- 2048x2048 nodes doubly
periodic (dx = 1 km), 64 layers stretched 5 m -> 250 m, 4 tracers (T, S, two
passive blobs), MUSCL horizontal + PPM vertical + FCT, FP32 form with each
value's FP32 rounding residual carried by the update; the plain FP64 path
(fast and bit-exact forms) is timed on the same workload beside it, and a
100-step FP32-vs-FP64 precision report follows. A step is one do_oce_adv_tra
for every tracer plus the tendency update, inputs resident in HBM (they are
far larger than the 129 MB L2, so no flush is needed). The batching form
(batch_16: 16 meshes in one union, CUDA graphs of 50 steps, against per-mesh
sequential FP64 steps) is the line's second figure, under "batch_16"; the
closed 1024^2 basin (FP32 residual form against fast FP64) and the 512^2 x 48
FP64 configuration with MUSCL and with upwind fluxes follow under "side".

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the CPU implementation of the path

Other workloads (--workload): the same at 512^2 (precision_512), with w_split
(wsplit_2048, wsplit_512), the plain FP64 form (fp64_512), a closed ragged
basin (closed_1024), 16 meshes in one union (batch_16), and the reference's pi
mesh refined 3 or 5 times (pi_refined3, pi_refined5).

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
    # The precision form at scale: 2048^2 x 64 doubly periodic, 4 tracers (default).
    # The FP32 form with each value's rounding residual (the precision form that meets the
    # conservation target) and the LO fluxes summed with compensation.
    "precision_2048": dict(kind="flat", nx=2049, L=2048e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT",
                           dt=400.0, precision="fp32", compare_fp64=True, report_steps=100, residual=True,
                           batch="batch_16", side=("closed_1024", "fp64_512", "fp64_512_upw1")),
    # The default workload with w_split: w = we + wi, we clipped at a quarter of
    # max |w|; the LO stage adds the implicit vertical solve with wi.
    "wsplit_2048": dict(kind="flat", nx=2049, L=2048e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT",
                        dt=400.0, precision="fp32", compare_fp64=False, wsplit=0.25),
    # The same on a 512x512 grid (profiling case of the implicit kernel).
    "wsplit_512": dict(kind="flat", nx=513, L=512e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=400.0,
                       precision="fp32", compare_fp64=False, wsplit=0.25),
    # Same configuration on a 512x512 grid (profiling case: a few hundred MB).
    "precision_512": dict(kind="flat", nx=513, L=512e3, nz=64, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=400.0,
                          precision="fp32", compare_fp64=False),
    # The plain FP64 drop-in: 512^2 x 48 periodic, 2 tracers, MUSCL-FCT + QR4C.
    "fp64_512": dict(kind="flat", nx=513, L=512e3, nz=48, K=2, hor="MUSCL", ver="QR4C", lim="FCT", dt=400.0,
                     precision="fp64", compare_fp64=False),
    # The same with upwind horizontal fluxes (the other scheme of that configuration).
    "fp64_512_upw1": dict(kind="flat", nx=513, L=512e3, nz=48, K=2, hor="UPW1", ver="QR4C", lim="FCT", dt=400.0,
                          precision="fp64", compare_fp64=False),
    # Closed ragged basin: 1024^2 with seeded bathymetry (8..64 layers), walls,
    # MUSCL-FCT + PPM; FP32 form against plain FP64 over 100 steps.
    "closed_1024": dict(kind="closed", nx=1025, L=1024e3, nz=64, min_layers=8, K=2, hor="MUSCL", ver="PPM",
                        lim="FCT", dt=400.0, precision="fp32", compare_fp64=True, report_steps=100, residual=True),
    # An unstructured global ocean mesh: the reference's pi mesh (coasts,
    # ragged bottom, 47 layers) with every triangle split into four 5 times
    # (3.0 M nodes, 9.0 M edges); FP32 form against plain FP64.
    "pi_refined5": dict(kind="files", refine=5, nz=47, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=600.0,
                        precision="fp32", compare_fp64=True, report_steps=3),
    "pi_refined3": dict(kind="files", refine=3, nz=47, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=600.0,
                        precision="fp32", compare_fp64=False),
    # pi_refined5 with its nodes, elements and edges renumbered at random (a
    # file order without locality): the kernels' Hilbert visit order, and
    # the file order for comparison.
    "pi_refined5_shuffled": dict(kind="files", refine=5, nz=47, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=600.0,
                                 precision="fp32", compare_fp64=False, shuffle=True),
    "pi_refined5_shuffled_fileorder": dict(kind="files", refine=5, nz=47, K=4, hor="MUSCL", ver="PPM", lim="FCT",
                                           dt=600.0, precision="fp32", compare_fp64=False, shuffle=True,
                                           keep_order=True),
    "pi_refined5_fileorder": dict(kind="files", refine=5, nz=47, K=4, hor="MUSCL", ver="PPM", lim="FCT", dt=600.0,
                                  precision="fp32", compare_fp64=False, keep_order=True),
    # Batching form: 16 periodic meshes of seeded uneven size (64..1024 nodes a
    # side, 16..64 layers), 8 tracers, one launch per stage over all of them,
    # 50 steps per CUDA graph; against per-mesh sequential plain FP64 steps.
    "batch_16": dict(kind="batch", parts=16, K=8, hor="MUSCL", ver="QR4C", lim="FCT", dt=300.0, precision="fp32",
                     compare_fp64="sequential", graph_steps=50),
}


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def job_rate(ms_local, cells_local, dist=None, device="cpu"):
    """Whole-job figures of a replicas run: each rank advanced its own copy
    (cells_local tracer-cell updates per step) in ms_local per step. The job's
    time per step is the slowest rank's, its work the sum over ranks. Returns
    (ms per step, tracer-cell updates/s)."""
    import torch

    tm = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    tc = torch.tensor([float(cells_local)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(tm, op=dist.ReduceOp.MAX)
        dist.all_reduce(tc, op=dist.ReduceOp.SUM)
    t_max = float(tm.item())
    return t_max, float(tc.item()) / (t_max / 1e3)


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
def stage_bytes(m, K, s, ver, fct=True, copy_ab=True, wsplit=False, residual=False):
    cells = m.N * m.nz  # node-layers; x K tracer-cells
    ta = 0 if copy_ab else 1
    e = 3
    qr = 2 if ver == "QR4C" else 0
    b = {"vflux": cells * s * 6}                                   # uv (2 comps x 2 elements), helem
    if fct:
        b["hflux"] = cells * s * K * (1 + ta + e)                  # T (+T_AB) -> adf_h
        b["lo"] = cells * s * (5 + qr + K * 2)                      # w, area, hnode, hnode_new, areasvol -> LO, adf_v
        if wsplit:
            b["lo"] += cells * s * 2                                # w_e, w_i (the implicit solve on LO in place)
        b["ratio"] = cells * s * K * (1 + 1 + e + 1 + 2)           # LO, T, adf_h, adf_v -> R+, R-
        b["update"] = cells * s * K * (e + 2 + 1 + 1 + 2)          # adf_h, R+-, adf_v, LO, T -> T
        if residual:
            b["update"] += cells * s * K * 2                        # the rounding residual, read and written
    else:
        b["hflux"] = cells * s * K * (1 + ta)                      # T (+T_AB)
        b["update"] = cells * s * (4 + qr + K * 1)                 # w_e, area, hnode_new, areasvol -> T
    return b


NOMINAL_HBM_GBS = 8000.0


def compulsory_bytes(s, K, ver):
    """Lower bound per tracer-cell update, not the roofline: the tracer read
    and written once (2 s) and the shared fields read once (uv 4, helem 2, w,
    area, hnode, hnode_new, areasvol, +2 for QR4C's Z and zbar) per K tracers."""
    return 2 * s + s * (11 + (2 if ver == "QR4C" else 0)) / K


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
def _pad_dim(x, dim, width):
    import torch

    if x.shape[dim] == width:
        return x
    shape = list(x.shape)
    shape[dim] = width - x.shape[dim]
    return torch.cat([x, torch.zeros(shape, dtype=x.dtype, device=x.device)], dim=dim)


def batch_parts(cfg, seed=20260301):
    """Seeded part list of the batching form: (nodes per side, layers, CFL)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sizes = rng.choice([64, 128, 256, 512, 1024], size=cfg["parts"])
    layers = rng.integers(16, 65, size=cfg["parts"])
    cfls = rng.uniform(0.2, 0.5, size=cfg["parts"])
    return [(int(n), int(z), float(c)) for n, z, c in zip(sizes, layers, cfls)]


def workload_config(name, cfg, world=1):
    """The workload as both arms report it (``config``): the mesh, its sizes
    and the schemes, from the workload's definition alone (no mesh is built,
    no library is loaded)."""
    kind = cfg["kind"]
    if kind == "flat":
        n = cfg["nx"] - 1
        N, E, M = n * n, 3 * n * n, 2 * n * n
        mesh = f"{n}x{n} doubly periodic analytic grid, dx=1 km, {cfg['nz']} layers 5->250 m"
    elif kind == "closed":
        nx = cfg["nx"]
        N, E, M = nx * nx, 3 * (nx - 1) ** 2 + 2 * (nx - 1), 2 * (nx - 1) ** 2
        mesh = (f"{nx - 1}x{nx - 1} closed basin ({nx}x{nx} nodes), seeded bathymetry, "
                f"{cfg['min_layers']}..{cfg['nz']} layers 5->250 m")
    elif kind == "files":
        N, E, M = 3140, 8986, 5839  # the reference's pi mesh (tests/data/pi)
        for _ in range(cfg["refine"]):  # each triangle split into four
            N, E, M = N + E, 2 * E + 3 * M, 4 * M
        order = ("nodes, elements and edges renumbered at random" if cfg.get("shuffle")
                 else "Morton-ordered nodes")
        visit = "file order" if cfg.get("keep_order") else "Hilbert visit order"
        mesh = (f"the reference's pi mesh (global ocean, coasts, ragged bottom of {cfg['nz']} layers) with each "
                f"triangle split into four {cfg['refine']} times, {order}, kernels in {visit}; synthetic "
                f"layered flow, W from continuity")
    else:
        parts = batch_parts(cfg)
        N = sum(n * n for n, _, _ in parts)
        E, M = 3 * N, 2 * N
        mesh = "union of %d periodic meshes (n, layers, CFL): %s" % (
            cfg["parts"], ", ".join(f"{n}^2/{z}/{c:.2f}" for n, z, c in parts))
    return {"workload": name, "mesh": mesh, "nodes": N, "edges": E, "elements": M, "tracers": cfg["K"],
            "schemes": f"{cfg['hor']}/{cfg['ver']}/{cfg['lim']}", "dt_s": cfg["dt"],
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}",
            "w_split": (f"we = w clipped at {cfg['wsplit']} max|w|, wi = w - we" if cfg.get("wsplit") else None)}


def _flat_part(n, nz, precision, device, dt, cfl, K, seed, upload=True):
    import numpy as np
    import torch

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    zb = synthetic.stretched_zbar(nz, 5.0, 250.0)
    m = Mesh(n + 1, n + 1, nz + 1, Lx=n * 1e3, Ly=n * 1e3, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb,
             upload=upload)
    dtype = torch.float32 if precision == "fp32" else torch.float64
    rng = np.random.default_rng(seed)
    vel, w = synthetic.flat_streamfunction_device(m, rng, dt, dtype, device, cfl=cfl)
    T = synthetic.tracers_device(m, K, seed, dtype, device)
    return m, vel, w, T


_FILES_CACHE = {}


def shuffled_numbering(a, seed):
    """The same mesh with its nodes, elements and edges renumbered by seeded
    random permutations (edges within the interior and the boundary ranges, so
    interior edges still come first): a file order without locality."""
    import numpy as np

    rng = np.random.default_rng(seed)
    N, M = len(a["lonlat"]), len(a["elem"])
    E, Ein = int(a["edgenum"][0]), int(a["edgenum"][1])
    pn, pm = rng.permutation(N), rng.permutation(M)   # new index of each old node / element
    pe = np.concatenate([rng.permutation(Ein), Ein + rng.permutation(E - Ein)])
    out = dict(a)
    out["lonlat"] = np.empty_like(a["lonlat"])
    out["lonlat"][pn] = a["lonlat"]
    out["nlvls"] = np.empty_like(a["nlvls"])
    out["nlvls"][pn] = a["nlvls"]
    elem = np.empty_like(a["elem"])
    elem[pm] = pn[a["elem"] - 1] + 1
    out["elem"] = elem
    out["elvls"] = np.empty_like(a["elvls"])
    out["elvls"][pm] = a["elvls"]
    edges = np.empty_like(a["edges"])
    edges[pe] = pn[a["edges"] - 1] + 1
    out["edges"] = edges
    et = a["edge_tri"]
    et_new = np.where(et > 0, pm[np.maximum(et, 1) - 1] + 1, et)
    out["edge_tri"] = np.empty_like(et)
    out["edge_tri"][pe] = et_new
    return out


def _files_case(cfg, precision, device, seed):
    """The refined pi mesh (host set-up shared by both forms), a layered
    streamfunction flow tapered at the coasts with W from continuity, and T, S
    and passive blobs; velocity, W and tracers built padded on the device."""
    import numpy as np
    import torch

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh
    from fesom2_tracer_dwarf_gb300.meshfiles import refine

    key = (cfg["refine"], cfg["K"], seed, bool(cfg.get("shuffle")), bool(cfg.get("keep_order")))
    if key not in _FILES_CACHE:
        with np.load(os.path.join(ROOT, "tests", "golden", "pi_mesh.npz")) as z:
            base = {k: z[k] for k in z.files}
        arrays = refine(base, cfg["refine"])
        if cfg.get("shuffle"):
            arrays = shuffled_numbering(arrays, seed)
        m = Mesh.from_arrays(**arrays, euler_degrees=True, cyclic_2pi=True, keep_order=bool(cfg.get("keep_order")))
        rng = np.random.default_rng(seed)
        u, s, w = synthetic.layered_flow(m, rng, cfg["dt"], cfl=0.4)
        T = [synthetic.gaussian_T(m, rng), synthetic.salinity(m, rng)]
        T += [synthetic.passive_blob(m, rng) for _ in range(cfg["K"] - 2)]
        _FILES_CACHE.clear()
        _FILES_CACHE[key] = (m, u, s, w, T)
    m, u, s, w, T = _FILES_CACHE[key]
    dt_ = torch.float32 if precision == "fp32" else torch.float64
    st = torch.zeros(m.LZ, dtype=dt_, device=device)
    st[: m.nz] = torch.from_numpy(s).to(device, dt_)
    vel = torch.from_numpy(u).to(device, dt_)[:, None, :] * st[None, :, None]
    wt = torch.zeros(m.N, m.LW, dtype=dt_, device=device)
    wt[:, : m.nl] = torch.from_numpy(w).to(device, dt_)
    T0 = torch.zeros(len(T), m.N, m.LZ, dtype=dt_, device=device)
    for i, t in enumerate(T):
        T0[i, :, : m.nz] = torch.from_numpy(t).to(device, dt_)
    return m, vel, wt, T0


def build_case(cfg, precision, device, seed=20260301):
    """Mesh, engine and initial tracer values (engine layout) of a workload."""
    import numpy as np
    import torch

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    sch = (cfg["hor"], cfg["ver"], cfg["lim"])
    res = bool(cfg.get("residual")) and precision == "fp32"  # the FP32 rounding residual
    if cfg["kind"] == "flat":
        m, vel, w, T0 = _flat_part(cfg["nx"] - 1, cfg["nz"], precision, device, cfg["dt"], 0.4, cfg["K"], seed)
        eng = TracerAdvection(m, cfg["K"], precision, *sch, copy_ab=True, device=device,
                              tracer_vec=cfg.get("tracer_vec") if precision == "fp32" else None, residual=res)
        eng.load_padded(T=T0, vel=vel, w=w)
        if cfg.get("wsplit"):
            c = float(w.abs().max()) * cfg["wsplit"]
            we = w.clamp(-c, c)
            eng.load_padded(we=we, wi=w - we)
            del we
    elif cfg["kind"] == "files":
        m, vel, w, T0 = _files_case(cfg, precision, device, seed)
        eng = TracerAdvection(m, cfg["K"], precision, *sch, copy_ab=True, device=device,
                              tracer_vec=cfg.get("tracer_vec") if precision == "fp32" else None, residual=res)
        eng.load_padded(T=T0, vel=vel, w=w)
        del vel, w, T0
    elif cfg["kind"] == "closed":
        rng = np.random.default_rng(seed)
        zb = synthetic.stretched_zbar(cfg["nz"], 5.0, 250.0)
        en = synthetic.bathymetry_levels(cfg["nx"], cfg["nx"], zb, rng, min_layers=cfg["min_layers"])
        m = Mesh(cfg["nx"], cfg["nx"], cfg["nz"] + 1, Lx=cfg["L"], Ly=cfg["L"], depth=-zb[-1], periodic=False,
                 orient_left=True, zbar=zb, elem_nlev=en)
        vel, w = synthetic.streamfunction_flow(m, rng, cfg["dt"], cfl=0.4, psi_wall_zero=True)
        T = np.stack([synthetic.gaussian_T(m, rng), synthetic.salinity(m, rng)] +
                     [synthetic.passive_blob(m, rng) for _ in range(cfg["K"] - 2)])
        eng = TracerAdvection(m, cfg["K"], precision, *sch, copy_ab=True, device=device,
                              tracer_vec=cfg.get("tracer_vec") if precision == "fp32" else None, residual=res)
        eng.set_velocity(vel, w)
        eng.set_tracers(T)
        del vel, w, T
    else:
        parts, vels, ws, Ts = [], [], [], []
        for i, (n, nz, cfl) in enumerate(batch_parts(cfg, seed)):
            p, v, w, T = _flat_part(n, nz, precision, device, cfg["dt"], cfl, cfg["K"], seed + i, upload=False)
            parts.append(p)
            vels.append(v)
            ws.append(w)
            Ts.append(T)
        m = Mesh.union(parts)
        vel = torch.cat([_pad_dim(v, 1, m.LZ) for v in vels], dim=0)
        w = torch.cat([_pad_dim(x, 1, m.LW) for x in ws], dim=0)
        T0 = torch.cat([_pad_dim(t, 2, m.LZ) for t in Ts], dim=1)
        del vels, ws, Ts
        eng = TracerAdvection(m, cfg["K"], precision, *sch, copy_ab=True, device=device,
                              tracer_vec=cfg.get("tracer_vec") if precision == "fp32" else None, residual=res)
        eng.load_padded(T=T0, vel=vel, w=w)
    return m, eng, eng.T.clone()


# (name, plain-sum mask or None for the engine's default, residual, anomaly offsets)
REPORT_VARIANTS = (("residual", None, True, None), ("residual_all_compensated", False, True, None),
                   ("residual_plain_sums", True, True, None), ("plain", None, False, None),
                   ("compensated", False, False, None), ("anomaly", None, False, "auto"))


def precision_report(m, e32, T32, e64, T64, dt, steps, variants=REPORT_VARIANTS):
    """The FP32 form against the fast FP64 form (within 1e-12 of the
    bit-exact form the oracle pins) from the same initial values after
    `steps` steps. Per tracer: the max-norm error relative to max |T|,
    the relative change of the volume integral sum(T hnode_new areasvol) --
    with the FP64 geometry, and with the FP32-rounded geometry the FP32 form
    itself runs on (its discrete invariant) -- and the FCT extremum
    violations (wet cells outside the initial [min, max], and the largest
    excursion relative to the initial range). The FP32 form runs several ways,
    which separates the error sources: "residual" (each value carries its FP32
    rounding residual; the low-order fluxes summed with compensation, the
    engine's default with the residual), "residual_all_compensated" (every sum
    compensated), "residual_plain_sums" (none), "plain" (no residual, plain
    sums: FP32 storage rounding), "compensated" (no residual, every sum
    compensated) and "anomaly" (no residual, each tracer stored as T - c about
    its initial mean where that shrinks the stored values, offsets="auto")."""
    import torch

    e64.T.copy_(T64)
    e64.step(dt, steps)
    torch.cuda.synchronize()
    dev = e64.T.device
    nz = m.nz
    nlev = torch.as_tensor(m.get("nlevels_nod2D"), device=dev)
    wet = (torch.arange(nz, device=dev)[None, :] < (nlev - 1)[:, None])
    av, hnn = m.get("areasvol")[:, :nz], m.get("hnode_new")
    vol = torch.as_tensor(av * hnn, device=dev) * wet
    vol32 = torch.as_tensor(av.astype("float32").astype("float64") * hnn.astype("float32").astype("float64"),
                            device=dev) * wet
    init = e64.from_layout(T64)[:, :, :nz].double()
    b = e64.from_layout(e64.T)[:, :, :nz]
    K = init.shape[0]
    s0 = [float((init[t] * vol).sum()) for t in range(K)]
    s0_32 = [float((init[t] * vol32).sum()) for t in range(K)]
    bounds = [(float(init[t][wet].min()), float(init[t][wet].max())) for t in range(K)]

    def extrema(x, t):
        lo, hi = bounds[t]
        xv = x[wet]
        return int(((xv < lo) | (xv > hi)).sum()), max(0.0, lo - float(xv.min()), float(xv.max()) - hi) / max(hi - lo,
                                                                                                             1e-300)

    out = {"steps": steps, "fp64": {"sum_rel_err": [abs(float((b[t] * vol).sum()) - s0[t]) / abs(s0[t])
                                                    for t in range(K)],
                                    "violations": [extrema(b[t], t)[0] for t in range(K)],
                                    "max_excursion": [extrema(b[t], t)[1] for t in range(K)]}}
    plain0, req0, res0 = e32.plain_sums, e32._offsets_req, e32.residual
    for name, plain, res, offs in variants:
        e32.plain_sums = plain
        e32.set_residual(res)
        e32._offsets_req = offs
        # from the FP64 initial values: rounded to FP32, with their residual where kept
        e32.load_padded(T=e64.from_layout(T64).clone())
        e32.step(dt, steps)
        torch.cuda.synchronize()
        a = e32.full_values()[:, :, :nz]
        r = {"max_rel_err": [float((a[t] - b[t])[wet].abs().max()) / float(b[t][wet].abs().max()) for t in range(K)],
             "sum_rel_err": [abs(float((a[t] * vol).sum()) - s0[t]) / abs(s0[t]) for t in range(K)],
             "sum_rel_err_fp32_geometry": [abs(float((a[t] * vol32).sum()) - s0_32[t]) / abs(s0_32[t])
                                           for t in range(K)],
             "violations": [extrema(a[t], t)[0] for t in range(K)],
             "max_excursion": [extrema(a[t], t)[1] for t in range(K)]}
        if offs:
            r["offsets"] = [float(c) for c in e32.offsets]
        out[name] = r
    e32.plain_sums, e32._offsets_req = plain0, req0
    e32.set_residual(res0)
    e32.offsets = None
    e32.T.copy_(T32)
    if e32.Tlo is not None:
        e32.load_padded(T=e64.from_layout(T64).clone())
    # the timed form's figures under the keys of earlier reports
    # the variant the engine itself runs (its sums and residual), else the first
    timed = next((v[0] for v in variants if v[1] is plain0 and v[2] == res0), variants[0][0])
    out["timed_form"] = timed
    out["max_rel_err"] = out[timed]["max_rel_err"]
    out["sum_rel_err_fp32"] = out[timed]["sum_rel_err"]
    out["sum_rel_err_fp64"] = out["fp64"]["sum_rel_err"]
    return out


def time_engine(eng, T0, dt, steps, warmup, dist_barrier, stage_steps=5):
    """Full steps between CUDA events (the timed region), then a per-stage
    breakdown on separate steps that launch one stage at a time (stages that
    overlap inside a full step are timed apart there)."""
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
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = eng.launches
    dist_barrier()
    torch.cuda.synchronize()
    start.record()
    for _ in range(steps):
        eng.step(dt)
    end.record()
    torch.cuda.synchronize()
    dist_barrier()
    total_ms = start.elapsed_time(end)
    launches = eng.launches - launches0
    # stage breakdown
    nst = max(1, min(steps, stage_steps))
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(nst)]
    for k in range(nst):
        ev[k][0].record()
        for i, st in enumerate(stages):
            eng.step(dt, stages=st)
            ev[k][i + 1].record()
    torch.cuda.synchronize()
    per = {n: statistics.mean(ev[k][i].elapsed_time(ev[k][i + 1]) for k in range(nst)) for i, n in enumerate(names)}
    eng.T.copy_(T0)
    return total_ms, per, launches


def time_e2e(eng, T0, dt, steps, dist_barrier):
    """Same steps through the public API with host buffers
    (TracerAdvection.run_host): every step is one batch whose tracer fields
    are copied host-to-device from pinned memory, stepped, and copied back
    device-to-host; the copies of neighbouring batches overlap the steps. The
    copy streams per direction (1, 2 or 4) are picked by six trial batches
    each before the timed run. Returns (ms, H2D bytes, D2H bytes per batch,
    copy streams, ms per trial batch by stream count)."""
    import torch

    host_in = torch.empty(T0.shape, dtype=T0.dtype, pin_memory=True)
    host_in.copy_(T0.cpu())
    host_out = torch.empty_like(host_in).pin_memory()
    if eng.Tlo is not None:  # the residual form: each batch is the pair (values, residuals)
        lo = torch.empty_like(host_in).pin_memory()
        lo.copy_(eng.Tlo.cpu())
        host_in, host_out = (host_in, lo), (host_out, torch.empty_like(lo).pin_memory())
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # warm-up, and the number of copy streams per direction that runs the
    # batches fastest on this machine (host-device copy rates vary by host)
    best, trials = None, {}
    for nc in (1, 2, 4):
        eng.run_host([host_in], [host_out], dt, copy_streams=nc)
        torch.cuda.synchronize()
        start.record()
        eng.run_host([host_in] * 6, [host_out] * 6, dt, copy_streams=nc)
        end.record()
        torch.cuda.synchronize()
        trials[nc] = round(start.elapsed_time(end) / 6, 2)
        if best is None or start.elapsed_time(end) < best[0]:
            best = (start.elapsed_time(end), nc)
    nc = best[1]
    eng.T.copy_(T0)
    torch.cuda.synchronize()
    dist_barrier()
    start.record()
    eng.run_host([host_in] * steps, [host_out] * steps, dt, copy_streams=nc)
    end.record()
    torch.cuda.synchronize()
    dist_barrier()
    eng.T.copy_(T0)
    halves = host_in if isinstance(host_in, tuple) else (host_in,)
    nbytes = sum(h.numel() * h.element_size() for h in halves)
    return start.elapsed_time(end), nbytes, nbytes, nc, trials


def cpu_sample_case(cfg, n=None, seed=7):
    """A bounded sample of a workload for the CPU legs, built by the oracle
    and numpy alone: a doubly periodic n x n grid with the workload's layers,
    tracers, schemes, dt and CFL (the same dx and flow construction)."""
    from oracle import workloads as WL

    nz = cfg.get("nz", 48)
    n = n or min(cfg.get("nx", 513) - 1, 512)
    m, vel, w, T = WL.flat_case(n, nz, cfg["K"], cfg["dt"], seed=seed)
    wsp = None
    if cfg.get("wsplit"):
        c = float(abs(w).max()) * cfg["wsplit"]
        we = w.clip(-c, c)
        wsp = dict(wi=w - we, we=we)
    desc = f"{n}x{n} periodic, {nz} layers, {cfg['K']} tracers, {cfg['hor']}/{cfg['ver']}/{cfg['lim']}"
    return m, vel, w, T, wsp, desc


def cpu_steps(case, cfg, threads, steps=None, seconds=None, warmup=1):
    """Whole steps of the oracle on a sample (cpu_sample_case) on `threads`
    threads: `warmup` untimed steps, then `steps` timed steps (or as many as
    fit in `seconds`, at least two). Returns (tracer-cell updates/s, timed
    steps, seconds)."""
    from oracle import oracle as O

    m, vel, w, T, wsp, _ = case
    O.set_threads(threads)
    vals = T.copy()
    vab = vals.copy()
    W = O.Work(m)
    sch = [(cfg["hor"], cfg["ver"], cfg["lim"])] * cfg["K"]
    kw = wsp or {}

    def one():
        O.analytic_step(m, W, cfg["dt"], vel, w, vals, vab, sch, copy_ab=True, **kw)

    for _ in range(warmup):
        one()
    n, el = 0, 0.0
    while True:
        t0 = time.perf_counter()
        one()
        el += time.perf_counter() - t0
        n += 1
        if (steps is not None and n >= steps) or (steps is None and n >= 2 and el >= seconds):
            break
    cells = m.nod2D * (m.nl - 1) * cfg["K"]
    return cells * n / el, n, el


def cpu_baseline(cfg, seconds=12.0):
    """The oracle on the host cores (all of them, and one) on a 256 x 256
    sample of the workload, about `seconds` of timed steps each."""
    from oracle import oracle as O

    O.build()
    case = cpu_sample_case(cfg, n=min(cfg.get("nx", 257) - 1, 256))
    cores = os.cpu_count() or 1
    v_all, n_all, el_all = cpu_steps(case, cfg, cores, seconds=seconds)
    v_one, n_one, el_one = cpu_steps(case, cfg, 1, seconds=seconds)
    return {"value": v_all, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"{case[5]}: {n_all} whole steps in {el_all:.1f} s on {cores} threads (the C restatement "
                       f"with OpenMP; the Fortran reference has no compiler here)"),
            "value_1_thread": v_one, "sample_1_thread": f"{n_one} steps in {el_one:.1f} s on 1 thread"}


def time_graph(eng, T0, dt, graph_steps, replays, warmup, dist_barrier):
    """The batching form's timing: `graph_steps` steps captured as one CUDA
    graph, replayed `replays` times between CUDA events."""
    import torch

    l0 = eng.launches
    g = eng.capture(dt, graph_steps)  # one eager step, then graph_steps captured steps
    launches_per_replay = (eng.launches - l0) * graph_steps // (graph_steps + 1)
    for _ in range(max(1, warmup // graph_steps)):
        g.replay()
    eng.T.copy_(T0)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_barrier()
    start.record()
    for _ in range(replays):
        g.replay()
    end.record()
    torch.cuda.synchronize()
    dist_barrier()
    return start.elapsed_time(end), launches_per_replay


def sequential_fp64(cfg, n64, device, dist, cells):
    """Per-mesh sequential plain FP64 steps of a batching workload (eager
    launches, one mesh after another): the denominator of the batching form."""
    import torch

    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection

    tot64, l64 = 0.0, 0
    for i, (n, nz, cfl) in enumerate(batch_parts(cfg)):
        p, v, w, T = _flat_part(n, nz, "fp64", device, cfg["dt"], cfl, cfg["K"], 20260301 + i)
        e = TracerAdvection(p, cfg["K"], "fp64", cfg["hor"], cfg["ver"], cfg["lim"], copy_ab=True, device=device)
        e.load_padded(T=T, vel=v, w=w)
        e.step(cfg["dt"])
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        l0 = e.launches
        t0.record()
        e.step(cfg["dt"], n64)
        t1.record()
        torch.cuda.synchronize()
        tot64 += t0.elapsed_time(t1)
        l64 += e.launches - l0
        del e, p, v, w, T
    ms64 = tot64 / n64
    return {"value": job_rate(ms64, cells, dist, device)[1], "ms_per_step": ms64, "steps": n64,
            "mode": "per-mesh sequential eager launches", "gpu_launches": l64}


def run_side_figure(name, args, device, dist, barrier):
    """A further configuration's figures on the same run: its own form timed
    over whole steps after tuning, and for an FP32 workload the fast FP64 form
    beside it (no precision report, no e2e: the headline carries those)."""
    import torch

    from fesom2_tracer_dwarf_gb300 import autotune

    cfg = WORKLOADS[name]
    m, eng, T0 = build_case(cfg, cfg["precision"], device)
    cells = m.wet_cells() * cfg["K"]
    tuned = None if args.no_tune else autotune.tune(eng, cfg["dt"], reps=1)
    steps = max(3, min(args.steps, 10))
    tot, per, launches = time_engine(eng, T0, cfg["dt"], steps, min(args.warmup, 3), barrier, stage_steps=2)
    t_max, value = job_rate(tot / steps, cells, dist, device)
    out = {"workload": name, "config": workload_config(name, cfg, dist.get_world_size() if dist else 1),
           "form": cfg["precision"], "residual": bool(eng.residual), "value": value, "unit": UNIT,
           "ms_per_step": t_max, "steps": steps, "tracer_cells_per_step": cells,
           "stage_ms": {k: round(v, 4) for k, v in per.items()},
           "launch_cfg": tuned["cfg"] if tuned else "default", "gpu_launches": launches}
    del eng, m, T0
    torch.cuda.empty_cache()
    if cfg["precision"] == "fp32" and not args.no_fp64:
        m64, e64, T64 = build_case(cfg, "fp64fast", device)
        n64 = max(2, min(args.steps, args.fp64_steps))
        tot64, _, _ = time_engine(e64, T64, cfg["dt"], n64, min(args.warmup, 2), barrier, stage_steps=1)
        out["fp64"] = {"form": "fp64fast", "ms_per_step": tot64 / n64, "value": job_rate(tot64 / n64, cells, dist,
                                                                                          device)[1]}
        out["fp32_over_fp64"] = value / out["fp64"]["value"]
        del e64, m64, T64
        torch.cuda.empty_cache()
    return out


def run_batch_form(name, args, device, dist, barrier, local):
    """The batching form as a second figure of a run: the union of the
    workload's meshes stepped by CUDA graphs of graph_steps steps (one launch
    per stage over every mesh), its own clocks, and the per-mesh sequential
    plain FP64 steps it replaces."""
    import torch

    from fesom2_tracer_dwarf_gb300 import autotune

    cfg = WORKLOADS[name]
    m, eng, T0 = build_case(cfg, cfg["precision"], device)
    cells = m.wet_cells() * cfg["K"]
    tuned = None if args.no_tune else autotune.tune(eng, cfg["dt"], reps=3)
    replays = max(1, args.batch_steps // cfg["graph_steps"])
    with ClockSampler(local) as clk:
        total_ms, per_replay = time_graph(eng, T0, cfg["dt"], cfg["graph_steps"], replays, args.warmup, barrier)
    nsteps = replays * cfg["graph_steps"]
    ms = total_ms / nsteps
    t_max, value = job_rate(ms, cells, dist, device)
    out = {"workload": name, "config": workload_config(name, cfg, dist.get_world_size() if dist else 1),
           "form": cfg["precision"], "value": value, "unit": UNIT, "ms_per_step": t_max, "steps": nsteps,
           "cuda_graph_steps": cfg["graph_steps"], "tracer_cells_per_step": cells,
           "launch_cfg": tuned["cfg"] if tuned else "default", "gpu_launches": per_replay * replays,
           "clocks": clk.summary()}
    del eng, m, T0
    torch.cuda.empty_cache()
    if not args.no_fp64:
        n64 = max(1, min(nsteps, args.fp64_steps))
        out["fp64"] = sequential_fp64(cfg, n64, device, dist, cells)
        out["over_fp64"] = value / out["fp64"]["value"]
    return out


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

    from fesom2_tracer_dwarf_gb300 import _lib, autotune

    _lib.load()
    cfg = WORKLOADS[args.workload]
    m, eng, T0 = build_case(cfg, cfg["precision"], device)
    K = cfg["K"]
    cells = m.wet_cells() * K
    tuned = None
    if not args.no_tune:
        tuned = autotune.tune(eng, cfg["dt"], reps=3)
    graph = cfg["kind"] == "batch"
    with ClockSampler(local) as clk:
        if graph:
            replays = max(1, args.steps // cfg["graph_steps"])
            total_ms, per_replay = time_graph(eng, T0, cfg["dt"], cfg["graph_steps"], replays, args.warmup, barrier)
            nsteps = replays * cfg["graph_steps"]
            launches = per_replay * replays
            per = None
        else:
            nsteps = args.steps
            total_ms, per, launches = time_engine(eng, T0, cfg["dt"], args.steps, args.warmup, barrier)
    clocks = clk.summary()
    ms = total_ms / nsteps
    t_max, value = job_rate(ms, cells, dist, device)
    s = 4 if cfg["precision"] == "fp32" else 8
    wet_frac = m.wet_cells() / (m.N * m.nz)
    sb = {k: v * wet_frac for k, v in stage_bytes(m, K, s, cfg["ver"], fct=cfg["lim"] == "FCT",
                                                  wsplit=bool(cfg.get("wsplit")), residual=eng.residual).items()}
    peak, peak_kind = load_peaks()
    step_bytes = sum(sb.values())
    if per is None:  # graph: per-stage times of one eager step for the roofline split
        _, per, _ = time_engine(eng, T0, cfg["dt"], 2, 1, barrier)
    dom = max(per, key=per.get)
    achieved = sb[dom] / (per[dom] / 1e3) / 1e9
    traffic = load_traffic(args.workload).get(dom)
    e2e_steps = 40  # the first H2D and the last D2H, which nothing overlaps, spread over 40 batches
    e2e_ms, h2d, d2h, e2e_nc, e2e_trials = time_e2e(eng, T0, cfg["dt"], e2e_steps, barrier)
    _, e2e_value = job_rate(e2e_ms / e2e_steps, cells, dist, device)
    config = workload_config(args.workload, cfg, world)
    assert (config["nodes"], config["edges"], config["elements"]) == (m.N, m.E, m.M), "workload sizes"
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": nsteps,
        "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if cfg["precision"] == "fp32" else "f64", "data": "synthetic",
        "config": config,
        "form": cfg["precision"], "tracer_cells_per_step": cells, "cuda_graph_steps": cfg.get("graph_steps"),
        "launch_cfg": tuned["cfg"] if tuned else "default",
        "stage_ms": {k: round(v, 4) for k, v in per.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": sb[dom]},
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "bytes_per_tracer_cell": step_bytes / cells,
                          "achieved_gbs": step_bytes / (ms / 1e3) / 1e9,
                          "frac": step_bytes / (ms / 1e3) / 1e9 / peak,
                          # against the nominal 8.0 TB/s of HBM3e
                          "frac_nominal": step_bytes / (ms / 1e3) / 1e9 / NOMINAL_HBM_GBS,
                          # informational: read T once, write T once, the shared fields once
                          "compulsory_bytes_per_tracer_cell": compulsory_bytes(s, K, cfg["ver"]),
                          "compulsory_frac": compulsory_bytes(s, K, cfg["ver"]) * cells / (ms / 1e3) / 1e9 / peak},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "ms_per_step": e2e_ms / e2e_steps, "copy_streams": e2e_nc,
                "trial_ms_per_batch": e2e_trials},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if cfg.get("compare_fp64") is True and not args.no_fp64:
        # the plain FP64 path: the fast FP64 form (fused multiply-add, shared
        # reciprocals; within 1e-12 of the bit-exact form) is the denominator of
        # fp32_over_fp64, the bit-exact form is timed beside it
        n64 = max(2, min(args.steps, args.fp64_steps))
        # the bit-exact form first; the fast form stays for the precision report
        for key, prec in (("fp64_exact", "fp64"), ("fp64", "fp64fast")):
            m64, e64, T64 = build_case(cfg, prec, device)
            if not args.no_tune:
                autotune.tune(e64, cfg["dt"], reps=1)
            tot64, per64, l64 = time_engine(e64, T64, cfg["dt"], n64, min(args.warmup, 2), barrier)
            ms64 = tot64 / n64
            result[key] = {"form": prec, "value": job_rate(ms64, cells, dist, device)[1], "ms_per_step": ms64,
                           "steps": n64, "stage_ms": {k: round(v, 3) for k, v in per64.items()},
                           "gpu_launches": l64}
            if key == "fp64_exact":
                del e64, m64, T64
                torch.cuda.empty_cache()  # the mesh and workspace allocations are the library's own
        result["fp32_over_fp64"] = value / result["fp64"]["value"]
        result["fp32_over_fp64_exact"] = value / result["fp64_exact"]["value"]
        # the FP64 forms' bound: this device's FP64 FMA and division rates
        result["fp64_peak"] = _lib.probe_fp64(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if cfg.get("report_steps") and not args.no_report:
            result["precision_report"] = precision_report(m, eng, T0, e64, T64, cfg["dt"], cfg["report_steps"])
        del e64, m64, T64
        torch.cuda.empty_cache()
    elif cfg.get("compare_fp64") == "sequential" and not args.no_fp64:
        n64 = max(1, min(args.steps, args.fp64_steps))
        result["fp64"] = sequential_fp64(cfg, n64, device, dist, cells)
        result["fp32_over_fp64"] = value / result["fp64"]["value"]
    if cfg.get("batch") and not args.no_batch:
        torch.cuda.empty_cache()
        result[cfg["batch"]] = run_batch_form(cfg["batch"], args, device, dist, barrier, local)
    if cfg.get("side") and not args.no_side:
        del eng, T0  # the headline's engine and tracer buffers
        torch.cuda.empty_cache()
        result["side"] = {name: run_side_figure(name, args, device, dist, barrier) for name in cfg["side"]}
    if cfg["kind"] == "files":
        lev = m.get("nlevels_nod2D") - 1
        result["mesh_layers"] = {"min": int(lev.min()), "max": int(lev.max()), "mean": float(lev.mean())}
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(cfg, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Reference arm: the CPU implementation of the path on all host cores
# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference's algorithm on the host CPU: the oracle (the C
    restatement of the Fortran; no Fortran compiler exists on these machines)
    with OpenMP on every host core. Each step is one whole step on a bounded
    sample of the workload (a 512 x 512 periodic grid with the workload's
    layers, tracers, schemes and dt, built by the oracle and numpy: no product
    library is loaded); `warmup` untimed steps, then `steps` steps timed one
    by one. Under torchrun only rank 0 runs."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    cfg = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    case = cpu_sample_case(cfg)
    O.set_threads(cores)
    # keep the whole run within a few minutes: a smaller sample if one step is slow
    _, _, el = cpu_steps(case, cfg, cores, steps=1, warmup=0)
    if el * (args.steps + args.warmup) > 240.0:
        case = cpu_sample_case(cfg, n=256)
    t0 = time.perf_counter()
    value, n, el = cpu_steps(case, cfg, cores, steps=args.steps, warmup=args.warmup)
    wall = time.perf_counter() - t0
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": n,
           "warmup": args.warmup, "ms_per_step": el / n * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(args.workload, cfg, world),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": (f"each step one whole step of a {case[5]} sample of the workload; "
                                       f"the C restatement of the Fortran with OpenMP on {cores} threads "
                                       f"(no Fortran compiler on this machine); {n} timed steps, {wall:.1f} s "
                                       f"with the warm-up")},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_profile(args):
    """The kernels of `args.profile` plain steps of a workload, nothing else
    timed or launched by this library (the command the ncu summaries cite)."""
    import torch

    from fesom2_tracer_dwarf_gb300 import _lib

    _lib.load()
    cfg = WORKLOADS[args.workload]
    m, eng, _ = build_case(cfg, args.precision or cfg["precision"], "cuda:0")
    if args.launch_cfg:
        eng.set_launch([int(x) for x in args.launch_cfg.split(",")])
    if args.plain_sums is not None:
        eng.plain_sums = int(args.plain_sums)
    if args.residual is not None:
        eng.set_residual(bool(args.residual))
    torch.cuda.synchronize()
    eng.step(cfg["dt"], args.profile)
    torch.cuda.synchronize()
    print(json.dumps({"workload": args.workload, "form": eng.precision, "steps": args.profile,
                      "launch_cfg": eng.cfg, "plain_sums": eng.plain_sums, "residual": eng.residual,
                      "launches": eng.launches}))


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
    ap.add_argument("--no-report", action="store_true", help="skip the FP32-vs-FP64 precision report")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching form's second figure")
    ap.add_argument("--no-side", action="store_true", help="skip the further configurations' figures")
    ap.add_argument("--batch-steps", type=int, default=100,
                    help="steps of the batching form's second figure (whole CUDA graphs)")
    ap.add_argument("--no-tune", action="store_true", help="use the default launch configuration")
    ap.add_argument("--profile", type=int, default=0, metavar="N",
                    help="build the workload, run N plain steps (for a profiler) and exit")
    ap.add_argument("--precision", choices=["fp32", "fp64", "fp64fast"], default=None,
                    help="with --profile: the form to run (default: the workload's)")
    ap.add_argument("--launch-cfg", default=None,
                    help="with --profile: launch configuration, comma-separated (default: the library's)")
    ap.add_argument("--plain-sums", type=int, default=None,
                    help="with --profile: FP32 plain-sum bit mask (1 LO, 2 update, 4 FCT sums; default: "
                         "6 with the residual, 7 without)")
    ap.add_argument("--residual", type=int, default=None, help="with --profile: 1 keeps the FP32 rounding residual")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
