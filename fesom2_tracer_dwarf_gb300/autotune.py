"""Launch-configuration autotuner for the tracer-advection step.

The step is five kernels (vertical fluxes, edge fluxes, FCT low-order
solution, FCT ratios, update); four of them have launch knobs that do not
change results (fgb_step_desc.cfg): edges per block of the edge-flux kernel
(FP32: or the tiled edge kernel), node columns per block of the three node
kernels, and tracers per chunk (FP64) or layers per lane per pass (FP32). The
best choice depends on the mesh size, the number of layers, the tracer count
and the precision, so this module times the candidates of each kernel on the
caller's own engine (its mesh, fields and schemes) and keeps the fastest.

Each kernel is tuned on its own: a full step fills the workspace, then every
candidate of one stage is run ``reps`` times between CUDA events on the
engine's stream and the median is kept. Re-running the flux, LO and ratio
stages is idempotent; the update stage advances the tracers, so the tracer
fields are saved before tuning and restored afterwards.

Results are cached by (device, precision, K, schemes, mesh size) in memory,
and in a JSON file when ``cache_path`` (or FGB_AUTOTUNE_CACHE) names one.
"""
from __future__ import annotations

import json
import os
from itertools import product

from . import _lib

EDGE_WARPS = (2, 4, 8)
NODE_WARPS = (1, 2, 4)
CHUNKS = (1, 2, 4)
SLICES = (1, 2)

_MEMO: dict = {}


def chunk_candidates(K: int):
    """Tracers per chunk that divide K (the library falls back otherwise)."""
    return [c for c in CHUNKS if K % c == 0]


def stage_candidates(stage: str, K: int, precision: str = "fp64", wsplit: bool = False):
    """Candidate knob values per tuned stage: a list of dicts of cfg index -> value.
    FP64: block size and tracers per chunk. FP32 (one tracer group at a time):
    block size and layers per lane per pass, and under w_split the solver of
    the implicit vertical step (part of the LO stage)."""
    if stage == "hflux":
        if precision == "fp32":
            # + the tiled kernel (node rows staged once per tile; its own launch shape)
            return [{0: w, 7: ns} for w, ns in product(EDGE_WARPS, SLICES)] + [{9: 1}]
        return [{0: w} for w in EDGE_WARPS]
    slot = {"lo": 0, "ratio": 1, "update": 2}[stage]
    if precision == "fp32":
        # the ratio kernel also has variants without shared memory (3; 4: fewer registers); the
        # LO stage a whole-column kernel (3: columns of at most 64 layers, not under w_split;
        # its block shape is fixed, so one candidate)
        slices = SLICES + ((3, 4) if stage == "ratio" else ())
        cands = [{1 + slot: w, 4 + slot: ns} for w, ns in product(NODE_WARPS, slices)]
        if stage == "lo" and not wsplit:
            cands.append({1 + slot: 4, 4 + slot: 3})
        if stage == "lo" and wsplit:
            cands = [{**c, 8: solver} for c in cands for solver in (0, 1)]
        return cands
    return [{1 + slot: w, 4 + slot: c} for w, c in product(NODE_WARPS, chunk_candidates(K))]


def cache_key(engine) -> str:
    import torch

    m = engine.mesh
    dev = torch.cuda.get_device_name(engine.device)
    return "|".join(str(x) for x in (dev, engine.precision, engine.K, engine.V, engine.hor, engine.ver, engine.lim,
                                     m.N, m.E, m.nz, "wsplit" if engine.wi is not None else "w"))


def _load_file(path):
    if not path or not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def _save_file(path, table):
    if not path:
        return
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time_stage(engine, mask, dt, reps):
    import torch

    stream = torch.cuda.current_stream(engine.device)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
    engine.step(dt, 1, mask)  # warm-up (also sets the shared-memory attribute)
    for r in range(reps):
        ev[2 * r].record(stream)
        engine.step(dt, 1, mask)
        ev[2 * r + 1].record(stream)
    torch.cuda.synchronize(engine.device)
    ts = sorted(ev[2 * r].elapsed_time(ev[2 * r + 1]) for r in range(reps))
    return ts[reps // 2]


def tune(engine, dt: float = 1.0, reps: int = 5, cache_path: str | None = None, force: bool = False):
    """Pick the fastest launch configuration for ``engine`` and apply it.

    Returns {"cfg": [12 ints], "ms": {stage: best ms}, "cached": bool}.
    """
    import torch

    cache_path = cache_path if cache_path is not None else os.environ.get("FGB_AUTOTUNE_CACHE")
    key = cache_key(engine)
    if not force:
        hit = _MEMO.get(key) or _load_file(cache_path).get(key)
        if hit:
            _MEMO[key] = hit
            engine.set_launch(hit["cfg"])
            return dict(hit, cached=True)

    saved = [engine.T.clone()] + ([engine.TA.clone()] if engine.TA is not None else [])
    saved_lo = engine.Tlo.clone() if getattr(engine, "Tlo", None) is not None else None
    fct = engine.lim == "FCT"
    stages = [("hflux", _lib.STAGE_HFLUX)]
    stages += [("lo", _lib.STAGE_LO), ("ratio", _lib.STAGE_RATIO)] if fct else []
    stages += [("update", _lib.STAGE_UPDATE)]
    cfg = [0] * _lib.NCFG
    engine.set_launch(cfg)
    engine.step(dt, 1)  # fills every workspace array the stages read
    best_ms = {}
    for name, mask in stages:
        best = None
        for cand in stage_candidates(name, engine.K, engine.precision, engine.wi is not None):
            trial = list(cfg)
            for i, v in cand.items():
                trial[i] = v
            engine.set_launch(trial)
            ms = _time_stage(engine, mask, dt, reps)
            if best is None or ms < best[0]:
                best = (ms, cand)
        for i, v in best[1].items():
            cfg[i] = v
        best_ms[name] = best[0]
    engine.set_launch(cfg)
    engine.T.copy_(saved[0])
    if engine.TA is not None:
        engine.TA.copy_(saved[1])
    if saved_lo is not None:
        engine.Tlo.copy_(saved_lo)
    torch.cuda.synchronize(engine.device)
    result = {"cfg": cfg, "ms": best_ms}
    _MEMO[key] = result
    if cache_path:
        table = _load_file(cache_path)
        table[key] = result
        _save_file(cache_path, table)
    return dict(result, cached=False)
