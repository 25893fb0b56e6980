"""FP32 form (tracer-grouped layout, regrouped arithmetic) against the FP64
oracle.

The FP32 form stores and computes in single precision and regroups the
reference's arithmetic (tracer-independent coefficients once per layer), so
the bar is a tolerance, not equality: the max-norm error relative to the
field's magnitude stays below 1e-5 (single steps and 20-step runs), for every
scheme combination on periodic, closed-wall and ragged meshes, for tracer
groups of 4, 2 and 1.
"""
import itertools
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import engine, mesh, synthetic

    return mesh, engine, synthetic


MESHES = {
    "periodic": dict(nx=11, ny=9, nl=8, periodic=True),
    "periodic_full": dict(nx=9, ny=10, nl=7, periodic=True, cluster_full=True),
    "closed": dict(nx=10, ny=8, nl=9, periodic=False),
    "closed_left": dict(nx=10, ny=8, nl=9, periodic=False, orient_left=True),
}


def _ragged(nx=12, ny=10, nl=12, seed=3):
    from fesom2_tracer_dwarf_gb300 import synthetic

    rng = np.random.default_rng(seed)
    zb = synthetic.stretched_zbar(nl - 1, 5.0, 120.0)
    en = synthetic.bathymetry_levels(nx, ny, zb, rng, min_layers=3)
    return dict(nx=nx, ny=ny, nl=nl, periodic=False, zbar=zb, elem_nlev=en, orient_left=True)


def _pair(O, mesh_mod, **kw):
    return O.Mesh(**kw), mesh_mod.Mesh(**kw)


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.parametrize("meshname", ["periodic", "periodic_full", "closed", "closed_left", "ragged"])
@pytest.mark.parametrize("hor,ver,lim", list(itertools.product(["UPW1", "MUSCL", "MFCT"],
                                                                ["UPW1", "QR4C", "CDIFF", "PPM"],
                                                                ["NONE", "FCT"])))
def test_fp32_single_step_all_schemes(pkg, oracle_mod, meshname, hor, ver, lim):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    kw = _ragged() if meshname == "ragged" else MESHES[meshname]
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(zlib.crc32(f"fp32/{meshname}/{hor}/{ver}/{lim}".encode()))
    vel, w = synthetic.random_flow(m, rng)
    K = 4
    T = synthetic.random_field(m, rng, K)
    TA = T + rng.normal(0, 0.05, size=T.shape)
    dt = 400.0
    vals = np.ascontiguousarray(T.copy())
    vab = np.ascontiguousarray(TA.copy())
    W = O.Work(om)
    O.analytic_step(om, W, dt, vel, w, vals, vab, [(hor, ver, lim, 0.7, 0.6)] * K)
    # FCT: also with each value's FP32 rounding residual (the benchmark's form)
    for residual in ((False, True) if lim == "FCT" else (False,)):
        eng = engine.TracerAdvection(m, K, "fp32", hor, ver, lim, ph=0.7, pv=0.6, residual=residual)
        assert eng.V == 4 and eng.residual == residual
        eng.set_tracers(T, TA)
        eng.set_velocity(vel, w)
        eng.step(dt)
        torch.cuda.synchronize()
        err = _rel(eng.values(), vals)
        assert err <= REL_TOL, f"{meshname} {hor}/{ver}/{lim} residual={residual}: relative max error {err:.3g}"


@pytest.mark.parametrize("K,V", [(1, 1), (2, 2), (3, 1), (6, 2), (8, 4), (4, 1), (4, 2)])
@pytest.mark.parametrize("sch", [("MUSCL", "PPM", "FCT"), ("MFCT", "QR4C", "NONE")])
def test_fp32_tracer_groups(pkg, oracle_mod, K, V, sch):
    """Every group width and group count gives the same per-tracer answer."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    om, m = _pair(O, mesh_mod, **_ragged(seed=K))
    rng = np.random.default_rng(100 + K)
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, K)
    dt = 300.0
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * K, copy_ab=True)
    eng = engine.TracerAdvection(m, K, "fp32", *sch, copy_ab=True, tracer_vec=V)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    eng.step(dt)
    torch.cuda.synchronize()
    assert _rel(eng.values(), vals) <= REL_TOL
    st = eng.stats()
    got = eng.values()
    assert np.allclose(st[:, 0], got.reshape(K, -1).min(axis=1))
    assert np.allclose(st[:, 1], got.reshape(K, -1).max(axis=1))
    assert np.allclose(st[:, 2], got.reshape(K, -1).sum(axis=1), rtol=1e-12)


@pytest.mark.parametrize("case", ["periodic_muscl_qr4c", "ragged_muscl_ppm", "closed_upw1_fct", "frozen_ab"])
def test_fp32_multistep(pkg, oracle_mod, case):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    copy_ab = case != "frozen_ab"
    if case == "periodic_muscl_qr4c":
        kw, sch = dict(MESHES["periodic"], orient_left=True), ("MUSCL", "QR4C", "FCT")
    elif case in ("ragged_muscl_ppm", "frozen_ab"):
        kw, sch = _ragged(), ("MUSCL", "PPM", "FCT")
    else:
        kw, sch = MESHES["closed_left"], ("UPW1", "UPW1", "FCT")
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(5)
    dt = 300.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4, psi_wall_zero=True)
    K = 4
    T = synthetic.random_field(m, rng, K)
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    engs = [engine.TracerAdvection(m, K, "fp32", *sch, copy_ab=copy_ab, residual=r) for r in (False, True)]
    for eng in engs:
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
    for _ in range(20):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * K, copy_ab=copy_ab)
        for eng in engs:
            eng.step(dt)
    torch.cuda.synchronize()
    for eng in engs:
        assert _rel(eng.values(), vals) <= REL_TOL, f"residual={eng.residual}"


def test_fp32_workspace_views_follow_groups(pkg, oracle_mod):
    """The per-tracer views of the grouped work arrays hold each tracer's LO
    solution (to FP32 rounding)."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    om, m = _pair(O, mesh_mod, **MESHES["periodic"])
    rng = np.random.default_rng(17)
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, 4)
    from fesom2_tracer_dwarf_gb300 import _lib

    eng = engine.TracerAdvection(m, 4, "fp32", "MUSCL", "QR4C", "FCT")
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    eng.step(300.0, stages=_lib.STAGE_VFLUX | _lib.STAGE_HFLUX | _lib.STAGE_LO)
    torch.cuda.synchronize()
    lo = eng.workspace_view("lo")[:, :, : m.nz].double().cpu().numpy()
    for t in range(4):
        W = O.Work(om)
        O.do_oce_adv_tra(om, W, 300.0, vel, w, T[t], T[t], "MUSCL", "QR4C", "FCT")
        assert _rel(lo[t], W.get("fct_LO")) <= REL_TOL


@pytest.mark.parametrize("meshname", ["periodic", "closed_left", "ragged"])
@pytest.mark.parametrize("hor,lim", [("UPW1", "FCT"), ("MUSCL", "FCT"), ("MFCT", "FCT"), ("MUSCL", "NONE")])
@pytest.mark.parametrize("K,V,frozen", [(4, 4, False), (4, 4, True), (6, 2, False), (3, 1, True)])
def test_fp32_tiled_edge_kernel(pkg, oracle_mod, meshname, hor, lim, K, V, frozen):
    """The tiled edge-flux kernel (cfg[9] = 1: node rows staged once per tile)
    gives the default kernel's fluxes and the oracle's step, with T_AB shared
    or separate, for every group width."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    kw = _ragged() if meshname == "ragged" else MESHES[meshname]
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(zlib.crc32(f"tile/{meshname}/{hor}/{lim}/{K}/{frozen}".encode()))
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, K)
    TA = T + rng.normal(0, 0.05, size=T.shape) if frozen else T
    dt = 300.0
    sch = (hor, "PPM", lim, 0.7, 0.6)
    vals, vab = np.ascontiguousarray(T.copy()), np.ascontiguousarray(TA.copy())
    O.analytic_step(om, O.Work(om), dt, vel, w, vals, vab, [sch] * K, copy_ab=not frozen)
    out = {}
    from fesom2_tracer_dwarf_gb300 import _lib

    for tiled in (0, 1):
        eng = engine.TracerAdvection(m, K, "fp32", *sch[:3], ph=0.7, pv=0.6, copy_ab=not frozen, tracer_vec=V)
        eng.set_launch([0] * 9 + [tiled])
        eng.set_tracers(T, TA if frozen else None)
        eng.set_velocity(vel, w)
        eng.step(dt, stages=_lib.STAGE_VFLUX | _lib.STAGE_HFLUX)
        torch.cuda.synchronize()
        out[tiled] = eng.workspace_view("adfh").cpu().numpy()
        eng.step(dt, stages=_lib.STAGE_ALL & ~(_lib.STAGE_VFLUX | _lib.STAGE_HFLUX))
        torch.cuda.synchronize()
        assert _rel(eng.values(), vals) <= REL_TOL
    assert np.allclose(out[1], out[0], rtol=1e-6, atol=1e-6 * np.abs(out[0]).max())


def test_fp32_anomaly_storage(pkg, oracle_mod):
    """Anomaly storage (offsets): with a continuity-consistent flow the stored
    anomalies advance like the full values, and FP32 error against the FP64
    oracle drops; zero offsets change nothing; stats add the offsets back."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    om, m = _pair(O, mesh_mod, **_ragged(14, 12, 14, seed=8))
    rng = np.random.default_rng(70)
    dt = 300.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4, psi_wall_zero=True)
    K = 4
    # (values stay below 1000: the FCT bound of dry elements is +-1e3, lib/oce_adv_tra_fct.F90:81,142-143)
    T = synthetic.random_field(m, rng, K) * 0.03 + np.array([35.0, 20.0, 500.0, 0.5])[:, None, None]
    sch = ("MUSCL", "PPM", "FCT")
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    for _ in range(20):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * K, copy_ab=True)
    errs = {}
    for off in (None, "mean", np.zeros(K)):
        eng = engine.TracerAdvection(m, K, "fp32", *sch, copy_ab=True, offsets=off)
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
        eng.step(dt, 20)
        torch.cuda.synchronize()
        got = eng.values()
        key = "zero" if isinstance(off, np.ndarray) else str(off)
        errs[key] = np.abs(got - vals).reshape(K, -1).max(axis=1) / np.abs(vals).reshape(K, -1).max(axis=1)
        if key == "zero":
            assert np.array_equal(got, plain)
        if key == "None":
            plain = got
        st = eng.stats()
        assert np.allclose(st[:, 0], got.reshape(K, -1).min(axis=1)) and np.allclose(st[:, 1], got.reshape(K, -1).max(axis=1))
        assert np.allclose(st[:, 2], got.reshape(K, -1).sum(axis=1), rtol=1e-10)
    assert np.all(errs["mean"] <= 1e-6), errs
    assert np.all(errs["mean"][:3] < 0.2 * errs["None"][:3]), errs


def test_run_host_batches(pkg, oracle_mod):
    """run_host: independent batches from host memory, copies overlapped with
    the steps, give what stepping each batch on its own gives."""
    mesh_mod, engine, synthetic = pkg
    m = mesh_mod.Mesh(**MESHES["periodic"])
    rng = np.random.default_rng(80)
    vel, w = synthetic.random_flow(m, rng)
    eng = engine.TracerAdvection(m, 4, "fp32", "MUSCL", "PPM", "FCT", copy_ab=True)
    eng.set_velocity(vel, w)
    fields = [synthetic.random_field(m, rng, 4) for _ in range(5)]
    expect = []
    for f in fields:
        eng.set_tracers(f)
        eng.step(300.0, 2)
        expect.append(eng.T.cpu().clone())
    host_in = []
    for f in fields:
        eng.set_tracers(f)
        host_in.append(eng.T.cpu().pin_memory())
    host_out = [torch.empty_like(h).pin_memory() for h in host_in]
    eng.run_host(host_in, host_out, 300.0, nsteps=2)
    torch.cuda.synchronize()
    for got, exp in zip(host_out, expect):
        assert torch.equal(got, exp)


def test_run_host_batches_with_residual(pkg, oracle_mod):
    """run_host on an engine that keeps the FP32 rounding residual: batches
    given as (values, residuals) pairs come back as the pair that stepping
    each batch on the device gives, bit for bit; a batch given as one tensor
    starts with a zero residual."""
    mesh_mod, engine, synthetic = pkg
    m = mesh_mod.Mesh(**MESHES["periodic"])
    rng = np.random.default_rng(81)
    vel, w = synthetic.random_flow(m, rng)
    eng = engine.TracerAdvection(m, 4, "fp32", "MUSCL", "PPM", "FCT", copy_ab=True, residual=True)
    eng.set_velocity(vel, w)
    fields = [synthetic.random_field(m, rng, 4) for _ in range(4)]
    expect, host_in = [], []
    for f in fields:
        eng.set_tracers(f)
        host_in.append((eng.T.cpu().pin_memory(), eng.Tlo.cpu().pin_memory()))
        eng.step(300.0, 2)
        expect.append((eng.T.cpu().clone(), eng.Tlo.cpu().clone()))
    assert any(float(lo.abs().max()) > 0 for _, lo in host_in)
    host_out = [(torch.empty_like(a).pin_memory(), torch.empty_like(b).pin_memory()) for a, b in host_in]
    eng.run_host(host_in, host_out, 300.0, nsteps=2)
    torch.cuda.synchronize()
    for (gt, gl), (et, el) in zip(host_out, expect):
        assert torch.equal(gt, et) and torch.equal(gl, el)
    # one tensor: the values alone, residual zero at the start of the batch
    eng.set_tracers(fields[0])
    vals = eng.T.cpu().pin_memory()
    eng.Tlo.zero_()
    eng.step(300.0)
    exp = eng.T.cpu().clone()
    out = torch.empty_like(vals).pin_memory()
    eng.run_host([vals], [out], 300.0)
    torch.cuda.synchronize()
    assert torch.equal(out, exp)
