"""GPU step against the CPU oracle (FP64 form: bit-exact).

Every scheme combination of do_oce_adv_tra (lib/oce_adv_tra_driver.F90:23-294)
on periodic, closed-wall and ragged meshes, single steps with intermediate
arrays and multi-step runs. The FP64 kernels are compiled without fused
multiply-add and keep the reference's evaluation order, so the bar is exact
equality; `TOL` only guards the reporting.
"""
import itertools
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 0.0  # bit-exact


@pytest.fixture(scope="module")
def pkg():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import engine, mesh, synthetic

    return mesh, engine, synthetic


def _pair(O, mesh_mod, nx, ny, nl, periodic, cluster_full=False, zbar=None, elem_nlev=None, orient_left=False):
    kw = dict(periodic=periodic, cluster_full=cluster_full, zbar=zbar, elem_nlev=elem_nlev, orient_left=orient_left)
    return O.Mesh(nx, ny, nl, **kw), mesh_mod.Mesh(nx, ny, nl, **kw)


MESHES = {
    "periodic": dict(nx=11, ny=9, nl=8, periodic=True),
    "periodic_full": dict(nx=9, ny=10, nl=7, periodic=True, cluster_full=True),
    "closed": dict(nx=10, ny=8, nl=9, periodic=False),
    "closed_left": dict(nx=10, ny=8, nl=9, periodic=False, orient_left=True),
}


def _ragged(nx=12, ny=10, nl=12, seed=3, orient_left=True):
    from fesom2_tracer_dwarf_gb300 import synthetic

    rng = np.random.default_rng(seed)
    zb = synthetic.stretched_zbar(nl - 1, 5.0, 120.0)
    en = synthetic.bathymetry_levels(nx, ny, zb, rng, min_layers=3)
    return dict(nx=nx, ny=ny, nl=nl, periodic=False, zbar=zb, elem_nlev=en, orient_left=orient_left)


def _max_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) if np.size(a) else 0.0


@pytest.mark.parametrize("meshname", ["periodic", "periodic_full", "closed", "closed_left", "ragged"])
@pytest.mark.parametrize("hor,ver,lim", list(itertools.product(["UPW1", "MUSCL", "MFCT"],
                                                                ["UPW1", "QR4C", "CDIFF", "PPM"],
                                                                ["NONE", "FCT"])))
def test_single_step_all_schemes(pkg, oracle_mod, meshname, hor, ver, lim):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    kw = _ragged() if meshname == "ragged" else MESHES[meshname]
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(zlib.crc32(f"{meshname}/{hor}/{ver}/{lim}".encode()))
    vel, w = synthetic.random_flow(m, rng)
    K = 2
    T = synthetic.random_field(m, rng, K)
    TA = T + rng.normal(0, 0.05, size=T.shape)
    dt = 400.0
    vals = np.ascontiguousarray(T.copy())
    vab = np.ascontiguousarray(TA.copy())
    W = O.Work(om)
    O.analytic_step(om, W, dt, vel, w, vals, vab, [(hor, ver, lim, 0.7, 0.6)] * K)
    eng = engine.TracerAdvection(m, K, "fp64", hor, ver, lim, ph=0.7, pv=0.6)
    eng.set_tracers(T, TA)
    eng.set_velocity(vel, w)
    eng.step(dt)
    torch.cuda.synchronize()
    err = _max_err(eng.values(), vals)
    assert err <= TOL, f"{meshname} {hor}/{ver}/{lim}: max |GPU - oracle| = {err}"


@pytest.mark.parametrize("hor,ver", [("MUSCL", "QR4C"), ("MUSCL", "PPM"), ("UPW1", "UPW1")])
def test_fct_intermediates(pkg, oracle_mod, hor, ver):
    """LO solution, antidiffusive fluxes and limiting factors of one tracer."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    om, m = _pair(O, mesh_mod, **MESHES["periodic"])
    rng = np.random.default_rng(11)
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, 1)
    dt = 300.0
    W = O.Work(om)
    O.do_oce_adv_tra(om, W, dt, vel, w, T[0], T[0], hor, ver, "FCT")
    eng = engine.TracerAdvection(m, 1, "fp64", hor, ver, "FCT")
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    from fesom2_tracer_dwarf_gb300 import _lib

    eng.step(dt, stages=_lib.STAGE_VFLUX | _lib.STAGE_HFLUX | _lib.STAGE_LO | _lib.STAGE_RATIO)
    torch.cuda.synchronize()
    nz, nl = m.nz, m.nl
    lo = eng.workspace_view("lo")[0, :, :nz].cpu().numpy()
    assert _max_err(lo, W.get("fct_LO")) <= TOL
    adfh = eng.workspace_view("adfh")[0, :, :nz].cpu().numpy()
    assert _max_err(adfh, W.get("adf_h_raw")) <= TOL
    adfv = eng.workspace_view("adfv")[0, :, :nl].cpu().numpy()
    assert _max_err(adfv, W.get("adf_v_raw")) <= TOL
    nlev = m.get("nlevels_nod2D")
    mask = np.arange(nz)[None, :] < (nlev - 1)[:, None]
    rp = eng.workspace_view("rp")[0, :, :nz].cpu().numpy()
    rm = eng.workspace_view("rm")[0, :, :nz].cpu().numpy()
    assert _max_err(rp[mask], W.get("fct_plus")[mask]) <= TOL
    assert _max_err(rm[mask], W.get("fct_minus")[mask]) <= TOL


@pytest.mark.parametrize("case", ["periodic_muscl_qr4c", "ragged_muscl_ppm", "closed_upw1_fct"])
def test_multistep(pkg, oracle_mod, case):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    if case == "periodic_muscl_qr4c":
        kw, sch = dict(MESHES["periodic"], orient_left=True), ("MUSCL", "QR4C", "FCT")
    elif case == "ragged_muscl_ppm":
        kw, sch = _ragged(), ("MUSCL", "PPM", "FCT")
    else:
        kw, sch = MESHES["closed_left"], ("UPW1", "UPW1", "FCT")
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(5)
    dt = 300.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4, psi_wall_zero=True)
    K = 3
    T = synthetic.random_field(m, rng, K)
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    eng = engine.TracerAdvection(m, K, "fp64", *sch, copy_ab=True)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    for _ in range(10):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * K, copy_ab=True)
        eng.step(dt)
    torch.cuda.synchronize()
    assert _max_err(eng.values(), vals) <= TOL


def test_dwarf_golden_on_gpu(pkg, oracle_mod):
    """The analytic dwarf on the GPU prints the reference README.md:51-52 lines."""
    mesh_mod, engine, synthetic = pkg
    from tests.test_oracle import GOLDEN, fortran_e

    m = mesh_mod.Mesh(20, 20, 10, periodic=True)
    om = oracle_mod.Mesh(20, 20, 10, periodic=True)
    T, S = om.dwarf_fields()
    vel, w = synthetic.dwarf_velocity(m)
    eng = engine.TracerAdvection(m, 2, "fp64")
    eng.set_tracers(np.stack([T, S]))
    eng.set_velocity(vel, w)
    for step in (1, 2):
        eng.step(1000.0)
        st = eng.stats()[0]
        gmin, gmax, gsum = GOLDEN[step]
        assert fortran_e(st[0], 6) == gmin and fortran_e(st[1], 6) == gmax and fortran_e(st[2], 10) == gsum
        assert st[3] == 0


def test_fp32_form_close(pkg, oracle_mod):
    """FP32 storage and arithmetic: relative max-norm error against FP64 after 20 steps."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    om, m = _pair(O, mesh_mod, **dict(MESHES["periodic"], orient_left=True))
    rng = np.random.default_rng(9)
    dt = 300.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4)
    T = synthetic.random_field(m, rng, 2)
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    eng = engine.TracerAdvection(m, 2, "fp32", "MUSCL", "QR4C", "FCT", copy_ab=True)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    for _ in range(20):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [("MUSCL", "QR4C", "FCT")] * 2, copy_ab=True)
        eng.step(dt)
    torch.cuda.synchronize()
    rel = _max_err(eng.values(), vals) / float(np.max(np.abs(vals)))
    assert rel <= 1e-5, rel


FAST64_TOL = 1e-12  # relative max-norm of the fast FP64 form against the oracle


@pytest.mark.parametrize("meshname", ["periodic", "closed_left", "ragged"])
@pytest.mark.parametrize("hor,ver,lim", list(itertools.product(["UPW1", "MUSCL", "MFCT"],
                                                                ["UPW1", "QR4C", "CDIFF", "PPM"],
                                                                ["NONE", "FCT"])))
def test_fast_fp64_within_1e12(pkg, oracle_mod, meshname, hor, ver, lim):
    """The fast FP64 form (fused multiply-add, reciprocal products) over five
    steps with copy-AB, against the oracle: relative max-norm <= 1e-12."""
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    kw = _ragged() if meshname == "ragged" else MESHES[meshname]
    om, m = _pair(O, mesh_mod, **kw)
    rng = np.random.default_rng(zlib.crc32(f"fast/{meshname}/{hor}/{ver}/{lim}".encode()))
    vel, w = synthetic.random_flow(m, rng)
    K = 2
    T = synthetic.random_field(m, rng, K)
    dt, steps = 400.0, 5
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    for _ in range(steps):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [(hor, ver, lim, 0.7, 0.6)] * K, copy_ab=True)
    eng = engine.TracerAdvection(m, K, "fp64fast", hor, ver, lim, ph=0.7, pv=0.6, copy_ab=True)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    eng.step(dt, steps)
    torch.cuda.synchronize()
    nlev = m.get("nlevels_nod2D")
    wet = np.arange(m.nz)[None, :] < (nlev - 1)[:, None]
    got = eng.values()
    rel = max(float(np.abs(got[t] - vals[t])[wet].max() / np.abs(vals[t][wet]).max()) for t in range(K))
    assert rel <= FAST64_TOL, f"{meshname} {hor}/{ver}/{lim}: fast FP64 relative error {rel:.3g}"


def test_fp64_probe_rates(pkg):
    """fgb_probe_fp64: the FP64 FMA and division rates of the device, the
    bound of the FP64 forms. GB300's FP64 units give about 1.2 TFLOP/s of
    FMA; the bounds only reject a probe that did not run or did no work."""
    from fesom2_tracer_dwarf_gb300 import _lib

    r = _lib.probe_fp64()
    assert 0.05 < r["fma_tflops"] < 200.0, r
    assert 0.5 < r["div_g_per_s"] < 20000.0, r
    assert r["ms"] > 0.0
