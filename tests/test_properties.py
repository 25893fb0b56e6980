"""Size-independent properties of the advection step, on the oracle (small
meshes, CPU) and on the GPU (up to the full benchmark meshes).

- a uniform tracer stays uniform under a discretely solenoidal flow (every
  scheme combination);
- zero velocity leaves the tracers unchanged, bit for bit;
- the volume integral sum(T * hnode_new * areasvol) over wet cells is
  conserved on closed-wall and ragged basins;
- FCT creates no new extrema under a solenoidal flow at CFL <= 0.5.

The FP32 form's bars, over 3-5 steps: the volume integral to 1e-9 (closed
basins) and 1e-10 (the 2048^2 mesh) with FP32 storage, to 1e-11 and 1e-13
when each value carries its FP32 rounding residual; within 2e-6 of the FP64
form in the max-norm; no excursion beyond 1e-6 of the initial range. (Largest
figures measured on a GB300: 2.2e-10, 1.1e-11, 1.4e-12, 2.1e-14, 3.4e-7.) The
sum is taken with FP64 volumes, which the FP32 kernels round: on the 129^2
basin that rounding alone is of order 1e-12.
"""
import itertools

import numpy as np
import pytest

SCHEMES = list(itertools.product(["UPW1", "MUSCL", "MFCT"], ["UPW1", "QR4C", "CDIFF", "PPM"], ["NONE", "FCT"]))


def _ragged_kw(nx=14, ny=12, nl=12, seed=3):
    from fesom2_tracer_dwarf_gb300 import synthetic

    rng = np.random.default_rng(seed)
    zb = synthetic.stretched_zbar(nl - 1, 5.0, 120.0)
    en = synthetic.bathymetry_levels(nx, ny, zb, rng, min_layers=3)
    return dict(nx=nx, ny=ny, nl=nl, periodic=False, zbar=zb, elem_nlev=en, orient_left=True)


def _wet(m):
    nlev = m.get("nlevels_nod2D")
    return np.arange(m.nz)[None, :] < (nlev - 1)[:, None]


def _volume(m):
    return m.get("areasvol")[:, : m.nz] * m.get("hnode_new") * _wet(m)


def _oracle_steps(O, om, vel, w, T, schemes, steps, dt):
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    for _ in range(steps):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [schemes] * vals.shape[0], copy_ab=True)
    return vals


# ---------------------------------------------------------------------------
# Oracle (CPU)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("hor,ver,lim", SCHEMES)
def test_oracle_uniform_stays_uniform(oracle_mod, hor, ver, lim):
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    kw = _ragged_kw()
    om, m = oracle_mod.Mesh(**kw), Mesh(**kw, upload=False)
    rng = np.random.default_rng(1)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4, psi_wall_zero=True)
    T = np.full((1, m.N, m.nz), 7.25)
    out = _oracle_steps(oracle_mod, om, vel, w, T, (hor, ver, lim), 3, 300.0)
    assert np.abs(out - 7.25)[:, _wet(m)].max() <= 1e-12 * 7.25


@pytest.mark.parametrize("hor,ver,lim", [("MUSCL", "PPM", "FCT"), ("MFCT", "QR4C", "NONE"), ("UPW1", "CDIFF", "FCT")])
def test_oracle_zero_velocity_identity(oracle_mod, hor, ver, lim):
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    kw = _ragged_kw()
    om, m = oracle_mod.Mesh(**kw), Mesh(**kw, upload=False)
    rng = np.random.default_rng(2)
    T = synthetic.random_field(m, rng, 2)
    vel = np.zeros((m.M, m.nz, 2))
    w = np.zeros((m.N, m.nl))
    out = _oracle_steps(oracle_mod, om, vel, w, T, (hor, ver, lim), 2, 300.0)
    assert np.array_equal(out, T)


@pytest.mark.parametrize("hor,ver,lim", [("MUSCL", "PPM", "FCT"), ("MUSCL", "QR4C", "FCT"), ("UPW1", "UPW1", "NONE"),
                                         ("MFCT", "CDIFF", "NONE")])
def test_oracle_conserves_volume_integral(oracle_mod, hor, ver, lim):
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    kw = _ragged_kw()
    om, m = oracle_mod.Mesh(**kw), Mesh(**kw, upload=False)
    rng = np.random.default_rng(3)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4, psi_wall_zero=True)
    T = synthetic.random_field(m, rng, 2)
    vol = _volume(m)
    before = (T * vol).sum(axis=(1, 2))
    out = _oracle_steps(oracle_mod, om, vel, w, T, (hor, ver, lim), 5, 300.0)
    after = (out * vol).sum(axis=(1, 2))
    assert np.all(np.abs(after - before) <= 1e-12 * np.abs(before))


@pytest.mark.parametrize("hor,ver", [("MUSCL", "PPM"), ("MFCT", "QR4C"), ("UPW1", "CDIFF")])
def test_oracle_fct_no_new_extrema(oracle_mod, hor, ver):
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    kw = _ragged_kw()
    om, m = oracle_mod.Mesh(**kw), Mesh(**kw, upload=False)
    rng = np.random.default_rng(4)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.5, psi_wall_zero=True)
    T = synthetic.random_field(m, rng, 2)
    wet = _wet(m)
    out = _oracle_steps(oracle_mod, om, vel, w, T, (hor, ver, "FCT"), 5, 300.0)
    for t in range(2):
        lo, hi = T[t][wet].min(), T[t][wet].max()
        assert out[t][wet].min() >= lo - 1e-12 * abs(lo) and out[t][wet].max() <= hi + 1e-12 * abs(hi)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
torch = pytest.importorskip("torch")


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _engine(m, K, precision, sch, vel, w, T):
    from fesom2_tracer_dwarf_gb300 import engine

    e = engine.TracerAdvection(m, K, precision, *sch, copy_ab=True)
    e.set_tracers(T)
    e.set_velocity(vel, w)
    return e


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("hor,ver,lim", SCHEMES)
def test_gpu_uniform_stays_uniform(precision, hor, ver, lim):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(**_ragged_kw(40, 36, 16, seed=5))
    rng = np.random.default_rng(6)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4, psi_wall_zero=True)
    T = np.full((4, m.N, m.nz), 7.25)
    e = _engine(m, 4, precision, (hor, ver, lim), vel, w, T)
    e.step(300.0, 5)
    tol = 1e-12 if precision == "fp64" else 5e-7
    assert np.abs(e.values() - 7.25)[:, _wet(m)].max() <= tol * 7.25


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_zero_velocity_identity(precision):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(**_ragged_kw(40, 36, 16, seed=7))
    rng = np.random.default_rng(8)
    T = synthetic.random_field(m, rng, 4)
    e = _engine(m, 4, precision, ("MUSCL", "PPM", "FCT"), np.zeros((m.M, m.nz, 2)), np.zeros((m.N, m.nl)), T)
    before = e.values()
    e.step(300.0, 3)
    assert np.array_equal(e.values(), before)


def _closed_basin(nx, nl, seed):
    """Closed ragged basin: seeded bathymetry, 8..nl-1 layers, walls."""
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    rng = np.random.default_rng(seed)
    zb = synthetic.stretched_zbar(nl - 1, 5.0, 250.0)
    en = synthetic.bathymetry_levels(nx, nx, zb, rng, min_layers=min(8, nl - 2))
    L = (nx - 1) * 1000.0
    return Mesh(nx, nx, nl, Lx=L, Ly=L, depth=-zb[-1], periodic=False, orient_left=True, zbar=zb, elem_nlev=en), rng


FP32_SUM_TOL = {"plain": 1e-9, "residual": 1e-11}


@pytest.mark.gpu
@pytest.mark.parametrize("nx,nl", [(129, 33), (1025, 65)])
@pytest.mark.parametrize("form", ["plain", "residual"])
def test_gpu_closed_basin_conservation_and_bounds(nx, nl, form):
    """Closed ragged basin (1025 grid points: the 1024^2 benchmark basin):
    FP64 conserves the volume integral to 1e-12 and FCT keeps every tracer in
    its initial range; the FP32 form (FP32 storage, or each value with its
    rounding residual) stays within 2e-6 of FP64, keeps the range to 1e-6 and
    conserves to 1e-9 (1e-11 with the residual)."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    m, rng = _closed_basin(nx, nl, 11)
    vel, w = synthetic.streamfunction_flow(m, rng, 400.0, cfl=0.4, psi_wall_zero=True)
    T = np.stack([synthetic.gaussian_T(m, rng), synthetic.salinity(m, rng)])
    vol = _volume(m)
    wet = _wet(m)
    before = (T * vol).sum(axis=(1, 2))
    sch = ("MUSCL", "PPM", "FCT")
    steps = 5
    e64 = _engine(m, 2, "fp64", sch, vel, w, T)
    e64.step(400.0, steps)
    v64 = e64.values()
    del e64
    e32 = engine.TracerAdvection(m, 2, "fp32", *sch, copy_ab=True, residual=form == "residual")
    assert e32.residual == (form == "residual")
    e32.set_tracers(T)
    e32.set_velocity(vel, w)
    e32.step(400.0, steps)
    v32 = e32.values()
    for t in range(2):
        a64 = (v64[t] * vol).sum()
        assert abs(a64 - before[t]) <= 1e-12 * abs(before[t])
        lo, hi = T[t][wet].min(), T[t][wet].max()
        assert v64[t][wet].min() >= lo - 1e-12 * abs(lo) and v64[t][wet].max() <= hi + 1e-12 * abs(hi)
        a32 = (v32[t] * vol).sum()
        rel = abs(a32 - before[t]) / abs(before[t])
        assert rel <= FP32_SUM_TOL[form], f"{form} tracer {t}: volume integral off by {rel:.3g}"
        assert np.abs(v32[t] - v64[t])[wet].max() <= 2e-6 * np.abs(v64[t]).max()
        assert v32[t][wet].min() >= lo - 1e-6 * abs(lo) and v32[t][wet].max() <= hi + 1e-6 * abs(hi)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "residual"])
def test_gpu_periodic_2048_fp32_properties(form):
    """The 2048^2 x 64-layer benchmark mesh, K = 4, MUSCL-FCT + PPM, FP32 form:
    uniform tracers stay uniform (5e-7), the volume integral of the others is
    conserved to 1e-10 (1e-13 with the rounding residual) and FCT creates no
    new extrema (1e-6 of the range)."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    zb = synthetic.stretched_zbar(64, 5.0, 250.0)
    m = Mesh(2049, 2049, 65, Lx=2048e3, Ly=2048e3, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb)
    rng = np.random.default_rng(12)
    vel, w = synthetic.flat_streamfunction_device(m, rng, 400.0, torch.float32, "cuda", cfl=0.4)
    T = synthetic.tracers_device(m, 4, 3, torch.float32, "cuda")
    T[3, :, : m.nz] = 7.25
    e = TracerAdvection(m, 4, "fp32", "MUSCL", "PPM", "FCT", copy_ab=True, residual=form == "residual")
    e.load_padded(T=T, vel=vel, w=w)
    vol = torch.as_tensor(m.get("areasvol")[:, : m.nz] * m.get("hnode_new"), device="cuda", dtype=torch.float64)
    Td = T[:, :, : m.nz].double()
    before = (Td * vol).sum(dim=(1, 2))
    mn, mx = Td.amin(dim=(1, 2)), Td.amax(dim=(1, 2))
    del Td
    e.step(400.0, 3)
    after_T = e.full_values()[:, :, : m.nz]
    after = (after_T * vol).sum(dim=(1, 2))
    rel = ((after - before).abs() / before.abs()).cpu().numpy()
    assert np.all(rel <= (1e-13 if form == "residual" else 1e-10)), rel
    amn, amx = after_T.amin(dim=(1, 2)), after_T.amax(dim=(1, 2))
    tol = 1e-6 * torch.maximum(mn.abs(), mx.abs())
    assert bool(torch.all(amn >= mn - tol)) and bool(torch.all(amx <= mx + tol))
    assert float((after_T[3] - 7.25).abs().max()) <= 5e-7 * 7.25
