"""Second-order Adams-Bashforth time level of valuesAB (the field the
high-order fluxes read): after each step valuesAB = -(0.5+eps) T_old +
(1.5+eps) T_new, FESOM2's tracer AB2 with the offset epsilon the reference
declares (lib/oce_modules.F90:75; valuesold, lib/tracer_c_interface.F90:561).

The oracle's driver loop is checked against the formula evaluated with numpy;
the GPU forms against the oracle over several steps (FP64 bit-exact, values and
valuesAB; FP32 within 1e-5 relative max-norm).
"""
import numpy as np
import pytest


def _ragged_kw(nx=12, ny=10, nl=12, seed=3):
    from fesom2_tracer_dwarf_gb300 import synthetic

    rng = np.random.default_rng(seed)
    zb = synthetic.stretched_zbar(nl - 1, 5.0, 120.0)
    en = synthetic.bathymetry_levels(nx, ny, zb, rng, min_layers=3)
    return dict(nx=nx, ny=ny, nl=nl, periodic=False, zbar=zb, elem_nlev=en, orient_left=True)


def _pair(O, kw):
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    return O.Mesh(**kw), Mesh(**kw, upload=False)


@pytest.mark.parametrize("eps", [0.1, 0.0])
def test_oracle_ab2_level(oracle_mod, eps):
    from fesom2_tracer_dwarf_gb300 import synthetic

    O = oracle_mod
    om, m = _pair(O, _ragged_kw())
    rng = np.random.default_rng(60)
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, 2)
    vals, vab = np.ascontiguousarray(T.copy()), np.ascontiguousarray(T.copy())
    W = O.Work(om)
    sch = [("MUSCL", "PPM", "FCT")] * 2
    for _ in range(3):
        old = vals.copy()
        O.analytic_step(om, W, 300.0, vel, w, vals, vab, sch, ab2_eps=eps)
        assert np.array_equal(vab, -(0.5 + eps) * old + (1.5 + eps) * vals)
    # the AB2 level changes the trajectory against copy-AB
    vals2, vab2 = np.ascontiguousarray(T.copy()), np.ascontiguousarray(T.copy())
    for _ in range(3):
        O.analytic_step(om, W, 300.0, vel, w, vals2, vab2, sch, copy_ab=True)
    assert not np.array_equal(vals, vals2)


torch = pytest.importorskip("torch")


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("sch", [("MUSCL", "PPM", "FCT"), ("UPW1", "QR4C", "NONE"), ("MFCT", "CDIFF", "FCT")])
def test_gpu_ab2_steps(oracle_mod, precision, sch):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    O = oracle_mod
    om, m = _pair(O, _ragged_kw(14, 12, 14, seed=7))
    rng = np.random.default_rng(61)
    dt = 300.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4, psi_wall_zero=True)
    K = 4
    T = synthetic.random_field(m, rng, K)
    vals, vab = np.ascontiguousarray(T.copy()), np.ascontiguousarray(T.copy())
    W = O.Work(om)
    eng = engine.TracerAdvection(m, K, precision, *sch, ab2_eps=0.1)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    for _ in range(5):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * K, ab2_eps=0.1)
        eng.step(dt)
    torch.cuda.synchronize()
    got = eng.values()
    got_ab = eng.from_layout(eng.TA)[:, :, : m.nz].double().cpu().numpy()
    if precision == "fp64":
        assert np.array_equal(got, vals)
        assert np.array_equal(got_ab, vab)
    else:
        assert _rel(got, vals) <= 1e-5
        assert _rel(got_ab, vab) <= 1e-5
