"""Edge cases of the step: the smallest analytic meshes (boundary edges without
triangles, every node on a wall), one-layer columns (UPW1 / CDIFF; QR4C and PPM
are refused), a single tracer, and the statistics with NaN values (min and max
skip NaN, the sum turns NaN, as src/fesom_analytic.F90:441-445 computes them).
"""
import itertools
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

SMALLEST = {
    "closed_2x2": dict(nx=2, ny=2, nl=3, periodic=False),
    "periodic_3x3": dict(nx=3, ny=3, nl=3, periodic=True),
}


def _one_layer_kw(nx=9, ny=8, nl=6):
    from fesom2_tracer_dwarf_gb300 import synthetic

    zb = synthetic.stretched_zbar(nl - 1, 5.0, 120.0)
    en = np.full(2 * (nx - 1) * (ny - 1), nl, dtype=np.int32)
    en[:20] = 2  # one-layer elements: their nodes' columns have one layer
    return dict(nx=nx, ny=ny, nl=nl, periodic=False, zbar=zb, elem_nlev=en)


def test_oracle_stats_with_nan(oracle_mod):
    om = oracle_mod.Mesh(5, 5, 4, periodic=False)
    v = np.arange(om.nod2D * (om.nl - 1), dtype=np.float64).reshape(om.nod2D, om.nl - 1) + 1.0
    v[2, 1] = np.nan
    mn, mx, sm, nan = om.stats(v)
    assert mn == 1.0 and mx == v.size and np.isnan(sm) and nan == 1


def test_anomaly_offsets_rule():
    """offsets="auto": the mean only where it shrinks the stored magnitude at
    least fourfold; fields touching zero keep offset 0 (exact zeros)."""
    from fesom2_tracer_dwarf_gb300.engine import anomaly_offsets

    rng = np.random.default_rng(5)
    S = 35.0 + 0.3 * rng.standard_normal((6, 5))
    blob = np.zeros((6, 5))
    blob[2:4, 1:3] = 1.0
    T = 10.0 + 8.0 * rng.standard_normal((6, 5))  # spread comparable to the values
    v = np.stack([S, blob, T])
    mean = anomaly_offsets(v, 3, "mean")
    assert np.allclose(mean, v.reshape(3, -1).mean(axis=1))
    auto = anomaly_offsets(v, 3, "auto")
    assert auto[0] == mean[0] and auto[1] == 0.0 and auto[2] == 0.0


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.mark.gpu
@pytest.mark.parametrize("meshname", ["closed_2x2", "periodic_3x3", "one_layer"])
@pytest.mark.parametrize("hor,ver,lim", list(itertools.product(["UPW1", "MUSCL", "MFCT"], ["UPW1", "CDIFF"],
                                                                ["NONE", "FCT"])))
def test_small_and_one_layer_meshes(oracle_mod, meshname, hor, ver, lim):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    O = oracle_mod
    kw = _one_layer_kw() if meshname == "one_layer" else SMALLEST[meshname]
    om, m = O.Mesh(**kw), Mesh(**kw)
    rng = np.random.default_rng(zlib.crc32(f"edge/{meshname}/{hor}/{ver}/{lim}".encode()))
    vel, w = synthetic.random_flow(m, rng)
    T = synthetic.random_field(m, rng, 2)
    dt = 300.0
    sch = (hor, ver, lim, 0.7, 0.6)
    vals, vab = np.ascontiguousarray(T.copy()), np.ascontiguousarray(T.copy())
    W = O.Work(om)
    for _ in range(3):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * 2, copy_ab=True)
    for precision in ("fp64", "fp32"):
        eng = engine.TracerAdvection(m, 2, precision, hor, ver, lim, ph=0.7, pv=0.6, copy_ab=True)
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
        eng.step(dt, 3)
        torch.cuda.synchronize()
        got = eng.values()
        if precision == "fp64":
            assert np.array_equal(got, vals), f"max |diff| {np.abs(got - vals).max()}"
        else:
            assert np.abs(got - vals).max() <= 1e-5 * max(1.0, np.abs(vals).max())


@pytest.mark.gpu
@pytest.mark.parametrize("ver", ["QR4C", "PPM"])
def test_one_layer_columns_refused_by_qr4c_ppm(ver):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(**_one_layer_kw())
    rng = np.random.default_rng(3)
    vel, w = synthetic.random_flow(m, rng)
    for precision in ("fp64", "fp32"):
        eng = engine.TracerAdvection(m, 1, precision, "UPW1", ver, "FCT")
        eng.set_tracers(synthetic.random_field(m, rng, 1))
        eng.set_velocity(vel, w)
        with pytest.raises(RuntimeError, match="two layers"):
            eng.step(300.0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,V", [("fp64", 1), ("fp32", 4), ("fp32", 1)])
def test_stats_with_nan(oracle_mod, precision, V):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    kw = dict(nx=9, ny=8, nl=6, periodic=True)
    om, m = oracle_mod.Mesh(**kw), Mesh(**kw)
    T = synthetic.random_field(m, np.random.default_rng(4), 4)
    T[1, 3, 2] = np.nan
    T[1, 7, 0] = np.nan
    eng = engine.TracerAdvection(m, 4, precision, tracer_vec=V)
    eng.set_tracers(T)
    st = eng.stats()
    for t in range(4):
        ref = om.stats(np.ascontiguousarray(eng.values()[t]))
        assert st[t, 0] == ref[0] and st[t, 1] == ref[1] and st[t, 3] == ref[3]
        if t == 1:
            assert np.isnan(st[t, 2]) and st[t, 3] == 2
        else:
            assert abs(st[t, 2] - ref[2]) <= 1e-12 * abs(ref[2])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,V,residual", [("fp64", 1, False), ("fp32", 4, True), ("fp32", 2, False)])
def test_input_check_names_non_finite_arrays(precision, V, residual):
    """fgb_check_inputs (engine.check_inputs): one device reduction per
    array; every array finite -> [], a NaN or an infinity planted in one
    input -> that array's name only. NaN and Inf are data, not faults: the
    step itself would carry them through, as the reference's does."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(14, 12, 9, periodic=True, orient_left=True)
    rng = np.random.default_rng(17)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4)
    T = synthetic.random_field(m, rng, 4)
    kw = dict(tracer_vec=V, residual=residual) if precision == "fp32" else {}
    e = engine.TracerAdvection(m, 4, precision, "MUSCL", "PPM", "FCT", copy_ab=True, **kw)
    e.set_tracers(T)
    e.set_velocity(vel, w)
    assert e.check_inputs() == []
    for field, bad in (("T", np.nan), ("vel", np.inf), ("w", -np.inf)):
        if field == "T":
            T2 = T.copy()
            T2[3, 5, 2] = bad  # the last tracer of the last group
            e.set_tracers(T2)
        elif field == "vel":
            v2 = vel.copy()
            v2[7, 1, 0] = bad
            e.set_velocity(v2, w)
        else:
            w2 = w.copy()
            w2[4, 3] = bad
            e.set_velocity(vel, w2)
        # a NaN value set with the residual kept also makes its residual NaN (value - float(value))
        want = ["T", "Tlo"] if (field == "T" and residual) else [field]
        assert e.check_inputs() == want, field
        e.set_tracers(T)
        e.set_velocity(vel, w)
        assert e.check_inputs() == []
    if residual:
        e.Tlo.view(-1)[123] = float("nan")
        assert e.check_inputs() == ["Tlo"]
    # a separate valuesAB array (frozen AB level) is checked as well
    f = engine.TracerAdvection(m, 4, precision, "MUSCL", "PPM", "FCT", **kw)
    T2 = T.copy()
    T2[0, 1, 1] = np.nan
    f.set_tracers(T2)
    f.set_velocity(vel, w)
    assert f.check_inputs() == (["T", "TA", "Tlo"] if residual else ["T", "TA"])


@pytest.mark.gpu
def test_cabi_input_checks_refuse_non_finite_values():
    """tracer_set_input_checks(1): tracer_advect_step returns -1 and names
    the array instead of stepping; off (the reference's behaviour) the step
    runs and the NaN propagates."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300.demo_tracer import FESOMTracerAdvection

    t = FESOMTracerAdvection(verbose=False)
    t.cleanup()
    try:
        assert t.generate_analytic_mesh(10, 9, 6, periodic=True) == 0
        nz, N = 5, t.nod2D
        assert t.allocate_tracers(1, 6, N) == 0
        v = np.asfortranarray(np.ones((nz, N)))
        v[2, 7] = np.nan
        assert t.set_values(1, v) == 0
        assert t.set_velocity_zero() == 0
        assert t.init_for_advection() == 0 and t.init_complete() == 0
        assert t.set_input_checks(True) == 0
        assert t.advect_step(10.0) == -1
        assert "values" in t.lib.fgb_last_error().decode()
        assert t.set_input_checks(False) == 0
        assert t.advect_step(10.0) == 0
        assert np.isnan(t.get_tracer_values()[2, 7])
    finally:
        t.cleanup()


@pytest.mark.gpu
def test_stats_sum_is_compensated():
    """The statistics' sum is a compensated FP64 sum: on values 1e10 + u,
    u in [0, 1), whose plain running sum loses about 1e-10 of its value, it
    agrees with the exactly rounded sum (math.fsum) to a few units in the
    last place; an infinite value gives an infinite sum, a NaN a NaN sum."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import math

    from fesom2_tracer_dwarf_gb300 import engine
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    m = Mesh(130, 130, 33, periodic=True)
    rng = np.random.default_rng(23)
    T = 1e10 + rng.random((2, m.N, m.nz))
    eng = engine.TracerAdvection(m, 2, "fp64")
    eng.set_tracers(T)
    st = eng.stats()
    for t in range(2):
        exact = math.fsum(T[t].ravel())
        assert abs(st[t, 2] - exact) <= 4 * math.ulp(exact), (st[t, 2], exact)
    T[0, 5, 3] = np.inf
    T[1, 9, 1] = np.nan
    eng.set_tracers(T)
    st = eng.stats()
    assert st[0, 2] == np.inf and np.isnan(st[1, 2]) and st[1, 3] == 1
