"""The reference's C interface (lib/tracer_c_interface.F90) as exported by
libfesom_tracer_gb300.so, driven through the reference-style ctypes wrapper.

CPU tests cover the status codes and call-order behaviour that need no device;
GPU tests run the array-initialisation sequence of the reference's Python
scripts and compare with the oracle's tracer_advect_step semantics
(lib/tracer_c_interface.F90:163-220: tracer 1 only, del_ttf accumulating,
w_e = 0, valuesAB frozen, uv read as vel(2,nl-1,elem2D)).
"""
import os

import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300.demo_tracer import FESOMTracerAdvection


@pytest.fixture()
def tracer():
    t = FESOMTracerAdvection(verbose=False)
    t.cleanup()
    yield t
    t.cleanup()


def test_status_codes_before_initialisation(tracer, tmp_path):
    L = tracer.lib
    assert tracer.initialize_mpi(0) == 0
    assert tracer.finalize_mpi() == 0
    assert tracer.advect_step(1.0) == -1                       # :168-173
    with pytest.raises(RuntimeError):
        tracer.get_statistics()                                # :233-241
    with pytest.raises(RuntimeError):
        tracer.get_tracer_values()
    assert tracer.initialize(str(tmp_path / "missing")) == -1  # :136-141
    os.makedirs(tmp_path / "np1")
    assert tracer.initialize(str(tmp_path)) == -1              # no restart files in it
    assert L.tracer_load_mesh_from_files(b"/nonexistent/") == -1
    assert tracer.finalize(str(tmp_path)) == -1
    assert L.tracer_run_workflow(str(tmp_path / "missing").encode(), 3, 1.0) == -1


def test_array_initialisation_sequence_host_side(tracer):
    assert tracer.generate_analytic_mesh(12, 10, 8, periodic=True) == 0
    import ctypes

    nz, nn = ctypes.c_int(), ctypes.c_int()
    assert tracer.lib.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn)) == 0
    assert (nz.value, nn.value) == (7, 11 * 9)
    assert tracer.allocate_tracers(2, 8, nn.value) == 0
    assert tracer.set_values(3, np.zeros((7, nn.value), order="F")) == -1  # :623-628
    assert tracer.set_values(1, np.ones((7, nn.value), order="F")) == 0
    assert tracer.set_schemes(1, "MUSCL", "QR4C", "FCT") == 0
    assert tracer.set_schemes(1, "WENO", "QR4C", "FCT") == -1
    assert tracer.set_precision("fp32") == 0


torch = pytest.importorskip("torch")


def _reference_layout_uv(vel, nz, edge2D):
    """A (nl-1, edge2D, 2) Fortran array whose memory starts with vel(2,nl-1,elem2D)."""
    buf = np.zeros(nz * edge2D * 2)
    flat = np.ascontiguousarray(vel).reshape(-1)  # (M, nz, 2) C order == vel(2, nz, M) Fortran order
    buf[: flat.size] = flat
    return buf.reshape((nz, edge2D, 2), order="F")


@pytest.mark.gpu
@pytest.mark.parametrize("schemes", [("UPW1", "UPW1", "NONE"), ("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT")])
def test_cabi_steps_match_oracle(tracer, oracle_mod, schemes):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    O = oracle_mod
    nx, ny, nl = 14, 12, 9
    assert tracer.generate_analytic_mesh(nx, ny, nl, periodic=True) == 0
    om = O.Mesh(nx, ny, nl, periodic=True)
    hm = Mesh(nx, ny, nl, periodic=True, upload=False)
    rng = np.random.default_rng(21)
    vel, w = synthetic.random_flow(hm, rng)
    T = synthetic.random_field(hm, rng, 1)[0]          # (N, nz)
    nz, N, E = nl - 1, hm.N, hm.E
    assert tracer.allocate_tracers(2, nl, N) == 0
    assert tracer.set_values(1, np.asfortranarray(T.T)) == 0
    assert tracer.set_values(2, np.asfortranarray(T.T + 1.0)) == 0
    assert tracer.set_velocity(_reference_layout_uv(vel, nz, E), np.asfortranarray(w.T)) == 0
    assert tracer.set_schemes(1, *schemes) == 0
    assert tracer.init_ale_arrays() == 0
    assert tracer.init_for_advection() == 0
    assert tracer.init_complete() == 0
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    del_ttf = np.zeros_like(vals)
    W = O.Work(om)
    for step in range(3):
        assert tracer.advect_step(600.0) == 0
        O.cabi_step(om, W, 600.0, vel, w, vals, vab, del_ttf, *schemes)
        got = tracer.get_tracer_values()               # (nz, nn)
        err = float(np.abs(got.T - vals).max())
        assert err == 0.0, f"step {step + 1}: max |C-ABI - oracle| = {err}"
        st = tracer.get_statistics()
        assert st["min"] == vals.min() and st["max"] == vals.max()
        assert abs(st["sum"] - vals.sum()) <= 1e-12 * abs(vals.sum())


@pytest.mark.gpu
def test_cabi_fp32_form_close(tracer, oracle_mod):
    """tracer_set_precision(1): the FP32 form through the reference interface,
    del_ttf kept in single precision, within 1e-5 of the FP64 oracle."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    O = oracle_mod
    nx, ny, nl = 14, 12, 9
    assert tracer.generate_analytic_mesh(nx, ny, nl, periodic=True) == 0
    om = O.Mesh(nx, ny, nl, periodic=True)
    hm = Mesh(nx, ny, nl, periodic=True, upload=False)
    rng = np.random.default_rng(22)
    vel, w = synthetic.random_flow(hm, rng)
    T = synthetic.random_field(hm, rng, 1)[0]
    nz, N, E = nl - 1, hm.N, hm.E
    assert tracer.allocate_tracers(1, nl, N) == 0
    assert tracer.set_values(1, np.asfortranarray(T.T)) == 0
    assert tracer.set_velocity(_reference_layout_uv(vel, nz, E), np.asfortranarray(w.T)) == 0
    assert tracer.set_schemes(1, "MUSCL", "PPM", "FCT") == 0
    assert tracer.set_precision("fp32") == 0
    assert tracer.init_ale_arrays() == 0 and tracer.init_for_advection() == 0 and tracer.init_complete() == 0
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    del_ttf = np.zeros_like(vals)
    W = O.Work(om)
    for _ in range(3):
        assert tracer.advect_step(600.0) == 0
        O.cabi_step(om, W, 600.0, vel, w, vals, vab, del_ttf, "MUSCL", "PPM", "FCT")
    got = tracer.get_tracer_values()
    assert float(np.abs(got.T - vals).max()) <= 1e-5 * float(np.abs(vals).max())
