"""fgb_adv_step_static: the step entry point for callers that cannot allocate
device memory (their framework owns the GPU memory through its own pool), whose
scratch is a fixed device array inside the library.

Checked through the C-ABI against fgb_adv_step with a caller-provided
workspace, on two calls in a row (the second reuses the array the first one
left behind). The FP64 form is bit-exact, so the tolerance is exact equality,
as in the other GPU tests. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import _lib

    return _lib


def _engine(mesh, synthetic, engine, T, vel, w):
    e = engine.TracerAdvection(mesh, T.shape[0], "fp64", "MUSCL", "QR4C", "FCT", copy_ab=True)
    e.set_tracers(T)
    e.set_velocity(vel, w)
    return e


def test_static_workspace_matches_caller_workspace(lib):
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    L = lib.load()
    m = Mesh(24, 20, 10, periodic=True, orient_left=True)
    rng = np.random.default_rng(4)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4)
    T = synthetic.random_field(m, rng, 2)
    ref = _engine(m, synthetic, engine, T, vel, w)
    sta = _engine(m, synthetic, engine, T, vel, w)
    need = L.fgb_workspace_bytes(m.handle, lib.FP64, 2)
    assert 0 < need <= L.fgb_static_workspace_bytes()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        ref.step(300.0)
        d = sta._desc(300.0)
        d.workspace = None  # ignored by the static entry point
        d.workspace_bytes = 0
        rc = L.fgb_adv_step_static(m.handle, ctypes.byref(d), stream)
        assert rc == 0, lib.last_error()
        torch.cuda.synchronize()
        diff = float(np.abs(sta.values() - ref.values()).max())
        assert diff == 0.0, f"call {call + 1}: max |static - workspace| = {diff}"


def test_static_workspace_fp32_groups_and_tiled_edges(lib):
    """The FP32 form through the static array: four tracers in one group
    (16-byte loads from the array) and the tiled edge kernel (cfg[9] = 1),
    which runs only when the workspace is 16-byte aligned. Both paths run the
    same kernels, so the results must be equal bit for bit."""
    from fesom2_tracer_dwarf_gb300 import engine, synthetic
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    L = lib.load()
    m = Mesh(24, 20, 10, periodic=True, orient_left=True)
    rng = np.random.default_rng(5)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4)
    T = synthetic.random_field(m, rng, 4)

    def make():
        e = engine.TracerAdvection(m, 4, "fp32", "MUSCL", "PPM", "FCT", copy_ab=True, tracer_vec=4)
        e.set_launch([0] * 9 + [1])
        e.set_tracers(T)
        e.set_velocity(vel, w)
        return e

    ref, sta = make(), make()
    assert ref.V == 4
    assert 0 < L.fgb_workspace_bytes(m.handle, lib.FP32, 4) <= L.fgb_static_workspace_bytes()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        ref.step(300.0)
        d = sta._desc(300.0)
        assert d.cfg[9] == 1 and d.tracer_vec == 4
        d.workspace = None
        d.workspace_bytes = 0
        rc = L.fgb_adv_step_static(m.handle, ctypes.byref(d), stream)
        assert rc == 0, lib.last_error()
        torch.cuda.synchronize()
        diff = float(np.abs(sta.values() - ref.values()).max())
        assert diff == 0.0, f"call {call + 1}: max |static - workspace| = {diff}"


def test_static_workspace_rejects_large_meshes(lib):
    from fesom2_tracer_dwarf_gb300 import engine
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    L = lib.load()
    m = Mesh(300, 300, 40, periodic=True)
    assert L.fgb_workspace_bytes(m.handle, lib.FP64, 1) > L.fgb_static_workspace_bytes()
    e = engine.TracerAdvection(m, 1, "fp64", "UPW1", "UPW1", "FCT", copy_ab=True)
    d = e._desc(100.0)
    rc = L.fgb_adv_step_static(m.handle, ctypes.byref(d), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -1
    assert "static workspace" in lib.last_error()
