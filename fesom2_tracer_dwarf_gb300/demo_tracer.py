"""The reference dwarf's Python wrapper (python/demo_tracer.py:40-208) over
libfesom_tracer_gb300.so.

``FESOMTracerAdvection`` keeps the reference class's methods, argument types and
return conventions (status ints; ``get_tracer_values`` returns an (nz, nn)
Fortran-ordered array; ``get_statistics`` a dict), and adds the calls the
reference interface lacks for building a system from arrays: an analytic mesh,
scheme selection and the precision form.

    tracer = FESOMTracerAdvection()
    tracer.initialize_mpi(0)
    tracer.generate_analytic_mesh(20, 20, 10, periodic=True)
    tracer.allocate_tracers(2, 10, tracer.nod2D)
    tracer.set_values(1, T)                       # (nl-1, nod2D), Fortran order
    tracer.set_velocity(uv, w)                    # (nl-1, edge2D, 2), (nl, nod2D)
    tracer.init_ale_arrays(); tracer.init_for_advection(); tracer.init_complete()
    for _ in range(10):
        tracer.advect_step(1000.0)
        print(tracer.get_statistics())

A FESOM mesh directory (the reference's tests/data/pi, or a refinement of it
by ``meshfiles``) replaces the analytic mesh with
``tracer.load_mesh_from_files(path)`` (tracer_load_mesh_from_files).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_F64F = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class FESOMTracerAdvection:
    """Python wrapper of the tracer-advection library (reference-compatible)."""

    def __init__(self, verbose: bool = True):
        self.lib = _lib.load()
        L = self.lib
        sig = {
            "tracer_init_mpi": (ctypes.c_int, [ctypes.c_int]),
            "tracer_finalize_mpi": (ctypes.c_int, []),
            "tracer_init": (ctypes.c_int, [ctypes.c_char_p]),
            "tracer_advect_step": (ctypes.c_int, [ctypes.c_double]),
            "tracer_get_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)] * 3),
            "tracer_get_size": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)] * 2),
            "tracer_get_values": (ctypes.c_int, [_F64F, ctypes.c_int, ctypes.c_int]),
            "tracer_finalize": (ctypes.c_int, [ctypes.c_char_p]),
            "tracer_run_workflow": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_double]),
            "tracer_cleanup": (ctypes.c_int, []),
            "tracer_set_mesh_dims": (ctypes.c_int, [ctypes.c_int] * 4),
            "tracer_set_levels": (ctypes.c_int, [_I32, _I32, ctypes.c_int]),
            "tracer_set_thickness": (ctypes.c_int, [_F64F, ctypes.c_int, ctypes.c_int]),
            "tracer_set_partition": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
            "tracer_allocate_tracers": (ctypes.c_int, [ctypes.c_int] * 4),
            "tracer_set_values": (ctypes.c_int, [ctypes.c_int, _F64F, ctypes.c_int, ctypes.c_int]),
            "tracer_set_velocity_zero": (ctypes.c_int, [ctypes.c_int] * 3),
            "tracer_set_velocity": (ctypes.c_int, [_F64F, _F64F, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "tracer_init_complete": (ctypes.c_int, []),
            "tracer_load_mesh_partition": (ctypes.c_int, [ctypes.c_char_p]),
            "tracer_load_mesh_from_files": (ctypes.c_int, [ctypes.c_char_p]),
            "tracer_init_ale_arrays": (ctypes.c_int, []),
            "tracer_init_for_advection": (ctypes.c_int, []),
            "tracer_generate_analytic_mesh": (ctypes.c_int, [ctypes.c_int] * 4),
            "tracer_set_schemes": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                                  ctypes.c_char_p, ctypes.c_double, ctypes.c_double]),
            "tracer_set_precision": (ctypes.c_int, [ctypes.c_int]),
            "tracer_set_input_checks": (ctypes.c_int, [ctypes.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        self.nl = self.nod2D = self.edge2D = self.elem2D = 0
        if verbose:
            print(f"Loaded tracer library: {_lib._build.LIB_PATH}")

    # ---- the reference class's methods (python/demo_tracer.py:101-208) -----
    def initialize_mpi(self, mpi_comm=0):
        return self.lib.tracer_init_mpi(mpi_comm)

    def initialize(self, restart_path="./fesom_bin_restart"):
        return self.lib.tracer_init(restart_path.encode())

    def advect_step(self, dt=1.0e-3):
        return self.lib.tracer_advect_step(dt)

    def get_tracer_values(self):
        nz, nn = ctypes.c_int(), ctypes.c_int()
        ret = self.lib.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn))
        if ret != 0:
            raise RuntimeError(f"tracer_get_size failed with code {ret}")
        values = np.zeros((nz.value, nn.value), dtype=np.float64, order="F")
        ret = self.lib.tracer_get_values(values, nz, nn)
        if ret != 0:
            raise RuntimeError(f"tracer_get_values failed with code {ret}")
        return values

    def get_statistics(self):
        tmin, tmax, tsum = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        ret = self.lib.tracer_get_stats(ctypes.byref(tmin), ctypes.byref(tmax), ctypes.byref(tsum))
        if ret != 0:
            raise RuntimeError(f"tracer_get_stats failed with code {ret}")
        return {"min": tmin.value, "max": tmax.value, "sum": tsum.value}

    def finalize(self, output_path="./fesom_bin_restart"):
        return self.lib.tracer_finalize(output_path.encode())

    def finalize_mpi(self):
        return self.lib.tracer_finalize_mpi()

    # ---- building a system from arrays ---------------------------------------
    def generate_analytic_mesh(self, nx, ny, nl, periodic=True):
        rc = self.lib.tracer_generate_analytic_mesh(nx, ny, nl, int(periodic))
        if rc == 0:
            if periodic:
                self.nod2D, self.elem2D, self.edge2D = (nx - 1) * (ny - 1), 2 * (nx - 1) * (ny - 1), 3 * (nx - 1) * (ny - 1)
            else:
                self.nod2D, self.elem2D = nx * ny, 2 * (nx - 1) * (ny - 1)
                self.edge2D = (nx - 1) * ny + nx * (ny - 1) + (nx - 1) * (ny - 1)
            self.nl = nl
        return rc

    def load_mesh_from_files(self, mesh_path):
        """tracer_load_mesh_from_files: a FESOM mesh directory as one partition."""
        rc = self.lib.tracer_load_mesh_from_files(str(mesh_path).encode())
        if rc == 0:
            nz, nn = ctypes.c_int(), ctypes.c_int()
            self.lib.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn))
            self.nl, self.nod2D = nz.value + 1, nn.value
        return rc

    def set_mesh_dims(self, nl, nod2D, edge2D, elem2D):
        return self.lib.tracer_set_mesh_dims(nl, nod2D, edge2D, elem2D)

    def set_levels(self, nlevels, ulevels):
        nlevels = np.ascontiguousarray(nlevels, dtype=np.int32)
        ulevels = np.ascontiguousarray(ulevels, dtype=np.int32)
        return self.lib.tracer_set_levels(nlevels, ulevels, len(nlevels))

    def set_thickness(self, hnode):
        hnode = np.asfortranarray(hnode, dtype=np.float64)
        return self.lib.tracer_set_thickness(hnode, hnode.shape[0] + 1, hnode.shape[1])

    def set_partition(self, myDim, eDim=0):
        return self.lib.tracer_set_partition(myDim, eDim)

    def allocate_tracers(self, num_tracers, nl, nod2D, AB_order=2):
        return self.lib.tracer_allocate_tracers(num_tracers, nl, nod2D, AB_order)

    def set_values(self, tracer_id, values):
        values = np.asfortranarray(values, dtype=np.float64)
        return self.lib.tracer_set_values(tracer_id, values, values.shape[0] + 1, values.shape[1])

    def set_velocity_zero(self):
        return self.lib.tracer_set_velocity_zero(self.nl, self.nod2D, self.edge2D)

    def set_velocity(self, uv, w):
        uv = np.asfortranarray(uv, dtype=np.float64)
        w = np.asfortranarray(w, dtype=np.float64)
        return self.lib.tracer_set_velocity(uv, w, uv.shape[0] + 1, w.shape[1], uv.shape[1])

    def set_schemes(self, tracer_id, hor="UPW1", ver="UPW1", lim="NONE", ph=1.0, pv=1.0):
        return self.lib.tracer_set_schemes(tracer_id, hor.encode(), ver.encode(), lim.encode(), ph, pv)

    def set_precision(self, precision="fp64"):
        return self.lib.tracer_set_precision({"fp64": 0, "fp32": 1}[precision])

    def set_input_checks(self, on=True):
        """Check before every step that its inputs are finite (tracer_set_input_checks)."""
        return self.lib.tracer_set_input_checks(int(bool(on)))

    def init_ale_arrays(self):
        return self.lib.tracer_init_ale_arrays()

    def init_for_advection(self):
        return self.lib.tracer_init_for_advection()

    def init_complete(self):
        return self.lib.tracer_init_complete()

    def cleanup(self):
        return self.lib.tracer_cleanup()
