"""Binary output of the analytic dwarf's ``--save-mesh`` / ``--save-scalars``
(lib/mesh_output.F90:19-160), in the reference's file layout, so the
reference's visualisation scripts read runs of this library unchanged:

- ``mesh_info.txt`` (``nod2D=``, ``elem2D=``, ``nl=``), ``coord_nod2D.bin``
  (float64 (nod2D, 2) in metres: coordinates x r_earth), ``elem2D_nodes.bin``
  (int32 (elem2D, 3), 0-based), ``zbar.bin`` (float64 (nl)), ``depth.bin``
  (float64 (nod2D));
- ``scalar_info.txt`` (``nod2D=``, ``nz=``, ``nsteps=``, ``num_tracers=``,
  ``wp=``, ``tracer_<n>=<name>``) and one ``<name>.bin`` per tracer holding
  nsteps + 1 frames of float64 (nod2D, nz), layer index fastest.

The reference names its two tracers temperature and salinity; further
tracers are named ``tracer<n>`` here.
"""
from __future__ import annotations

import os

import numpy as np

R_EARTH = 6367500.0  # lib/oce_modules.F90:24
TRACER_NAMES = ("temperature", "salinity")


def tracer_name(n: int) -> str:
    """Name of tracer n (0-based)."""
    return TRACER_NAMES[n] if n < len(TRACER_NAMES) else f"tracer{n + 1}"


def node_depth(mesh) -> np.ndarray:
    """mesh%depth: -max_depth on every node of the reference's flat analytic
    mesh (lib/analytic_mesh.F90:372-373); on meshes with bathymetry the
    depth of each node's deepest interface."""
    nlev = mesh.get("nlevels_nod2D")
    if getattr(mesh, "depth", None) is not None and bool(np.all(nlev == mesh.nl)):
        return np.full(mesh.N, -float(mesh.depth))
    return mesh.get("zbar")[nlev - 1].astype(np.float64)


def write_mesh_for_python(mesh, output_dir: str) -> None:
    """write_mesh_for_python (lib/mesh_output.F90:19-77) of a ``Mesh``."""
    os.makedirs(output_dir, exist_ok=True)
    with open(os.path.join(output_dir, "mesh_info.txt"), "w") as f:
        f.write(f"nod2D={mesh.N}\nelem2D={mesh.M}\nnl={mesh.nl}\n")
    coords = np.ascontiguousarray(mesh.get("coord")[: mesh.N], dtype=np.float64) * R_EARTH
    coords.tofile(os.path.join(output_dir, "coord_nod2D.bin"))
    np.ascontiguousarray(mesh.get("elem_nodes"), dtype=np.int32).tofile(os.path.join(output_dir, "elem2D_nodes.bin"))
    np.ascontiguousarray(mesh.get("zbar"), dtype=np.float64).tofile(os.path.join(output_dir, "zbar.bin"))
    np.ascontiguousarray(node_depth(mesh), dtype=np.float64).tofile(os.path.join(output_dir, "depth.bin"))


class ScalarOutput:
    """open_scalar_output / write_scalar_step / close_scalar_output
    (lib/mesh_output.F90:80-160). ``wp`` is the byte width of the run's
    working precision (8 for the FP64 form, 4 for the FP32 form); the files
    hold float64 either way."""

    def __init__(self, nod2D: int, nz: int, nsteps: int, num_tracers: int, output_dir: str, wp: int = 8):
        os.makedirs(output_dir, exist_ok=True)
        self.nod2D, self.nz, self.num_tracers = int(nod2D), int(nz), int(num_tracers)
        with open(os.path.join(output_dir, "scalar_info.txt"), "w") as f:
            f.write(f"nod2D={nod2D}\nnz={nz}\nnsteps={nsteps}\nnum_tracers={num_tracers}\nwp={wp}\n")
            for n in range(num_tracers):
                f.write(f"tracer_{n + 1}={tracer_name(n)}\n")
        self._files = [open(os.path.join(output_dir, f"{tracer_name(n)}.bin"), "wb") for n in range(num_tracers)]

    def write_step(self, values) -> None:
        """values: (num_tracers, >= nod2D, >= nz) array-like."""
        for n, f in enumerate(self._files):
            frame = np.asarray(values[n], dtype=np.float64)[: self.nod2D, : self.nz]
            f.write(np.ascontiguousarray(frame).tobytes())

    def close(self) -> None:
        for f in self._files:
            f.close()
        self._files = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
