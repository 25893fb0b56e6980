"""The analytic dwarf driver on the GPU (src/fesom_analytic.F90), same command
line and console lines:

    python -m fesom2_tracer_dwarf_gb300.analytic [nx] [ny] [nl] [--periodic]
        [--save-mesh] [--save-scalars] [--output-dir DIR] [--precision fp64|fp32]

Analytic mesh of nx x ny grid points and nl levels over 100 km x 100 km x
1000 m (:66-68; defaults 20 20 10, :80-82), temperature and salinity set as in
:300-331, u = (0.1, 0) m/s and W = 0, UPW1 / UPW1 / no limiter, valuesAB
frozen at the initial values (:335), 10 steps of 1000 s (:385-386), each
followed by the line ``Step n: T min, max, sum = ...`` of :448-449.
``--save-mesh`` / ``--save-scalars`` write the reference's binary files
(``output.py``). ``--precision fp32`` runs the FP32 form (an extension).
"""
from __future__ import annotations

import argparse
import math
import sys

import numpy as np

from . import output

LX = LY = 100000.0  # src/fesom_analytic.F90:66-67
MAX_DEPTH = 1000.0  # :68
PI = 3.14159265358979  # lib/oce_modules.F90:19
NSTEPS, DT = 10, 1000.0  # :385-386


def fortran_e(x: float, w: int, d: int) -> str:
    """Fortran Ew.d: 0.<d digits>E+xx, right-aligned in w characters."""
    if x != x:
        s = "NaN"
    elif x == 0.0:
        s = "0." + "0" * d + "E+00"
    else:
        mant, exp = f"{abs(x):.{d - 1}e}".split("e")
        e = int(exp) + 1
        s = ("-" if x < 0 else "") + "0." + mant.replace(".", "") + f"E{'+' if e >= 0 else '-'}{abs(e):02d}"
    return s.rjust(w)


def dwarf_fields(mesh):
    """Initial temperature and salinity (2, N, nz) of src/fesom_analytic.F90:300-331,
    evaluated with the C library's sin, cos and exp in the reference's order."""
    c = mesh.get("coord")[: mesh.N]
    nz = mesh.nz
    zn = np.array([(k - 1) / (nz - 1) for k in range(1, nz + 1)]) if nz > 1 else np.zeros(1)
    xc, yc = 0.5 * LX, 0.5 * LY
    T = np.empty((mesh.N, nz))
    S = np.empty((mesh.N, nz))
    for n in range(mesh.N):
        xn, yn = c[n, 0] * output.R_EARTH, c[n, 1] * output.R_EARTH
        ridge = (5.0 * math.sin(((2.0 * PI) * xn) / LX)) * math.cos(((2.0 * PI) * yn) / LY)
        r = math.sqrt((xn - xc) * (xn - xc) + (yn - yc) * (yn - yc))
        blob = 2.0 * math.exp(-(r * r) / ((0.1 * LX) * (0.1 * LX)))
        T[n] = (15.0 + ridge) - 10.0 * zn
        S[n] = 34.0 + blob * (1.0 - zn)
    return np.stack([T, S])


def run(nx=20, ny=20, nl=10, periodic=False, save_mesh=False, save_scalars=False, output_dir="mesh_output",
        precision="fp64", nsteps=NSTEPS, out=sys.stdout):
    """Runs the dwarf; returns the per-step (min, max, sum, NaN count) of the
    temperature."""
    from .engine import TracerAdvection
    from .mesh import Mesh
    from .synthetic import dwarf_velocity

    m = Mesh(nx, ny, nl, Lx=LX, Ly=LY, depth=MAX_DEPTH, periodic=periodic)
    if save_mesh:
        print(f"  --> Writing mesh to {output_dir}", file=out)
        output.write_mesh_for_python(m, output_dir)
    vals = dwarf_fields(m)
    eng = TracerAdvection(m, 2, precision, "UPW1", "UPW1", "NONE")
    eng.set_tracers(vals)
    eng.set_velocity(*dwarf_velocity(m))
    print(f"  Steps: {nsteps:6d}, dt = {fortran_e(DT, 12, 4)}", file=out)
    scal = None
    if save_scalars:
        print(f"  --> Writing scalar output to {output_dir}", file=out)
        scal = output.ScalarOutput(m.N, m.nz, nsteps, 2, output_dir, wp=8 if precision == "fp64" else 4)
        scal.write_step(vals)
    rows = []
    for step in range(1, nsteps + 1):
        eng.step(DT)
        tmin, tmax, tsum, nan = (float(v) for v in eng.stats()[0])
        rows.append((tmin, tmax, tsum, int(nan)))
        print(f"  Step {step:4d}: T min, max, sum = {fortran_e(tmin, 14, 6)}{fortran_e(tmax, 14, 6)}"
              f"{fortran_e(tsum, 18, 10)}  NaN:{int(nan):6d}", file=out)
        if scal is not None:
            scal.write_step(eng.values())
    if scal is not None:
        scal.close()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("dims", nargs="*", type=int, help="nx ny nl")
    ap.add_argument("--periodic", action="store_true")
    ap.add_argument("--save-mesh", action="store_true")
    ap.add_argument("--save-scalars", action="store_true")
    ap.add_argument("--output-dir", default="mesh_output")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    a = ap.parse_args(argv)
    if len(a.dims) > 3:
        ap.error("at most three positional arguments: nx ny nl")
    nx, ny, nl = (a.dims + [20, 20, 10][len(a.dims):])[:3]
    if nx < 2 or ny < 2:
        ap.error("nx and ny must be >= 2")
    run(nx, ny, nl, a.periodic, a.save_mesh, a.save_scalars, a.output_dir, a.precision)


if __name__ == "__main__":
    main()
