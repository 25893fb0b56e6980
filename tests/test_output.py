"""The analytic dwarf driver and its binary output (src/fesom_analytic.F90,
lib/mesh_output.F90:19-160).

CPU: the files have the reference's layout (read back the way the reference's
visualisation scripts read them: np.fromfile, frames of (nod2D, nz)); the
driver's initial fields equal the oracle's bit for bit; the Fortran E
formatting. GPU: the driver prints the golden lines of the reference README
and writes nsteps + 1 frames.
"""
import io
import os

import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300 import analytic, output
from fesom2_tracer_dwarf_gb300.mesh import Mesh


def _read_info(path):
    info = {}
    with open(path) as f:
        for line in f:
            k, v = line.strip().split("=", 1)
            info[k] = v
    return info


def test_mesh_files(tmp_path):
    m = Mesh(9, 7, 6, periodic=True, upload=False)
    output.write_mesh_for_python(m, str(tmp_path))
    info = _read_info(tmp_path / "mesh_info.txt")
    assert info == {"nod2D": str(m.N), "elem2D": str(m.M), "nl": str(m.nl)}
    coords = np.fromfile(tmp_path / "coord_nod2D.bin", dtype=np.float64).reshape(m.N, 2)
    assert np.array_equal(coords, m.get("coord")[: m.N] * 6367500.0)
    tri = np.fromfile(tmp_path / "elem2D_nodes.bin", dtype=np.int32).reshape(m.M, 3)
    assert tri.min() == 0 and tri.max() == m.N - 1 and np.array_equal(tri, m.get("elem_nodes"))
    zbar = np.fromfile(tmp_path / "zbar.bin", dtype=np.float64)
    assert zbar.shape == (m.nl,) and zbar[0] == 0.0 and zbar[-1] == -1000.0
    depth = np.fromfile(tmp_path / "depth.bin", dtype=np.float64)
    assert np.array_equal(depth, np.full(m.N, -1000.0))


def test_scalar_files(tmp_path):
    rng = np.random.default_rng(0)
    N, nz, nsteps = 11, 4, 3
    frames = rng.normal(size=(nsteps + 1, 3, N + 2, nz + 1))  # extra rows/columns are cut
    with output.ScalarOutput(N, nz, nsteps, 3, str(tmp_path), wp=4) as out:
        for f in frames:
            out.write_step(f)
    info = _read_info(tmp_path / "scalar_info.txt")
    assert info["nod2D"] == str(N) and info["nz"] == str(nz) and info["nsteps"] == str(nsteps)
    assert info["wp"] == "4" and info["tracer_1"] == "temperature" and info["tracer_2"] == "salinity"
    for n in range(3):
        raw = np.fromfile(tmp_path / f"{info[f'tracer_{n + 1}']}.bin", dtype=np.float64)
        assert raw.size == (nsteps + 1) * nz * N
        assert np.array_equal(raw.reshape(nsteps + 1, N, nz), frames[:, n, :N, :nz])


def test_dwarf_fields_equal_oracle(oracle_mod):
    m = Mesh(20, 20, 10, periodic=True, upload=False)
    om = oracle_mod.Mesh(20, 20, 10, periodic=True)
    T, S = om.dwarf_fields()
    got = analytic.dwarf_fields(m)
    assert np.array_equal(got[0], T) and np.array_equal(got[1], S)


def test_fortran_e():
    assert analytic.fortran_e(0.02463941, 14, 6) == "  0.246394E-01"
    assert analytic.fortran_e(32490.0, 18, 10) == "  0.3249000000E+05"
    assert analytic.fortran_e(-19.97356, 14, 6) == " -0.199736E+02"
    assert analytic.fortran_e(0.0, 12, 4) == "  0.0000E+00"
    assert analytic.fortran_e(1000.0, 12, 4) == "  0.1000E+04"


torch = pytest.importorskip("torch")


@pytest.mark.gpu
def test_dwarf_driver_golden_and_scalars(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from tests.test_oracle import GOLDEN

    buf = io.StringIO()
    rows = analytic.run(20, 20, 10, periodic=True, save_mesh=True, save_scalars=True, output_dir=str(tmp_path),
                        out=buf)
    lines = [ln for ln in buf.getvalue().splitlines() if ln.startswith("  Step ")]
    assert len(rows) == 10 and len(lines) == 10
    for step, (gmin, gmax, gsum) in GOLDEN.items():
        # README.md:51-52 (the README drops the two leading blanks of the Fortran format)
        assert lines[step - 1] == f"  Step {step:4d}: T min, max, sum =   {gmin}  {gmax}  {gsum}  NaN:     0"
    info = _read_info(tmp_path / "scalar_info.txt")
    N, nz = int(info["nod2D"]), int(info["nz"])
    raw = np.fromfile(tmp_path / "temperature.bin", dtype=np.float64).reshape(11, N, nz)
    assert np.array_equal(raw[0], analytic.dwarf_fields(Mesh(20, 20, 10, periodic=True, upload=False))[0])
    assert abs(raw[-1].sum() - rows[-1][2]) <= 1e-9 * abs(rows[-1][2])
    assert os.path.exists(tmp_path / "coord_nod2D.bin")


@pytest.mark.gpu
def test_dwarf_driver_fp32_form():
    """The dwarf in the FP32 form: per-step min and max within FP32 rounding of
    the FP64 run, the sum within 1e-8 relative (it drifts by a few 1e-10 over
    10 steps: every value is rounded to FP32 each step)."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    buf = io.StringIO()
    r64 = analytic.run(20, 20, 10, periodic=True, out=buf)
    r32 = analytic.run(20, 20, 10, periodic=True, precision="fp32", out=buf)
    for a, b in zip(r32, r64):
        assert abs(a[0] - b[0]) <= 2e-6 * abs(b[1]) and abs(a[1] - b[1]) <= 2e-6 * abs(b[1])
        assert abs(a[2] - b[2]) <= 1e-8 * abs(b[2]) and a[3] == 0
