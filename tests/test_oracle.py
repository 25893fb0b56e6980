"""The oracle against the reference's only golden vectors (README.md:51-52).

`run.sh 1 20 20 10 --periodic` of the analytic dwarf (src/fesom_analytic.F90)
prints, per step, T min/max/sum with format (A,I4,A,2E14.6,E18.10,A,I6)
(src/fesom_analytic.F90:447-448). The first two lines are quoted in README.md.
"""
import math

import numpy as np
import pytest

GOLDEN = {
    1: ("0.246394E-01", "0.199736E+02", "0.3249000000E+05"),
    2: ("0.322013E-01", "0.199642E+02", "0.3249000000E+05"),
}


def fortran_e(x, d):
    """Fortran Ew.d mantissa/exponent text (0.ddddddE+xx) without padding."""
    if x == 0.0:
        return "0." + "0" * d + "E+00"
    e = math.floor(math.log10(abs(x))) + 1
    m = abs(x) / 10.0 ** e
    digits = round(m * 10 ** d)
    if digits >= 10 ** d:
        digits //= 10
        e += 1
    s = "-" if x < 0 else ""
    return f"{s}0.{digits:0{d}d}E{'+' if e >= 0 else '-'}{abs(e):02d}"


def run_dwarf(O, steps, nx=20, ny=20, nl=10):
    m = O.Mesh(nx, ny, nl, periodic=True)
    T, S = m.dwarf_fields()
    nz = m.nl - 1
    vel = np.zeros((m.elem2D, nz, 2))
    vel[..., 0] = 0.1
    w = np.zeros((m.nod2D, m.nl))
    vals = np.ascontiguousarray(np.stack([T, S]))
    vab = vals.copy()
    W = O.Work(m)
    out = []
    for _ in range(steps):
        O.analytic_step(m, W, 1000.0, vel, w, vals, vab, [("UPW1", "UPW1", "NONE")] * 2)
        out.append(m.stats(vals[0]))
    return m, out


def test_fortran_e_format():
    assert fortran_e(0.0246394, 6) == "0.246394E-01"
    assert fortran_e(32490.0, 10) == "0.3249000000E+05"


def test_mesh_sizes(oracle_mod):
    m = oracle_mod.Mesh(20, 20, 10, periodic=True)
    assert (m.nod2D, m.elem2D, m.edge2D) == (361, 722, 1083)
    mc = oracle_mod.Mesh(20, 20, 10, periodic=False)
    assert (mc.nod2D, mc.elem2D, mc.edge2D) == (400, 722, 19 * 20 * 2 + 19 * 19)
    assert mc.edge2D - mc.edge2D_in == 2 * 19 + 2 * 19


def test_golden_readme_lines(oracle_mod):
    _, stats = run_dwarf(oracle_mod, 2)
    for step, (gmin, gmax, gsum) in GOLDEN.items():
        tmin, tmax, tsum, nan = stats[step - 1]
        assert fortran_e(tmin, 6) == gmin
        assert fortran_e(tmax, 6) == gmax
        assert fortran_e(tsum, 10) == gsum
        assert nan == 0


def test_dwarf_linear_drift_frozen_ab(oracle_mod):
    """valuesAB is frozen at the initial field (src/fesom_analytic.F90:335), so the
    minimum drifts linearly in time."""
    _, stats = run_dwarf(oracle_mod, 10)
    mins = np.array([s[0] for s in stats])
    d = np.diff(mins)
    assert np.allclose(d, d[0], rtol=1e-9)
    sums = np.array([s[2] for s in stats])
    assert np.all(np.abs(sums - 32490.0) / 32490.0 < 1e-14)


SCHEMES = [(h, v, l) for h in ("UPW1", "MUSCL", "MFCT") for v in ("UPW1", "QR4C", "PPM", "CDIFF")
           for l in ("NONE", "FCT") if not (v == "CDIFF" and l == "NONE")]


def _random_case(O, rng, periodic, ragged):
    nx, ny, nl = 15, 13, 11
    en = None
    if ragged:
        en = rng.integers(4, nl + 1, size=2 * (nx - 1) * (ny - 1)).astype(np.int32)
    m = O.Mesh(nx, ny, nl, periodic=periodic, elem_nlev=en)
    nz = m.nl - 1
    vel = rng.uniform(-0.3, 0.3, size=(m.elem2D, nz, 2))
    w = rng.uniform(-2e-3, 2e-3, size=(m.nod2D, m.nl))
    nlev = m.geti("nlevels_nod2D")
    for n in range(m.nod2D):
        w[n, nlev[n] - 1:] = 0.0
    T = 10.0 + rng.normal(0.0, 1.0, size=(2, m.nod2D, nz))
    return m, vel, w, np.ascontiguousarray(T)


@pytest.mark.parametrize("periodic,ragged", [(True, False), (False, True)])
def test_threads_change_no_result(oracle_mod, periodic, ragged):
    """The oracle's OpenMP loops keep every result bit for bit: 1 thread
    against 5 (node ranges that cut the mesh unevenly), every scheme
    combination, two steps with copy-AB, and w_split under FCT."""
    O = oracle_mod
    rng = np.random.default_rng(11)
    m, vel, w, T = _random_case(O, rng, periodic, ragged)
    wi = 0.5 * w
    before = O.get_threads()
    try:
        for sch in SCHEMES:
            outs = []
            for nt in (1, 5):
                O.set_threads(nt)
                vals, vab = T.copy(), T.copy()
                W = O.Work(m)
                kw = dict(wi=wi, we=w - wi) if sch[2] == "FCT" and sch[1] != "UPW1" else {}
                for _ in range(2):
                    O.analytic_step(m, W, 300.0, vel, w, vals, vab, [sch] * 2, copy_ab=True, **kw)
                outs.append(vals)
            assert np.array_equal(outs[0], outs[1]), sch
    finally:
        O.set_threads(before)
