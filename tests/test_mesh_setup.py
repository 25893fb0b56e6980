"""Host-side mesh set-up of the library against the oracle's restatement of
lib/analytic_mesh.F90 and lib/oce_mesh.F90 (CPU only, no GPU needed)."""
import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300 import synthetic
from fesom2_tracer_dwarf_gb300.mesh import Mesh

INT_ARRAYS = [("elem_nodes", "elem2D_nodes", 1), ("edges", "edges", 1), ("edge_tri", "edge_tri", 1),
              ("nlevels", "nlevels", 0), ("nlevels_nod2D", "nlevels_nod2D", 0),
              ("nlevels_nod2D_min", "nlevels_nod2D_min", 0), ("ulevels_nod2D_max", "ulevels_nod2D_max", 0),
              ("edge_up_dn_tri", "edge_up_dn_tri", 1), ("nboundary_lay", "nboundary_lay", 0),
              ("nod_in_elem2D_num", "nod_in_elem2D_num", 0)]
DBL_ARRAYS = ["coord", "elem_area", "area", "areasvol", "edge_dxdy", "edge_cross_dxdy", "gradient_sca", "hnode",
              "hnode_new", "helem", "Z_3d_n", "zbar_3d_n"]


def _cases():
    rng = np.random.default_rng(1)
    zb = synthetic.stretched_zbar(9, 5.0, 80.0)
    en = synthetic.bathymetry_levels(9, 8, zb, rng, min_layers=2)
    return [
        dict(nx=20, ny=20, nl=10, periodic=True),
        dict(nx=7, ny=11, nl=5, periodic=True, cluster_full=True),
        dict(nx=9, ny=6, nl=6, periodic=False),
        dict(nx=8, ny=9, nl=7, periodic=True, orient_left=True),
        dict(nx=9, ny=8, nl=10, periodic=False, zbar=zb, elem_nlev=en, orient_left=True),
    ]


@pytest.mark.parametrize("kw", _cases())
def test_host_mesh_equals_oracle(oracle_mod, kw):
    m = Mesh(upload=False, **kw)
    o = oracle_mod.Mesh(**kw)
    assert (m.N, m.E, m.M) == (o.nod2D, o.edge2D, o.elem2D)
    for mine, theirs, off in INT_ARRAYS:
        np.testing.assert_array_equal(m.get(mine), o.geti(theirs) - off, err_msg=mine)
    for name in DBL_ARRAYS:
        a, b = m.get(name), o.getd(name)
        assert a.shape == b.shape, name
        assert np.array_equal(a, b), f"{name}: max diff {np.abs(a - b).max()}"
    nie_m, nie_o = m.get("nod_in_elem2D"), o.geti("nod_in_elem2D") - 1
    w = min(nie_m.shape[1], nie_o.shape[1])
    num = m.get("nod_in_elem2D_num")
    for n in range(m.N):
        np.testing.assert_array_equal(nie_m[n, : num[n]], nie_o[n, : num[n]])
    assert w >= num.max()


def test_periodic_streamfunction_is_solenoidal():
    """With edge_tri(1) on the left the rotated-gradient flow telescopes: W ~ 0."""
    m = Mesh(13, 11, 6, periodic=True, orient_left=True, upload=False)
    vel, w = synthetic.streamfunction_flow(m, np.random.default_rng(2), 300.0)
    assert np.abs(w).max() < 1e-12
    assert abs(synthetic.max_cfl(m, vel, 300.0) - 0.4) < 1e-12


def test_reference_mesh_orientation_quirk():
    """The reference's analytic grid keeps edge_tri(1) right of horizontal and
    vertical edges (lib/analytic_mesh.F90:386-426), so the same flow is not
    discretely solenoidal there."""
    m = Mesh(13, 11, 6, periodic=True, upload=False)
    _, w = synthetic.streamfunction_flow(m, np.random.default_rng(2), 300.0)
    assert np.abs(w).max() > 1e-3


def test_gather_tables_cover_every_edge_twice():
    m = Mesh(9, 7, 5, periodic=False, upload=False)
    ptr, code = m.get("ne_ptr"), m.get("ne_code")
    assert ptr[-1] == 2 * m.E
    counts = np.bincount(code // 2, minlength=m.E)
    assert np.all(counts == 2)
    for n in range(m.N):
        e = code[ptr[n]:ptr[n + 1]] // 2
        assert np.all(np.diff(e) > 0), "incident edges must be in ascending edge order"
