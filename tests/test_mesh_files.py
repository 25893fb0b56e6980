"""FESOM mesh files: the pi mesh of the reference (tests/golden/pi_mesh.npz,
written back as a mesh directory) read by the library (fgb_hmesh_from_files,
tracer_load_mesh_from_files) and by the oracle (its own parser and
om_mesh_from_arrays).

CPU: the library's set-up (read_mesh, test_tri, load_edges, find_levels,
mesh_areas and mesh_auxiliary_arrays of lib/oce_mesh.F90 on the sphere) equals
the oracle's bit for bit under the reference's defaults and under FESOM2's
namelist handling; the sizes are those python/test_mesh_from_files.py prints;
malformed directories are refused; in the oracle a zero velocity leaves the
tracers unchanged and a continuity-consistent flow keeps a uniform tracer
uniform on this unstructured, ragged, coastal mesh; the refinement tool keeps
the topology and orientation, and its layered flow is continuity-consistent.
GPU: the step on the pi mesh and on its refinement equals the oracle (FP64 bit
for bit, FP32 to 1e-5), through the engine and through the C ABI, and the
reference's mesh-from-files workflow runs through the C ABI.
"""
import itertools
import os
import zlib

import numpy as np
import pytest

from fesom_files import load_pi, write_mesh_dir, write_pi, write_pi_refined

FLAGS = [dict(), dict(euler_degrees=True, cyclic_2pi=True), dict(rotate=False)]
REAL = ["coord", "elem_area", "area", "areasvol", "edge_dxdy", "edge_cross_dxdy", "elem_cos", "gradient_sca",
        "hnode", "hnode_new", "helem", "Z_3d_n", "zbar_3d_n"]
INDEX = {"elem_nodes": ("elem2D_nodes", 1), "edges": ("edges", 1), "edge_tri": ("edge_tri", 1),
         "edge_up_dn_tri": ("edge_up_dn_tri", 1), "nlevels": ("nlevels", 0), "nlevels_nod2D": ("nlevels_nod2D", 0),
         "nlevels_nod2D_min": ("nlevels_nod2D_min", 0), "nboundary_lay": ("nboundary_lay", 0),
         "nod_in_elem2D_num": ("nod_in_elem2D_num", 0)}


@pytest.fixture(scope="module")
def pi_dir(tmp_path_factory):
    return write_pi(str(tmp_path_factory.mktemp("pi")))


@pytest.fixture(scope="module")
def pi_refined_dir(tmp_path_factory):
    return write_pi_refined(str(tmp_path_factory.mktemp("pi_refined")), 1)


def _mesh(path, upload=False, **kw):
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    return Mesh.from_files(path, upload=upload, **kw)


def test_sizes_as_the_reference_test_prints(pi_dir):
    m = _mesh(pi_dir)
    assert (m.nl, m.N, m.E, m.M, m.edge2D_in) == (48, 3140, 8986, 5839, 8531)
    assert m.nz == 47 and m.max_nie == 8
    lev = m.get("nlevels_nod2D")
    assert lev.min() == 5 and lev.max() == 46  # ragged bottom


@pytest.mark.parametrize("flags", FLAGS, ids=["reference", "fesom2_namelist", "no_rotation"])
def test_setup_matches_oracle(pi_dir, oracle_mod, flags):
    m = _mesh(pi_dir, **flags)
    om = oracle_mod.Mesh.from_files(pi_dir, **flags)
    assert (om.nod2D, om.edge2D, om.elem2D, om.nl, om.edge2D_in) == (m.N, m.E, m.M, m.nl, m.edge2D_in)
    for name in REAL:
        a = m.get(name)
        b = om.getd(name).reshape(a.shape)
        assert np.array_equal(a, b), f"{name}: max |diff| {np.abs(a - b).max()}"
    for name, (oname, off) in INDEX.items():
        a = m.get(name)
        b = om.geti(oname).reshape(a.shape) - off
        assert np.array_equal(a, b), f"{name}: {(a != b).sum()} entries differ"


def test_reference_defaults_leave_the_seam_untrimmed(pi_dir):
    """cyclic_length stays 360 against radian coordinates, so elements across
    the rotated grid's seam get the full 2*pi longitude jump in their area;
    FESOM2's 2*pi trims it (elements of the same order as their neighbours)."""
    ref = _mesh(pi_dir).get("elem_area")
    fixed = _mesh(pi_dir, euler_degrees=True, cyclic_2pi=True).get("elem_area")
    assert ref.max() > 100 * np.median(ref)
    assert fixed.max() < 50 * np.median(fixed)


def test_malformed_directories_are_refused(tmp_path, pi_dir):
    from fesom2_tracer_dwarf_gb300 import _lib

    with pytest.raises(RuntimeError, match="can not open file"):
        _mesh(str(tmp_path / "missing"))
    d = load_pi()
    elem = d["elem"].copy()
    elem[7, 1] = 99999
    p = write_mesh_dir(str(tmp_path / "bad_elem"), d["lonlat"], elem, d["zbar"], d["edges"], d["edge_tri"],
                       d["edgenum"], d["elvls"], d["nlvls"])
    with pytest.raises(RuntimeError, match="node index out of range"):
        _mesh(p)
    p = write_mesh_dir(str(tmp_path / "short"), d["lonlat"], d["elem"], d["zbar"], d["edges"][:-5],
                       d["edge_tri"][:-5], d["edgenum"], d["elvls"], d["nlvls"])
    with pytest.raises(RuntimeError, match="unexpected end of data"):
        _mesh(p)
    p = write_mesh_dir(str(tmp_path / "two_levels"), d["lonlat"], d["elem"], d["zbar"][:2], d["edges"],
                       d["edge_tri"], d["edgenum"], d["elvls"], d["nlvls"])
    with pytest.raises(RuntimeError, match="less than 3"):
        _mesh(p)
    # the path may end without '/'
    assert _mesh(pi_dir.rstrip("/")).N == 3140
    assert _lib.load().tracer_load_mesh_from_files(str(tmp_path / "missing").encode()) == -1


def test_list_directed_input_forms(tmp_path, pi_dir):
    """The reader takes what Fortran list-directed input takes: CRLF line
    ends, blank lines before a record, commas and tabs as separators, D
    exponents, and extra items after a record's last value (skipped)."""
    import shutil

    d = load_pi()
    p = str(tmp_path / "forms")
    shutil.copytree(pi_dir, p)
    with open(os.path.join(p, "nod2d.out"), "w", newline="") as f:
        f.write(f"\r\n  {len(d['lonlat'])}\r\n")
        for i, (x, y) in enumerate(d["lonlat"]):
            f.write(f"{i + 1},\t{float(x)!r}, {float(y)!r}  0   trailing items\r\n")
    with open(os.path.join(p, "aux3d.out"), "w") as f:
        f.write(f"{len(d['zbar'])}\n\n")
        zs = [f"{z:.17e}".replace("e", "D") for z in d["zbar"]]
        f.write(" ".join(zs[:10]) + "\n" + "\n".join(zs[10:]) + "\n")
    a, b = _mesh(p), _mesh(pi_dir)
    for name in REAL:
        assert np.array_equal(a.get(name), b.get(name)), name


def test_refined_mesh(oracle_mod, pi_refined_dir):
    """meshfiles.refine: four children per triangle, the topology kept
    (N - E + M of the pi mesh, -7: a sphere with its coasts cut out),
    edge_tri(1) left of node1 -> node2, node levels the deepest adjacent
    element's; the library and the oracle set it up identically, and the
    arrays path equals the files path."""
    from fesom2_tracer_dwarf_gb300.mesh import Mesh
    from fesom2_tracer_dwarf_gb300.meshfiles import _xyz, refine

    d = load_pi()
    r = refine(d, 1)
    N, M, E = len(r["lonlat"]), len(r["elem"]), len(r["edges"])
    assert M == 4 * len(d["elem"]) and N == len(d["lonlat"]) + len(d["edges"])
    assert N - E + M == len(d["lonlat"]) - len(d["edges"]) + len(d["elem"]) == -7
    xyz = _xyz(r["lonlat"])
    ed, et, el = r["edges"] - 1, r["edge_tri"] - 1, r["elem"] - 1
    third = np.array([[v for v in el[t] if v not in e][0] for e, t in zip(ed, et[:, 0])])
    assert np.all(np.einsum("ij,ij->i", np.cross(xyz[ed[:, 0]], xyz[ed[:, 1]]), xyz[third]) > 0)
    assert np.all(et[: r["edgenum"][1], 1] >= 0) and np.all(et[r["edgenum"][1]:, 1] < 0)
    mx = np.zeros(N, int)
    np.maximum.at(mx, el.reshape(-1), np.repeat(r["elvls"], 3))
    assert np.array_equal(mx, r["nlvls"])
    for flags in FLAGS[:2]:
        m = _mesh(pi_refined_dir, **flags)
        om = oracle_mod.Mesh.from_files(pi_refined_dir, **flags)
        a = Mesh.from_arrays(**r, upload=False, **flags)
        for name in REAL:
            assert np.array_equal(m.get(name), om.getd(name).reshape(m.get(name).shape)), name
            assert np.array_equal(m.get(name), a.get(name)), name
        assert np.array_equal(m.get("edge_up_dn_tri"), om.geti("edge_up_dn_tri") - 1)


def test_build_edges_on_two_triangles():
    """meshfiles.build_edges: a quad of two triangles near the equator has one
    interior edge (listed first) and four coast edges, each with its element
    on the left of node1 -> node2 (east-north frame seen from outside)."""
    from fesom2_tracer_dwarf_gb300.meshfiles import _xyz, build_edges, morton_order

    lonlat = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    elem0 = np.array([[0, 1, 2], [0, 2, 3]])
    edges, edge_tri, n_in = build_edges(elem0, _xyz(lonlat))
    assert n_in == 1 and len(edges) == 5
    assert sorted(edges[0]) == [0, 2] and sorted(edge_tri[0]) == [0, 1]
    assert np.all(edge_tri[1:, 1] == -1)
    for (a, b), (t, _) in zip(edges, edge_tri):
        c = [v for v in elem0[t] if v not in (a, b)][0]
        (x1, y1), (x2, y2), (x3, y3) = lonlat[a], lonlat[b], lonlat[c]
        assert (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1) > 0
    # Morton order visits the lower-left quadrant before the upper-right one
    pts = np.array([[0.9, 0.9], [0.1, 0.1], [0.9, 0.1], [0.1, 0.9]])
    order = morton_order(pts)
    assert order[0] == 1 and order[-1] == 0


def test_refinement_cli_round_trip(tmp_path, pi_dir):
    """python -m fesom2_tracer_dwarf_gb300.meshfiles SRC DST TIMES writes the
    directory that refine + write_fesom_dir produce from the same input."""
    from fesom2_tracer_dwarf_gb300 import meshfiles

    dst = str(tmp_path / "cli")
    assert meshfiles.main([pi_dir, dst, "1"]) == 0
    a, b = meshfiles.read_fesom_dir(dst), meshfiles.refine(meshfiles.read_fesom_dir(pi_dir), 1)
    assert np.array_equal(a["lonlat"], b["lonlat"]) and np.array_equal(a["elem"], b["elem"])
    assert np.array_equal(a["elvls"], b["elvls"]) and np.array_equal(a["zbar"], b["zbar"])
    assert _mesh(dst).N == len(b["lonlat"])


def test_union_with_a_file_mesh_shifts_its_tables(pi_dir):
    """Mesh.union of the pi mesh and an analytic grid: each part's gather
    tables and levels reappear shifted by the part offsets, layers padded to
    the deeper part."""
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    parts = [_mesh(pi_dir, euler_degrees=True, cyclic_2pi=True), Mesh(9, 8, 6, periodic=True, upload=False)]
    u = Mesh.union(parts, upload=False)
    assert u.N == sum(p.N for p in parts) and u.nl == 48
    for i, p in enumerate(parts):
        o = u.parts[i]
        j0 = u.get("ne_ptr")[o["node"]]
        pc = p.get("ne_code")
        assert np.array_equal(u.get("ne_code")[j0: j0 + len(pc)], pc + 2 * o["edge"])
        assert np.array_equal(u.part_view(u.get("nlevels_nod2D"), i), p.get("nlevels_nod2D"))
        assert np.array_equal(u.part_view(u.get("area"), i)[:, : p.nl], p.get("area"))
        assert np.array_equal(u.get("gradient_sca")[o["elem"]: o["elem"] + p.M], p.get("gradient_sca"))


def test_visit_order_follows_a_hilbert_curve(pi_dir, pi_refined_dir):
    """File meshes: the kernels visit node columns along a Hilbert curve and
    each edge with its first-visited node; numbering and every mesh array stay
    the file's (keep_order=True: node index order, edges by lower node)."""
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    for d in (pi_dir, pi_refined_dir):
        h, k = _mesh(d), _mesh(d, keep_order=True)
        order = h.get("node_order")
        assert sorted(order.tolist()) == list(range(h.N))
        assert not np.array_equal(order, np.arange(h.N))
        assert k.get("node_order").size == 0
        for name in ("edges", "elem_nodes", "edge_tri", "ne_ptr", "ne_code", "cl_node", "nlevels_nod2D"):
            assert np.array_equal(h.get(name), k.get(name)), name
        for name in ("area", "gradient_sca", "edge_cross_dxdy"):
            assert np.array_equal(h.get(name), k.get(name)), name
        rank = np.empty(h.N, np.int64)
        rank[order] = np.arange(h.N)
        ed = h.get("edges")
        first = np.minimum(rank[ed[:, 0]], rank[ed[:, 1]])
        eo = h.get("edge_order")
        assert sorted(eo.tolist()) == list(range(h.E))
        assert np.all(np.diff(first[eo]) >= 0)
        eo_k = k.get("edge_order")
        assert np.all(np.diff(ed[eo_k].min(axis=1)) >= 0)
        # consecutive columns along the curve are close: the mean step is a
        # small multiple of the mean edge length
        c = h.get("coord")
        step = np.hypot(*(c[order[1:]] - c[order[:-1]]).T)
        elen = np.hypot(*(c[ed[:, 0]] - c[ed[:, 1]]).T)
        assert np.median(step) <= 2.0 * np.median(elen)
    # analytic meshes keep node index order unless asked
    assert Mesh(9, 8, 6, periodic=True, upload=False).get("node_order").size == 0
    hm = Mesh(9, 8, 6, periodic=True, upload=False, hilbert=True)
    assert sorted(hm.get("node_order").tolist()) == list(range(hm.N))
    # a union keeps each part's visit order, the parts one after another
    parts = [_mesh(pi_dir), Mesh(9, 8, 6, periodic=True, upload=False)]
    u = Mesh.union(parts, upload=False)
    uo = u.get("node_order")
    assert np.array_equal(uo[: parts[0].N], parts[0].get("node_order"))
    assert np.array_equal(uo[parts[0].N:], parts[0].N + np.arange(parts[1].N))


def test_layered_flow_is_continuity_consistent(pi_refined_dir):
    """synthetic.layered_flow's W equals diagnose_w of its velocity, and its
    Courant numbers are at most the target."""
    from fesom2_tracer_dwarf_gb300 import synthetic

    m = _mesh(pi_refined_dir, euler_degrees=True, cyclic_2pi=True)
    u, s, w = synthetic.layered_flow(m, np.random.default_rng(6), 600.0, cfl=0.4)
    vel = u[:, None, :] * s[None, :, None]
    assert np.abs(w - synthetic.diagnose_w(m, vel)).max() <= 1e-12 * np.abs(w).max()
    assert synthetic.max_cfl(m, vel, 600.0) <= 0.4 + 1e-12
    zb = m.get("zbar")
    h = zb[:-1] - zb[1:]
    cv = np.abs(w[:, : m.nz]) * 600.0 / np.minimum(np.concatenate([h[:1], h[:-1]]), h)[None, :]
    assert cv.max() <= 0.4 + 1e-12


def _pi_pair(oracle_mod, pi_dir, **flags):
    return oracle_mod.Mesh.from_files(pi_dir, **flags), _mesh(pi_dir, **flags)


@pytest.mark.parametrize("schemes", [("UPW1", "UPW1", "NONE"), ("MUSCL", "PPM", "FCT")])
def test_oracle_zero_velocity_is_identity(oracle_mod, pi_dir, schemes):
    """The reference's mesh-from-files test steps with zero velocity."""
    om, m = _pi_pair(oracle_mod, pi_dir)
    nz = m.nz
    T = np.repeat((20.0 - 15.0 * np.arange(nz) / (nz - 1))[None, :], m.N, axis=0)
    vals = np.ascontiguousarray(np.stack([T, np.full_like(T, 35.0)]))
    before = vals.copy()
    W = oracle_mod.Work(om)
    for _ in range(5):
        oracle_mod.analytic_step(om, W, 1.0e-3, np.zeros((m.M, nz, 2)), np.zeros((m.N, m.nl)), vals, vals.copy(),
                                 [schemes + (1.0, 1.0)] * 2, copy_ab=True)
    assert np.array_equal(vals, before)


@pytest.mark.parametrize("schemes", [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT"), ("UPW1", "UPW1", "NONE")])
def test_oracle_uniform_stays_uniform(oracle_mod, pi_dir, schemes):
    from fesom2_tracer_dwarf_gb300 import synthetic

    om, m = _pi_pair(oracle_mod, pi_dir, euler_degrees=True, cyclic_2pi=True)
    rng = np.random.default_rng(31)
    vel = rng.uniform(-0.2, 0.2, size=(m.M, m.nz, 2))
    w = synthetic.diagnose_w(m, vel)
    vals = np.full((1, m.N, m.nz), 12.5)
    W = oracle_mod.Work(om)
    for _ in range(3):
        oracle_mod.analytic_step(om, W, 1800.0, vel, w, vals, vals.copy(), [schemes + (0.7, 0.6)], copy_ab=True)
    nlev = m.get("nlevels_nod2D")
    wet = np.arange(m.nz)[None, :] < (nlev - 1)[:, None]
    assert np.abs(vals[0][wet] - 12.5).max() <= 1e-12 * 12.5


torch = pytest.importorskip("torch")


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


SCHEMES = [("UPW1", "UPW1", "NONE"), ("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT"), ("MUSCL", "CDIFF", "NONE"),
           ("UPW1", "PPM", "FCT"), ("MFCT", "QR4C", "NONE")]


@pytest.mark.gpu
@pytest.mark.parametrize("flags,schemes", list(itertools.product([0, 1], SCHEMES)))
def test_step_on_pi_matches_oracle(oracle_mod, pi_dir, flags, schemes):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    kw = FLAGS[flags]
    om, m = oracle_mod.Mesh.from_files(pi_dir, **kw), _mesh(pi_dir, upload=True, **kw)
    rng = np.random.default_rng(zlib.crc32(f"pi/{flags}/{schemes}".encode()))
    vel, w = synthetic.random_flow(m, rng, umax=0.2, wmax=2e-5)
    T = synthetic.random_field(m, rng, 2)
    dt = 900.0
    sch = schemes + (0.7, 0.6)
    vals = np.ascontiguousarray(T.copy())
    W = oracle_mod.Work(om)
    for _ in range(3):
        oracle_mod.analytic_step(om, W, dt, vel, w, vals, vals.copy(), [sch] * 2, copy_ab=True)
    for precision in ("fp64", "fp32"):
        eng = engine.TracerAdvection(m, 2, precision, *schemes, ph=0.7, pv=0.6, copy_ab=True)
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
@pytest.mark.parametrize("schemes", [("MUSCL", "PPM", "FCT"), ("UPW1", "QR4C", "NONE")])
def test_step_on_refined_pi_matches_oracle(oracle_mod, pi_refined_dir, schemes):
    """The refined pi mesh (12126 nodes, Morton order) with a layered flow:
    FP64 bit for bit, FP32 within 1e-5, 4 tracers (one FP32 group of 4)."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    kw = FLAGS[1]
    om, m = oracle_mod.Mesh.from_files(pi_refined_dir, **kw), _mesh(pi_refined_dir, upload=True, **kw)
    rng = np.random.default_rng(zlib.crc32(f"pir/{schemes}".encode()))
    u, s, w = synthetic.layered_flow(m, rng, 900.0, cfl=0.5)
    vel = np.ascontiguousarray(u[:, None, :] * s[None, :, None])
    T = synthetic.random_field(m, rng, 4)
    sch = schemes + (1.0, 1.0)
    vals = np.ascontiguousarray(T.copy())
    W = oracle_mod.Work(om)
    for _ in range(3):
        oracle_mod.analytic_step(om, W, 900.0, vel, w, vals, vals.copy(), [sch] * 4, copy_ab=True)
    for precision in ("fp64", "fp32"):
        eng = engine.TracerAdvection(m, 4, precision, *schemes, copy_ab=True)
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
        eng.step(900.0, 3)
        torch.cuda.synchronize()
        got = eng.values()
        if precision == "fp64":
            assert np.array_equal(got, vals), f"max |diff| {np.abs(got - vals).max()}"
        else:
            assert np.abs(got - vals).max() <= 1e-5 * max(1.0, np.abs(vals).max())


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp64fast"])
def test_visit_order_changes_no_result(pi_refined_dir, precision):
    """The same steps with the Hilbert visit order and with file order give
    the same values bit for bit, in every form (each column and edge is
    computed once whatever the order)."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    kw = FLAGS[1]
    out = []
    for keep in (False, True):
        m = _mesh(pi_refined_dir, upload=True, keep_order=keep, **kw)
        rng = np.random.default_rng(31)
        u, s, w = synthetic.layered_flow(m, rng, 900.0, cfl=0.5)
        vel = np.ascontiguousarray(u[:, None, :] * s[None, :, None])
        T = synthetic.random_field(m, rng, 4)
        eng = engine.TracerAdvection(m, 4, precision, "MUSCL", "PPM", "FCT", copy_ab=True)
        eng.set_launch([0] * 9 + [1] if precision == "fp32" else [0] * 12)
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
        eng.step(900.0, 3)
        torch.cuda.synchronize()
        out.append(eng.values())
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
@pytest.mark.parametrize("schemes", [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT")])
def test_cabi_steps_on_pi_match_oracle(oracle_mod, pi_dir, schemes):
    """tracer_load_mesh_from_files + tracer_set_velocity on the pi mesh, three
    tracer_advect_step calls against the oracle's C-ABI step
    (lib/tracer_c_interface.F90:163-220 semantics), bit for bit."""
    _gpu()
    import ctypes

    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.demo_tracer import FESOMTracerAdvection

    om, m = oracle_mod.Mesh.from_files(pi_dir), _mesh(pi_dir)
    rng = np.random.default_rng(zlib.crc32(f"cabi-pi/{schemes}".encode()))
    vel, w = synthetic.random_flow(m, rng, umax=0.2, wmax=2e-5)
    T = synthetic.random_field(m, rng, 1)[0]
    nz, N, E = m.nz, m.N, m.E
    uv = np.zeros(nz * E * 2)
    flat = np.ascontiguousarray(vel).reshape(-1)  # vel(2, nz, M) in Fortran order
    uv[: flat.size] = flat
    t = FESOMTracerAdvection(verbose=False)
    t.cleanup()
    try:
        L = t.lib
        assert L.tracer_load_mesh_from_files(pi_dir.encode()) == 0
        nzc, nn = ctypes.c_int(), ctypes.c_int()
        assert L.tracer_get_size(ctypes.byref(nzc), ctypes.byref(nn)) == 0 and (nzc.value, nn.value) == (nz, N)
        assert t.allocate_tracers(1, m.nl, N) == 0
        assert t.set_values(1, np.asfortranarray(T.T)) == 0
        assert t.set_velocity(uv.reshape((nz, E, 2), order="F"), np.asfortranarray(w.T)) == 0
        assert t.set_schemes(1, *schemes) == 0
        assert t.init_ale_arrays() == 0 and t.init_for_advection() == 0 and t.init_complete() == 0
        vals = np.ascontiguousarray(T.copy())
        vab = vals.copy()
        del_ttf = np.zeros_like(vals)
        W = oracle_mod.Work(om)
        for step in range(3):
            assert t.advect_step(900.0) == 0
            oracle_mod.cabi_step(om, W, 900.0, vel, w, vals, vab, del_ttf, *schemes)
            got = t.get_tracer_values()
            assert np.array_equal(got.T, vals), f"step {step + 1}: max |diff| {np.abs(got.T - vals).max()}"
    finally:
        t.cleanup()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("mode", ["w_split", "ab2"])
def test_wsplit_and_ab2_on_pi(oracle_mod, pi_dir, precision, mode):
    """w_split (implicit vertical LO step, columns of 4..45 layers) and the AB2
    time level on the pi mesh, three steps against the oracle."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import engine, synthetic

    kw = FLAGS[1]
    om, m = oracle_mod.Mesh.from_files(pi_dir, **kw), _mesh(pi_dir, upload=True, **kw)
    rng = np.random.default_rng(zlib.crc32(f"pi-{mode}".encode()))
    u, s, w = synthetic.layered_flow(m, rng, 900.0, cfl=0.6)
    vel = np.ascontiguousarray(u[:, None, :] * s[None, :, None])
    T = synthetic.random_field(m, rng, 4)
    vals = np.ascontiguousarray(T.copy())
    W = oracle_mod.Work(om)
    if mode == "w_split":
        c = 0.25 * np.abs(w).max()
        we = np.clip(w, -c, c)
        wi = w - we
        sch = ("MUSCL", "PPM", "FCT")
        for _ in range(3):
            oracle_mod.analytic_step(om, W, 900.0, vel, w, vals, vals.copy(), [sch + (1.0, 1.0)] * 4, copy_ab=True,
                                     wi=wi, we=we)
        eng = engine.TracerAdvection(m, 4, precision, *sch, copy_ab=True)
        eng.set_tracers(T)
        eng.set_velocity(vel, w, we=we, wi=wi)
    else:
        sch = ("MFCT", "QR4C", "FCT")
        vab = vals.copy()
        for _ in range(3):
            oracle_mod.analytic_step(om, W, 900.0, vel, w, vals, vab, [sch + (1.0, 1.0)] * 4, ab2_eps=0.1)
        eng = engine.TracerAdvection(m, 4, precision, *sch, ab2_eps=0.1)
        eng.set_tracers(T)
        eng.set_velocity(vel, w)
    eng.step(900.0, 3)
    torch.cuda.synchronize()
    got = eng.values()
    if precision == "fp64":
        assert np.array_equal(got, vals), f"max |diff| {np.abs(got - vals).max()}"
    else:
        assert np.abs(got - vals).max() <= 1e-5 * max(1.0, np.abs(vals).max())


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_union_of_pi_and_grid(precision):
    """The batching form with a file mesh: the pi mesh and an analytic grid as
    one union mesh (layers padded to the pi mesh's 47) step as each does alone."""
    _gpu()
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection
    from fesom2_tracer_dwarf_gb300.mesh import Mesh

    d = load_pi()
    pi = Mesh.from_arrays(**{k: d[k] for k in ("lonlat", "elem", "edges", "edge_tri", "edgenum", "elvls", "nlvls",
                                                "zbar")}, euler_degrees=True, cyclic_2pi=True)
    grid = Mesh(14, 12, 10, periodic=True, orient_left=True)
    parts = [pi, grid]
    u = Mesh.union(parts)
    rng = np.random.default_rng(41)
    dt, K = 900.0, 4
    flows = [synthetic.layered_flow(pi, rng, dt, cfl=0.4), synthetic.streamfunction_flow(grid, rng, dt, cfl=0.3)]
    vel = [np.ascontiguousarray(flows[0][0][:, None, :] * flows[0][1][None, :, None]), flows[1][0]]
    w = [flows[0][2], flows[1][1]]
    T = [synthetic.random_field(p, rng, K) for p in parts]
    sch = ("MUSCL", "PPM", "FCT")
    eu = TracerAdvection(u, K, precision, *sch, copy_ab=True)
    eu.set_tracers(u.join_parts(T, axis=1, layer_axis=2))
    eu.set_velocity(u.join_parts(vel, layer_axis=1), u.join_parts(w, layer_axis=1, layers="nl"))
    eu.step(dt, 3)
    got = eu.values()
    for i, p in enumerate(parts):
        e = TracerAdvection(p, K, precision, *sch, copy_ab=True)
        e.set_tracers(T[i])
        e.set_velocity(vel[i], w[i])
        e.step(dt, 3)
        ref = e.values()
        part = u.part_view(got, i, axis=1)[:, :, : p.nz]
        if precision == "fp64":
            assert np.array_equal(part, ref), f"part {i}"
        else:
            assert np.abs(part - ref).max() <= 1e-6 * np.abs(ref).max(), f"part {i}"


@pytest.mark.gpu
def test_reference_mesh_from_files_workflow(oracle_mod, pi_dir):
    """python/test_mesh_from_files.py through the C ABI: load the pi mesh,
    allocate T and S, zero velocity, 5 steps of dt = 1e-3, statistics."""
    _gpu()
    import ctypes

    from fesom2_tracer_dwarf_gb300.demo_tracer import FESOMTracerAdvection

    t = FESOMTracerAdvection(verbose=False)
    t.cleanup()
    try:
        L = t.lib
        assert t.initialize_mpi(0) == 0
        assert L.tracer_load_mesh_from_files(pi_dir.encode()) == 0
        nz, nn = ctypes.c_int(), ctypes.c_int()
        assert L.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn)) == 0
        assert (nz.value + 1, nn.value) == (48, 3140)
        nl, nod2D = nz.value + 1, nn.value
        assert t.allocate_tracers(2, nl, nod2D, 2) == 0
        temp = np.zeros((nz.value, nod2D), order="F")
        for k in range(nz.value):
            temp[k, :] = 20.0 - 15.0 * k / max(1, nz.value - 1)
        assert t.set_values(1, temp) == 0
        assert t.set_values(2, np.full((nz.value, nod2D), 35.0, order="F")) == 0
        assert L.tracer_set_velocity_zero(nl, nod2D, 3 * nod2D) == 0
        assert t.init_ale_arrays() == 0 and t.init_for_advection() == 0 and t.init_complete() == 0
        om = oracle_mod.Mesh.from_files(pi_dir)
        ref = om.stats(np.ascontiguousarray(temp.T))
        for _ in range(5):
            assert t.advect_step(1.0e-3) == 0
            st = t.get_statistics()
            assert st["min"] == ref[0] and st["max"] == ref[1]
            assert abs(st["sum"] - ref[2]) <= 1e-12 * abs(ref[2])
        assert np.array_equal(t.get_tracer_values(), temp)
        assert t.finalize_mpi() == 0
    finally:
        t.cleanup()
