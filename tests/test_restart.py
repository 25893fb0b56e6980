"""Derived-type binary restarts through the reference's C interface:
tracer_finalize writes <dir>/np1/t_mesh.0, t_partit.0, t_tracer.0,
t_dynamics.0 and <dir>/meta.time (write_all_bin_restarts,
lib/io_restart_derivedtype.F90:33-125), tracer_init and
tracer_load_mesh_partition read them (:132-199).

No Fortran compiler exists on these machines, so no file written by the
reference itself can be read here. The files are checked instead with an
independent reader in this test: one gfortran sequential unformatted record
per file (4-byte length markers, subrecords with signed markers), the
fields in the order of the types' WRITE(UNFORMATTED) procedures
(lib/MOD_MESH.F90:185-275, lib/MOD_PARTIT.F90:113-185,
lib/MOD_TRACER.F90:104-230, lib/MOD_DYN.F90:189-300), each allocatable
array as its extents followed by its elements in column-major order.

CPU: write -> parse -> read round trips of the host state (no device call);
records split into subrecords; truncated records, unknown schemes and
missing files refused with a message. GPU: steps interrupted by a
finalize/init round trip equal the uninterrupted steps bit for bit, del_ttf
included.
"""
import ctypes
import os
import shutil
import struct

import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300.demo_tracer import FESOMTracerAdvection

I4, R8, L4, C20 = "i4", "r8", "l4", "c20"

# (name, kind, rank) in the order of the reference's procedures
MESH = [("nod2D", I4, 0), ("ocean_area", R8, 0), ("ocean_areawithcav", R8, 0), ("edge2D", I4, 0),
        ("edge2D_in", I4, 0), ("elem2D", I4, 0), ("elem2D_nodes", I4, 2), ("edges", I4, 2), ("edge_tri", I4, 2),
        ("elem_edges", I4, 2), ("elem_area", R8, 1), ("edge_dxdy", R8, 2), ("edge_cross_dxdy", R8, 2),
        ("elem_cos", R8, 1), ("metric_factor", R8, 1), ("elem_neighbors", I4, 2), ("nod_in_elem2D", I4, 2),
        ("x_corners", R8, 2), ("y_corners", R8, 2), ("nod_in_elem2D_num", I4, 1), ("depth", R8, 1),
        ("gradient_vec", R8, 2), ("gradient_sca", R8, 2), ("bc_index_nod2D", I4, 1), ("nl", I4, 0),
        ("zbar", R8, 1), ("Z", R8, 1), ("elem_depth", R8, 1), ("ulevels", I4, 1), ("ulevels_nod2D", I4, 1),
        ("ulevels_nod2D_max", I4, 1), ("nlevels", I4, 1), ("nlevels_nod2D", I4, 1), ("nlevels_nod2D_min", I4, 1),
        ("area", R8, 2), ("area_inv", R8, 2), ("areasvol", R8, 2), ("areasvol_inv", R8, 2),
        ("mesh_resolution", R8, 1), ("cavity_flag_n", I4, 1), ("cavity_flag_e", I4, 1), ("cavity_depth", R8, 1),
        ("cavity_nrst_cavlpnt_xyz", R8, 2), ("ssh_dim", I4, 0), ("ssh_nza", I4, 0), ("ssh_rowptr", I4, 1),
        ("ssh_colind", I4, 1), ("ssh_values", R8, 1), ("ssh_colind_loc", I4, 1), ("ssh_rowptr_loc", I4, 1),
        ("lump2d_south", R8, 1), ("lump2d_north", R8, 1), ("ind_south", I4, 1), ("ind_north", I4, 1),
        ("nn_size", I4, 0), ("nn_num", I4, 1), ("nn_pos", I4, 2), ("hnode", R8, 2), ("hnode_new", R8, 2),
        ("zbar_3d_n", R8, 2), ("Z_3d_n", R8, 2), ("Z_3d_n_ib", R8, 2), ("helem", R8, 2),
        ("bottom_elem_thickness", R8, 1), ("bottom_node_thickness", R8, 1), ("dhe", R8, 1), ("hbar", R8, 1),
        ("hbar_old", R8, 1), ("zbar_n_bot", R8, 1), ("zbar_e_bot", R8, 1), ("zbar_n_srf", R8, 1),
        ("zbar_e_srf", R8, 1), ("coriolis", R8, 1), ("coriolis_node", R8, 1)]
COM = [("rPEnum", I4, 0), ("rPE", I4, 1), ("rptr", I4, 1), ("rlist", I4, 1), ("sPEnum", I4, 0), ("sPE", I4, 1),
       ("sptr", I4, 1), ("slist", I4, 1), ("nreq", I4, 0)]
PARTIT = ([(f"{c}%{n}", k, r) for c in ("com_nod2D", "com_elem2D", "com_elem2D_full") for n, k, r in COM] +
          [("npes", I4, 0), ("mype", I4, 0), ("maxPEnum", I4, 0), ("part", I4, 1), ("myDim_nod2D", I4, 0),
           ("eDim_nod2D", I4, 0), ("myList_nod2D", I4, 1), ("myDim_elem2D", I4, 0), ("eDim_elem2D", I4, 0),
           ("eXDim_elem2D", I4, 0), ("myList_elem2D", I4, 1), ("myDim_edge2D", I4, 0), ("eDim_edge2D", I4, 0),
           ("myList_edge2D", I4, 1), ("pe_status", I4, 0)])
TRACER_DATA = [("values", R8, 2), ("valuesold", R8, 3), ("valuesAB", R8, 2), ("smooth_bh_tra", L4, 0),
               ("gamma0_tra", R8, 0), ("gamma1_tra", R8, 0), ("gamma2_tra", R8, 0), ("i_vert_diff", L4, 0),
               ("tra_adv_hor", C20, 0), ("tra_adv_ver", C20, 0), ("tra_adv_lim", C20, 0), ("tra_adv_ph", R8, 0),
               ("tra_adv_pv", R8, 0), ("ID", I4, 0)]
TRACER_WORK = [("del_ttf", R8, 2), ("del_ttf_advhoriz", R8, 2), ("del_ttf_advvert", R8, 2),
               ("dvd_trflx_hor", R8, 3), ("dvd_trflx_ver", R8, 3), ("fct_LO", R8, 2), ("adv_flux_hor", R8, 2),
               ("adv_flux_ver", R8, 2), ("fct_ttf_max", R8, 2), ("fct_ttf_min", R8, 2), ("fct_plus", R8, 2),
               ("fct_minus", R8, 2), ("edge_up_dn_grad", R8, 3), ("nboundary_lay", I4, 1),
               ("edge_up_dn_tri", I4, 2)]
DYN = [("opt_visc", I4, 0), ("visc_gamma0", R8, 0), ("visc_gamma1", R8, 0), ("visc_gamma2", R8, 0),
       ("visc_easybsreturn", R8, 0), ("use_ivertvisc", L4, 0), ("momadv_opt", I4, 0), ("use_freeslip", L4, 0),
       ("use_wsplit", L4, 0), ("wsplit_maxcfl", R8, 0), ("use_ssh_se_subcycl", L4, 0), ("ident", I4, 0),
       ("maxiter", I4, 0), ("restart", I4, 0), ("fillin", I4, 0), ("lutype", I4, 0), ("droptol", R8, 0),
       ("soltol", R8, 0), ("rr", R8, 1), ("zz", R8, 1), ("pp", R8, 1), ("App", R8, 1), ("uvnode_rhs", R8, 3),
       ("u_c", R8, 2), ("v_c", R8, 2), ("u_b", R8, 2), ("v_b", R8, 2), ("uv", R8, 3), ("uv_rhs", R8, 3),
       ("uv_rhsAB", R8, 4), ("uvnode", R8, 3), ("w", R8, 2), ("w_e", R8, 2), ("w_i", R8, 2), ("cfl_z", R8, 2)]


def read_record(path):
    """The payload of the one sequential unformatted record a file holds."""
    b = open(path, "rb").read()
    out, pos = bytearray(), 0
    while True:
        (lead,) = struct.unpack_from("<i", b, pos)
        n = abs(lead)
        out += b[pos + 4: pos + 4 + n]
        (trail,) = struct.unpack_from("<i", b, pos + 4 + n)
        assert abs(trail) == n
        pos += 8 + n
        if lead >= 0:
            break
    assert pos == len(b), "one record per file"
    return bytes(out)


def frame(payload, max_sub):
    """A record split into subrecords of at most max_sub bytes."""
    chunks = [payload[i: i + max_sub] for i in range(0, len(payload), max_sub)] or [b""]
    out = bytearray()
    for i, c in enumerate(chunks):
        lead = -len(c) if i + 1 < len(chunks) else len(c)
        trail = -len(c) if i > 0 else len(c)
        out += struct.pack("<i", lead) + c + struct.pack("<i", trail)
    return bytes(out)


class Parser:
    def __init__(self, b):
        self.b, self.p = b, 0

    def take(self, fmt, n=1):
        v = struct.unpack_from("<" + fmt * n, self.b, self.p)
        self.p += struct.calcsize("<" + fmt * n)
        return v

    def field(self, kind, rank):
        if rank == 0:
            if kind == C20:
                s = self.b[self.p: self.p + 20].decode()
                self.p += 20
                return s
            return self.take({I4: "i", L4: "i", R8: "d"}[kind])[0]
        dims = list(self.take("i", rank))
        n = int(np.prod(dims)) if all(d > 0 for d in dims) else 0
        dt = np.dtype("<i4" if kind == I4 else "<f8")
        a = np.frombuffer(self.b, dtype=dt, count=n, offset=self.p).copy()
        self.p += n * dt.itemsize
        return a.reshape(dims, order="F") if n else np.zeros([0] * rank, dt)

    def fields(self, spec, prefix=""):
        return {prefix + name: self.field(kind, rank) for name, kind, rank in spec}


def parse_tracer(b):
    p = Parser(b)
    out = {"num_tracers": p.field(I4, 0)}
    for t in range(out["num_tracers"]):
        out.update(p.fields(TRACER_DATA, f"data({t + 1})%"))
    out.update(p.fields(TRACER_WORK, "work%"))
    assert p.p == len(b)
    return out


def parse(spec, b):
    p = Parser(b)
    out = p.fields(spec)
    assert p.p == len(b), f"{len(b) - p.p} bytes left"
    return out


@pytest.fixture()
def tracer():
    t = FESOMTracerAdvection(verbose=False)
    t.cleanup()
    yield t
    t.cleanup()


def _state(t, nx=10, ny=9, nl=7, schemes=("MUSCL", "QR4C", "FCT"), seed=5):
    """An analytic-mesh state with 2 tracers and a velocity, host side only."""
    assert t.generate_analytic_mesh(nx, ny, nl, periodic=True) == 0
    nz, N, E = nl - 1, t.nod2D, t.edge2D
    rng = np.random.default_rng(seed)
    assert t.allocate_tracers(2, nl, N) == 0
    vals = [np.asfortranarray(rng.uniform(1, 2, (nz, N))), np.asfortranarray(rng.uniform(30, 35, (nz, N)))]
    for i, v in enumerate(vals):
        assert t.set_values(i + 1, v) == 0
    assert t.set_schemes(1, *schemes, 0.7, 0.6) == 0
    uv = np.asfortranarray(rng.uniform(-0.1, 0.1, (nz, E, 2)))
    w = np.asfortranarray(rng.uniform(-1e-5, 1e-5, (nl, N)))
    assert t.set_velocity(uv, w) == 0
    return vals, uv, w


def test_written_files_follow_the_procedures(tracer, tmp_path):
    vals, uv, w = _state(tracer)
    nl, N, M, E = 7, tracer.nod2D, tracer.elem2D, tracer.edge2D
    assert tracer.finalize(str(tmp_path)) == 0
    d = tmp_path / "np1"
    assert sorted(os.listdir(d)) == ["t_dynamics.0", "t_mesh.0", "t_partit.0", "t_tracer.0"]
    meta = open(tmp_path / "meta.time").read().split("\n")
    assert meta[:3] == ["0", "0", "! year: 0"] and "!   t_tracer" in meta and "!   t_dynamics" in meta
    tr = parse_tracer(read_record(d / "t_tracer.0"))
    assert tr["num_tracers"] == 2
    for i in range(2):
        assert np.array_equal(tr[f"data({i + 1})%values"], vals[i])
        assert np.array_equal(tr[f"data({i + 1})%valuesAB"], vals[i])
        assert tr[f"data({i + 1})%valuesold"].size == 0
    assert tr["data(1)%tra_adv_hor"] == "MUSCL".ljust(20) and tr["data(1)%tra_adv_lim"] == "FCT".ljust(20)
    assert tr["data(2)%tra_adv_ver"] == "UPW1".ljust(20)
    assert (tr["data(1)%tra_adv_ph"], tr["data(1)%tra_adv_pv"]) == (0.7, 0.6)
    assert tr["work%del_ttf"].shape == (nl - 1, N) and not tr["work%del_ttf"].any()
    assert tr["work%edge_up_dn_tri"].shape == (2, E) and tr["work%nboundary_lay"].shape == (N,)
    mesh = parse(MESH, read_record(d / "t_mesh.0"))
    assert (mesh["nod2D"], mesh["elem2D"], mesh["edge2D"], mesh["nl"]) == (N, M, E, nl)
    assert mesh["elem2D_nodes"].shape == (3, M) and mesh["elem2D_nodes"].min() == 1 and mesh["elem2D_nodes"].max() == N
    assert mesh["area"].shape == (nl, N) and mesh["hnode"].shape == (nl - 1, N) and mesh["helem"].shape == (nl - 1, M)
    assert mesh["ocean_area"] == pytest.approx(mesh["area"][0].sum())
    assert mesh["coriolis"].size == 0 and mesh["ssh_dim"] == 0
    part = parse(PARTIT, read_record(d / "t_partit.0"))
    assert (part["npes"], part["mype"], part["myDim_nod2D"], part["eDim_nod2D"]) == (1, 0, N, 0)
    assert np.array_equal(part["myList_nod2D"], np.arange(1, N + 1))
    assert part["com_nod2D%rPE"].shape == (32,) and part["com_nod2D%rptr"].shape == (33,)
    dyn = parse(DYN, read_record(d / "t_dynamics.0"))
    assert dyn["uv"].shape == (2, nl - 1, M)
    # the step reads tracer_set_velocity's (nl-1, edge2D, 2) memory as vel(2, nl-1, elem2D)
    assert np.array_equal(dyn["uv"].reshape(-1, order="F"), uv.reshape(-1, order="F")[: 2 * (nl - 1) * M])
    assert np.array_equal(dyn["w"], w) and not dyn["w_e"].any() and not dyn["w_i"].any()
    assert (dyn["opt_visc"], dyn["maxiter"], dyn["use_wsplit"], dyn["use_ssh_se_subcycl"]) == (5, 2000, 0, 0)


def test_init_reads_back_what_finalize_wrote(tracer, tmp_path):
    vals, uv, w = _state(tracer)
    a, b = tmp_path / "a", tmp_path / "b"
    assert tracer.finalize(str(a)) == 0
    tracer.cleanup()
    assert tracer.initialize(str(a)) == 0
    nz, nn = ctypes.c_int(), ctypes.c_int()
    assert tracer.lib.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn)) == 0
    assert (nz.value, nn.value) == vals[0].shape
    assert np.array_equal(tracer.get_tracer_values(), vals[0])
    # written again unchanged: the same bytes
    assert tracer.finalize(str(b)) == 0
    for f in ("t_mesh.0", "t_partit.0", "t_tracer.0", "t_dynamics.0"):
        assert open(a / "np1" / f, "rb").read() == open(b / "np1" / f, "rb").read(), f
    # the mesh alone
    tracer.cleanup()
    assert tracer.lib.tracer_load_mesh_partition(str(a).encode()) == 0
    assert tracer.lib.tracer_get_size(ctypes.byref(nz), ctypes.byref(nn)) == 0
    assert (nz.value, nn.value) == vals[0].shape


def test_records_split_into_subrecords(tracer, tmp_path):
    vals, _, _ = _state(tracer)
    assert tracer.finalize(str(tmp_path)) == 0
    for f in ("t_tracer.0", "t_mesh.0"):
        p = tmp_path / "np1" / f
        payload = read_record(p)
        open(p, "wb").write(frame(payload, 1000))
        assert read_record(p) == payload
    tracer.cleanup()
    assert tracer.initialize(str(tmp_path)) == 0
    assert np.array_equal(tracer.get_tracer_values(), vals[0])


def test_bad_restarts_are_refused(tracer, tmp_path):
    _state(tracer)
    assert tracer.finalize(str(tmp_path)) == 0
    tracer.cleanup()
    good = tmp_path / "good"
    shutil.copytree(tmp_path / "np1", good / "np1")
    L = tracer.lib
    last = lambda: L.fgb_last_error().decode()  # noqa: E731
    # truncated record
    p = tmp_path / "np1" / "t_tracer.0"
    payload = read_record(p)
    open(p, "wb").write(frame(payload[:-16], 1 << 30))
    assert tracer.initialize(str(tmp_path)) == -1 and "t_tracer" in last()
    # an unknown scheme (the reference aborts, lib/oce_adv_tra_driver.F90:252-254)
    bad = payload.replace(b"MUSCL".ljust(20), b"WENO5".ljust(20), 1)
    assert bad != payload
    open(p, "wb").write(frame(bad, 1 << 30))
    assert tracer.initialize(str(tmp_path)) == -1 and "Unknown horizontal advection type" in last()
    # extents whose product exceeds the record (data(1)%values: the two extents after num_tracers)
    huge = payload[:4] + struct.pack("<ii", 2 ** 30, 2 ** 30) + payload[12:]
    open(p, "wb").write(frame(huge, 1 << 30))
    assert tracer.initialize(str(tmp_path)) == -1 and "t_tracer" in last()
    # a missing file
    os.remove(p)
    assert tracer.initialize(str(tmp_path)) == -1 and "t_tracer" in last()
    # the missing directory: the reference's message (:136-141)
    assert tracer.initialize(str(tmp_path / "nowhere")) == -1
    assert "could not find restart directory" in last()
    assert tracer.initialize(str(good)) == 0


torch = pytest.importorskip("torch")


@pytest.mark.gpu
@pytest.mark.parametrize("schemes", [("MUSCL", "QR4C", "FCT"), ("UPW1", "PPM", "NONE")])
def test_steps_continue_across_a_restart(tracer, tmp_path, schemes):
    """3 steps, finalize, cleanup, init, 3 more steps == 6 steps, bit for bit
    (FP64), including del_ttf, which the reference's step accumulates."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")

    def setup():
        _state(tracer, nx=14, ny=12, nl=9, schemes=schemes, seed=11)
        assert tracer.init_for_advection() == 0 and tracer.init_complete() == 0

    setup()
    for _ in range(6):
        assert tracer.advect_step(60.0) == 0
    want = tracer.get_tracer_values()
    tracer.cleanup()
    setup()
    for _ in range(3):
        assert tracer.advect_step(60.0) == 0
    assert tracer.finalize(str(tmp_path)) == 0
    tracer.cleanup()
    assert tracer.initialize(str(tmp_path)) == 0
    for _ in range(3):
        assert tracer.advect_step(60.0) == 0
    got = tracer.get_tracer_values()
    assert np.array_equal(got, want), f"max |diff| {np.abs(got - want).max()}"
    tr = parse_tracer(read_record(tmp_path / "np1" / "t_tracer.0"))
    assert tr["work%del_ttf"].any()  # the accumulated tendency was carried over


@pytest.mark.gpu
def test_run_workflow_from_a_restart(tracer, tmp_path):
    """tracer_run_workflow(dir, nsteps, dt) (lib/tracer_c_interface.F90:356-388):
    tracer_init from dir, nsteps steps with statistics, tracer_finalize back
    into dir; the restart it leaves equals stepping the same state by hand."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    _state(tracer, nx=12, ny=11, nl=8, schemes=("MFCT", "PPM", "FCT"), seed=13)
    a, b = tmp_path / "a", tmp_path / "b"
    assert tracer.finalize(str(a)) == 0
    shutil.copytree(a, b)
    tracer.cleanup()
    assert tracer.lib.tracer_run_workflow(str(a).encode(), 4, 120.0) == 0
    tracer.cleanup()
    assert tracer.initialize(str(b)) == 0
    for _ in range(4):
        assert tracer.advect_step(120.0) == 0
    assert tracer.finalize(str(b)) == 0
    ta, tb = (parse_tracer(read_record(d / "np1" / "t_tracer.0")) for d in (a, b))
    assert np.array_equal(ta["data(1)%values"], tb["data(1)%values"])
    assert np.array_equal(ta["work%del_ttf"], tb["work%del_ttf"]) and ta["work%del_ttf"].any()
