"""Batching form: several independent meshes of uneven size and depth as one
disjoint-union mesh advanced by one launch per stage, and whole steps
captured as a CUDA graph.

The union keeps every part's gather order, so the FP64 union step equals the
per-part steps bit for bit.
"""
import numpy as np
import pytest

from fesom2_tracer_dwarf_gb300.mesh import Mesh

PARTS = [dict(nx=10, ny=8, nl=6), dict(nx=13, ny=11, nl=9), dict(nx=9, ny=12, nl=12)]


def _parts(upload=False, **extra):
    return [Mesh(**p, periodic=True, orient_left=True, upload=upload, **extra) for p in PARTS]


def test_union_tables_are_shifted_part_tables():
    parts = _parts()
    u = Mesh.union(parts, upload=False)
    assert u.N == sum(p.N for p in parts) and u.E == sum(p.E for p in parts) and u.nl == 12
    ne_ptr, code, other = u.get("ne_ptr"), u.get("ne_code"), u.get("ne_other")
    cl_ptr, cl_node, cl_lev = u.get("cl_ptr"), u.get("cl_node"), u.get("cl_lev")
    for i, p in enumerate(parts):
        o = u.parts[i]
        pp, pc, po = p.get("ne_ptr"), p.get("ne_code"), p.get("ne_other")
        j0 = ne_ptr[o["node"]]
        assert np.array_equal(ne_ptr[o["node"]: o["node"] + p.N + 1] - j0, pp)
        assert np.array_equal(code[j0: j0 + len(pc)], pc + 2 * o["edge"])
        assert np.array_equal(other[j0: j0 + len(po)], po + o["node"])
        c0 = cl_ptr[o["node"]]
        pcl = p.get("cl_node")
        assert np.array_equal(cl_node[c0: c0 + len(pcl)], pcl + o["node"])
        assert np.array_equal(cl_lev[c0: c0 + len(pcl)], p.get("cl_lev"))
        assert np.array_equal(u.part_view(u.get("nlevels_nod2D"), i), p.get("nlevels_nod2D"))
        assert np.array_equal(u.part_view(u.get("hnode"), i)[:, : p.nz], p.get("hnode"))
        assert np.all(u.part_view(u.get("hnode"), i)[:, p.nz:] == 0)


torch = pytest.importorskip("torch")


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _fields(parts, rng, dt, K):
    from fesom2_tracer_dwarf_gb300 import synthetic

    vel, w, T = [], [], []
    for i, p in enumerate(parts):
        v, ww = synthetic.streamfunction_flow(p, rng, dt, cfl=0.2 + 0.1 * i)
        vel.append(v)
        w.append(ww)
        T.append(synthetic.random_field(p, rng, K))
    return vel, w, T


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("sch", [("MUSCL", "QR4C", "FCT"), ("MFCT", "PPM", "FCT"), ("UPW1", "UPW1", "NONE")])
def test_union_step_equals_part_steps(precision, sch):
    _gpu()
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection

    parts = _parts(upload=True)
    u = Mesh.union(parts)
    rng = np.random.default_rng(31)
    dt, K = 300.0, 4
    vel, w, T = _fields(parts, rng, dt, K)
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
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_graph_replay_equals_eager_steps(precision):
    _gpu()
    from fesom2_tracer_dwarf_gb300 import synthetic
    from fesom2_tracer_dwarf_gb300.engine import TracerAdvection

    m = Mesh(24, 20, 10, periodic=True, orient_left=True)
    rng = np.random.default_rng(32)
    vel, w = synthetic.streamfunction_flow(m, rng, 300.0, cfl=0.4)
    T = synthetic.random_field(m, rng, 4)
    e = TracerAdvection(m, 4, precision, "MUSCL", "QR4C", "FCT", copy_ab=True)
    e.set_velocity(vel, w)
    e.set_tracers(T)
    g = e.capture(300.0, 5)
    e.set_tracers(T)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    got = e.values()
    ref = TracerAdvection(m, 4, precision, "MUSCL", "QR4C", "FCT", copy_ab=True)
    ref.set_velocity(vel, w)
    ref.set_tracers(T)
    ref.step(300.0, 10)
    assert np.array_equal(got, ref.values())
