"""FESOM mesh directories as numpy arrays: write one, and refine one.

The library reads mesh directories itself (``Mesh.from_files``,
``tracer_load_mesh_from_files``); this module produces them:

- ``write_fesom_dir`` writes nod2d.out, elem2d.out, aux3d.out, edgenum.out,
  edges.out, edge_tri.out, elvls.out and nlvls.out in the layouts
  lib/oce_mesh.F90 reads (1-based indices, interior edges first, 0 for a
  missing second element);
- ``refine`` splits every triangle into four at its great-circle edge
  midpoints (children keep the parent's vertex order and bottom level; node
  levels are the deepest adjacent element's, as in FESOM's nlvls.out), renumbers
  nodes along a Morton curve of (lon, lat) for locality, and rebuilds edges
  and edge_tri with edge_tri(1) on the left of node1 -> node2. Refining a
  real coastal mesh gives large unstructured test meshes with its coasts and
  bathymetry.

Arrays follow the files: ``lonlat`` (N, 2) degrees, ``elem`` (M, 3) 1-based,
``elvls`` (M), ``nlvls`` (N), ``zbar`` (nl), ``edges``/``edge_tri`` (E, 2)
1-based, ``edgenum`` (edge2D, edge2D_in).

    python -m fesom2_tracer_dwarf_gb300.meshfiles SRC_DIR DST_DIR TIMES
"""
from __future__ import annotations

import os

import numpy as np


def write_fesom_dir(path, lonlat, elem, zbar, edges, edge_tri, edgenum, elvls, nlvls, coast=None):
    """Write a FESOM mesh directory; floats as shortest round-trip decimals."""
    os.makedirs(path, exist_ok=True)
    N, M = len(lonlat), len(elem)
    coast = np.zeros(N, np.int64) if coast is None else np.asarray(coast)
    ids = np.arange(1, N + 1)

    def lines(fmt_rows):
        return "".join(fmt_rows)

    with open(os.path.join(path, "nod2d.out"), "w") as f:
        f.write(f"{N:8d}\n")
        f.write(lines(f"{i:8d} {float(x)!r} {float(y)!r} {int(c):8d}\n"
                      for i, x, y, c in zip(ids, lonlat[:, 0], lonlat[:, 1], coast)))
    with open(os.path.join(path, "elem2d.out"), "w") as f:
        f.write(f"{M:8d}\n")
        np.savetxt(f, np.asarray(elem, np.int64), fmt="%8d")
    with open(os.path.join(path, "aux3d.out"), "w") as f:
        f.write(f"{len(zbar)}\n")
        f.write(lines(f"{float(z)!r}\n" for z in zbar))
    with open(os.path.join(path, "edgenum.out"), "w") as f:
        f.write(f"{int(edgenum[0]):12d}\n{int(edgenum[1]):12d}\n")
    for name, arr in (("edges.out", edges), ("edge_tri.out", edge_tri)):
        with open(os.path.join(path, name), "w") as f:
            np.savetxt(f, np.asarray(arr, np.int64), fmt="%12d")
    for name, arr in (("elvls.out", elvls), ("nlvls.out", nlvls)):
        with open(os.path.join(path, name), "w") as f:
            np.savetxt(f, np.asarray(arr, np.int64).reshape(-1, 1), fmt="%12d")
    return path


def _xyz(lonlat):
    lon, lat = np.radians(lonlat[:, 0]), np.radians(lonlat[:, 1])
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], axis=1)


def _lonlat(xyz):
    xyz = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    return np.stack([np.degrees(np.arctan2(xyz[:, 1], xyz[:, 0])), np.degrees(np.arcsin(np.clip(xyz[:, 2], -1, 1)))],
                    axis=1)


def build_edges(elem0, xyz):
    """Edges of a triangle list (0-based elem0): interior edges first, each
    sorted by (lower node, upper node); edge_tri(1) is the element on the left
    of node1 -> node2 seen from outside the sphere, edge_tri(2) the other
    (-1 on the coast). Returns 0-based (edges, edge_tri, n_interior)."""
    M = len(elem0)
    a = elem0[:, [0, 1, 2]].reshape(-1)
    b = elem0[:, [1, 2, 0]].reshape(-1)
    t = np.repeat(np.arange(M), 3)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo.astype(np.int64) * (int(hi.max()) + 1) + hi
    order = np.argsort(key, kind="stable")
    key, lo, hi, t = key[order], lo[order], hi[order], t[order]
    first = np.ones(len(key), bool)
    first[1:] = key[1:] != key[:-1]
    start = np.flatnonzero(first)
    count = np.diff(np.append(start, len(key)))
    if count.max() > 2:
        raise ValueError("an edge is shared by more than two elements")
    e_lo, e_hi, t1 = lo[start], hi[start], t[start]
    t2 = np.where(count == 2, t[np.minimum(start + 1, len(t) - 1)], -1)

    # third vertex of t1: the element's node that is neither end of the edge
    def third(tt):
        v = elem0[tt]
        return np.where((v[:, 0] != e_lo) & (v[:, 0] != e_hi), v[:, 0],
                        np.where((v[:, 1] != e_lo) & (v[:, 1] != e_hi), v[:, 1], v[:, 2]))

    c = third(t1)
    left = np.einsum("ij,ij->i", np.cross(xyz[e_lo], xyz[e_hi]), xyz[c]) > 0
    n1 = np.where(left, e_lo, e_hi)
    n2 = np.where(left, e_hi, e_lo)
    edges = np.stack([n1, n2], axis=1)
    edge_tri = np.stack([t1, t2], axis=1)
    interior = t2 >= 0
    idx = np.concatenate([np.flatnonzero(interior), np.flatnonzero(~interior)])
    return edges[idx], edge_tri[idx], int(interior.sum())


def morton_order(lonlat, bits=16):
    """Node permutation along a Morton curve of (lon, lat)."""
    q = []
    for k in range(2):
        v = lonlat[:, k]
        span = max(float(v.max() - v.min()), 1e-300)
        q.append(np.minimum(((v - v.min()) / span * ((1 << bits) - 1)).astype(np.uint64), (1 << bits) - 1))
    code = np.zeros(len(lonlat), np.uint64)
    for bit in range(bits):
        for k in range(2):
            code |= ((q[k] >> np.uint64(bit)) & np.uint64(1)) << np.uint64(2 * bit + k)
    return np.argsort(code, kind="stable")


def refine(mesh, times=1):
    """Split each triangle into four, ``times`` times (see the module doc).
    ``mesh``: dict with lonlat, elem (1-based), elvls, zbar. Returns a dict
    ready for ``write_fesom_dir``."""
    lonlat = np.asarray(mesh["lonlat"], np.float64)
    elem0 = np.asarray(mesh["elem"], np.int64) - 1
    elvls = np.asarray(mesh["elvls"], np.int64)
    xyz = _xyz(lonlat)
    for _ in range(times):
        N, M = len(xyz), len(elem0)
        a = elem0[:, [0, 1, 2]].reshape(-1)
        b = elem0[:, [1, 2, 0]].reshape(-1)
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo * N + hi
        uniq, inv = np.unique(key, return_inverse=True)
        mid = N + inv.reshape(M, 3)  # midpoint node of edges (0-1), (1-2), (2-0)
        ulo, uhi = uniq // N, uniq % N
        pm = xyz[ulo] + xyz[uhi]
        xyz = np.concatenate([xyz, pm / np.linalg.norm(pm, axis=1, keepdims=True)])
        v0, v1, v2 = elem0[:, 0], elem0[:, 1], elem0[:, 2]
        m01, m12, m20 = mid[:, 0], mid[:, 1], mid[:, 2]
        kids = np.stack([np.stack([v0, m01, m20], 1), np.stack([m01, v1, m12], 1), np.stack([m20, m12, v2], 1),
                         np.stack([m01, m12, m20], 1)], axis=1)  # (M, 4, 3), parent's vertex order
        elem0 = kids.reshape(-1, 3)
        elvls = np.repeat(elvls, 4)
    ll = _lonlat(xyz)
    # keep the input's longitude convention (e.g. 0..360) where it had one
    if lonlat[:, 0].min() >= 0.0:
        ll[:, 0] = np.where(ll[:, 0] < 0.0, ll[:, 0] + 360.0, ll[:, 0])
    perm = morton_order(ll)
    rank = np.empty_like(perm)
    rank[perm] = np.arange(len(perm))
    ll, xyz = ll[perm], xyz[perm]
    elem0 = rank[elem0]
    eorder = np.argsort(elem0.min(axis=1), kind="stable")
    elem0, elvls = elem0[eorder], elvls[eorder]
    nlvls = np.zeros(len(ll), np.int64)
    np.maximum.at(nlvls, elem0.reshape(-1), np.repeat(elvls, 3))
    edges, edge_tri, n_in = build_edges(elem0, xyz)
    return dict(lonlat=ll, elem=elem0 + 1, elvls=elvls, nlvls=nlvls, zbar=np.asarray(mesh["zbar"], np.float64),
                edges=edges + 1, edge_tri=np.where(edge_tri >= 0, edge_tri + 1, 0),
                edgenum=np.array([len(edges), n_in]))


def read_fesom_dir(path):
    """The arrays ``refine`` takes, from a mesh directory (whitespace-separated
    items as the reference's list-directed reads take them)."""
    def items(name, dtype):
        with open(os.path.join(path, name)) as f:
            return np.array(f.read().split(), dtype=dtype)

    nod = items("nod2d.out", np.float64)
    N = int(nod[0])
    el = items("elem2d.out", np.int64)
    aux = items("aux3d.out", np.float64)
    nl = int(aux[0])
    return dict(lonlat=nod[1:1 + 4 * N].reshape(N, 4)[:, 1:3], elem=el[1:1 + 3 * int(el[0])].reshape(-1, 3),
                elvls=items("elvls.out", np.int64), zbar=aux[1:1 + nl])


def main(argv=None):
    import sys

    args = sys.argv[1:] if argv is None else argv
    if len(args) != 3:
        print(__doc__)
        return 2
    r = refine(read_fesom_dir(args[0]), int(args[2]))
    write_fesom_dir(args[1], r["lonlat"], r["elem"], r["zbar"], r["edges"], r["edge_tri"], r["edgenum"], r["elvls"],
                    r["nlvls"])
    print(f"{args[1]}: {len(r['lonlat'])} nodes, {len(r['elem'])} elements, {len(r['edges'])} edges")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
