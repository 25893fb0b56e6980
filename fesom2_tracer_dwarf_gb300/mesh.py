"""Meshes of the tracer step: host set-up in the library, uploaded to the GPU.

``Mesh`` builds the analytic mesh of the reference dwarf
(lib/analytic_mesh.F90:114-829 with the geometry of lib/oce_mesh.F90) through
``fgb_hmesh_analytic``, or reads a FESOM mesh directory (``Mesh.from_files``,
``fgb_hmesh_from_files``), and uploads it with ``fgb_mesh_create``. Arrays are
returned 0-based as ``(outer, inner)`` numpy arrays, e.g. ``area[node, level]``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_SHAPES2 = {
    "elem_nodes": 3, "edges": 2, "edge_tri": 2, "edge_up_dn_tri": 2, "edge_lev": 4, "edge_gm": 2, "coord": 2,
    "edge_dxdy": 2, "edge_cross_dxdy": 4, "gradient_sca": 6, "edge_dxa": 2,
}


class Mesh:
    """Host mesh plus (optionally) its device copy.

    cluster_full and orient_left select the two documented corrections of the
    reference's analytic mesh (see fgb_hmesh_analytic in the C header); the
    defaults reproduce the reference mesh exactly. hilbert=True makes the
    kernels visit node columns along a Hilbert curve (the order of the work
    only; file meshes do so unless keep_order=True)."""

    def __init__(self, nx: int, ny: int, nl: int, Lx: float = 100000.0, Ly: float = 100000.0,
                 depth: float = 1000.0, periodic: bool = True, cluster_full: bool = False,
                 orient_left: bool = False, zbar=None, elem_nlev=None, upload: bool = True, hilbert: bool = False):
        L = _lib.load()
        self.nx, self.ny, self.Lx, self.Ly, self.depth = nx, ny, Lx, Ly, depth
        self.periodic, self.cluster_full, self.orient_left = periodic, cluster_full, orient_left
        flags = (1 if cluster_full else 0) | (2 if orient_left else 0) | (4 if hilbert else 0)
        zb = None if zbar is None else np.ascontiguousarray(zbar, dtype=np.float64)
        en = None if elem_nlev is None else np.ascontiguousarray(elem_nlev, dtype=np.int32)
        h = ctypes.c_void_p()
        rc = L.fgb_hmesh_analytic(nx, ny, nl, Lx, Ly, depth, int(periodic), flags,
                                  None if zb is None else zb.ctypes.data_as(_lib._dp),
                                  None if en is None else en.ctypes.data_as(_lib._ip), ctypes.byref(h))
        _lib.check(rc, "fgb_hmesh_analytic")
        self.parts = None
        self._attach(h, upload)

    def _attach(self, h, upload):
        L = _lib.load()
        self._h = h
        s = (ctypes.c_longlong * 8)()
        _lib.check(L.fgb_hmesh_sizes(h, s), "fgb_hmesh_sizes")
        self.N, self.E, self.M, self.nl, self.max_nie, self.edge2D_in = (int(v) for v in s[:6])
        self.nz = self.nl - 1
        self.LZ, self.LW = (self.nz + 3) // 4 * 4, (self.nl + 3) // 4 * 4  # padded layers / interfaces
        self._d = None
        if upload:
            self.upload()

    @classmethod
    def from_files(cls, path: str, rotate: bool = True, euler_degrees: bool = False, cyclic_2pi: bool = False,
                   upload: bool = True, keep_order: bool = False) -> "Mesh":
        """A FESOM mesh directory (nod2d.out, elem2d.out, aux3d.out,
        edgenum.out, edges.out, edge_tri.out, elvls.out, nlvls.out) as one
        partition, set up as lib/oce_mesh.F90 mesh_setup does on the sphere.
        The defaults are the reference's (rotation with the Euler angles
        50/15/-90 used as given, cyclic_length 360 against radians);
        euler_degrees and cyclic_2pi select FESOM2's namelist handling. The
        kernels visit node columns along a Hilbert curve through the node
        coordinates (keep_order=True: in file order); numbering, layouts and
        results are the file's either way."""
        L = _lib.load()
        flags = (0 if rotate else 1) | (2 if euler_degrees else 0) | (4 if cyclic_2pi else 0) | (8 if keep_order else 0)
        h = ctypes.c_void_p()
        _lib.check(L.fgb_hmesh_from_files(str(path).encode(), flags, ctypes.byref(h)), "fgb_hmesh_from_files")
        self = cls.__new__(cls)
        self.nx = self.ny = None
        self.Lx = self.Ly = self.depth = None
        self.periodic, self.cluster_full, self.orient_left = False, False, False
        self.path = str(path)
        self.parts = None
        self._attach(h, upload)
        return self

    @classmethod
    def from_arrays(cls, lonlat, elem, edges, edge_tri, edgenum, elvls, nlvls, zbar, rotate: bool = True,
                    euler_degrees: bool = False, cyclic_2pi: bool = False, upload: bool = True,
                    keep_order: bool = False) -> "Mesh":
        """The same as ``from_files`` from arrays laid out as the files are
        (``fgb_hmesh_from_arrays``; e.g. ``meshfiles.refine`` output)."""
        L = _lib.load()
        flags = (0 if rotate else 1) | (2 if euler_degrees else 0) | (4 if cyclic_2pi else 0) | (8 if keep_order else 0)
        i32 = [np.ascontiguousarray(a, dtype=np.int32) for a in (elem, edges, edge_tri, elvls, nlvls)]
        ll = np.ascontiguousarray(lonlat, dtype=np.float64)
        zb = np.ascontiguousarray(zbar, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = L.fgb_hmesh_from_arrays(len(ll), len(i32[0]), int(edgenum[0]), int(edgenum[1]), len(zb),
                                     ll.ctypes.data_as(_lib._dp), *[a.ctypes.data_as(_lib._ip) for a in i32],
                                     zb.ctypes.data_as(_lib._dp), flags, ctypes.byref(h))
        _lib.check(rc, "fgb_hmesh_from_arrays")
        self = cls.__new__(cls)
        self.nx = self.ny = None
        self.Lx = self.Ly = self.depth = None
        self.periodic, self.cluster_full, self.orient_left = False, False, False
        self.parts = None
        self._attach(h, upload)
        return self

    @classmethod
    def union(cls, parts, upload: bool = True) -> "Mesh":
        """Disjoint union of independent meshes (``fgb_hmesh_union``), one
        mesh that a single launch per stage advances. ``parts`` keeps, per
        part, its node/edge/element offsets and layer count (``part_view``)."""
        L = _lib.load()
        arr = (ctypes.c_void_p * len(parts))(*[p._h.value for p in parts])
        h = ctypes.c_void_p()
        _lib.check(L.fgb_hmesh_union(arr, len(parts), ctypes.byref(h)), "fgb_hmesh_union")
        self = cls.__new__(cls)
        self.nx = self.ny = None
        self.Lx = self.Ly = self.depth = None
        self.periodic = all(p.periodic for p in parts)
        self.cluster_full, self.orient_left = parts[0].cluster_full, parts[0].orient_left
        offs, no, eo, mo = [], 0, 0, 0
        for p in parts:
            offs.append(dict(node=no, edge=eo, elem=mo, N=p.N, E=p.E, M=p.M, nz=p.nz, nl=p.nl))
            no, eo, mo = no + p.N, eo + p.E, mo + p.M
        self.parts = offs
        self._attach(h, upload)
        return self

    def join_parts(self, arrays, axis: int = 0, layer_axis: int | None = None, layers: str = "nz"):
        """Concatenate one array per part along the part axis (nodes or
        elements: axis 0, or 1 for (K, N, nz) tracer stacks), zero-padding the
        layer axis to this mesh's nz (layers="nz") or nl ("nl")."""
        width = self.nz if layers == "nz" else self.nl
        out = []
        for a in arrays:
            a = np.asarray(a)
            if layer_axis is not None:
                pad = [(0, 0)] * a.ndim
                pad[layer_axis] = (0, width - a.shape[layer_axis])
                a = np.pad(a, pad)
            out.append(a)
        return np.concatenate(out, axis=axis)

    def part_view(self, a, i: int, kind: str = "node", axis: int = 0):
        """Part i's slice of a node or element array of this union mesh."""
        p = self.parts[i]
        lo, n = (p["node"], p["N"]) if kind == "node" else (p["elem"], p["M"])
        idx = [slice(None)] * np.ndim(a)
        idx[axis] = slice(lo, lo + n)
        return a[tuple(idx)]

    # ---- host arrays -------------------------------------------------------
    def get(self, name: str) -> np.ndarray:
        L = _lib.load()
        kind = ctypes.c_int()
        n = L.fgb_hmesh_get(self._h, name.encode(), None, ctypes.byref(kind))
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n, np.int32 if kind.value == 0 else np.float64)
        L.fgb_hmesh_get(self._h, name.encode(), out.ctypes.data_as(ctypes.c_void_p), None)
        if name in _SHAPES2:
            return out.reshape(-1, _SHAPES2[name])
        if name == "nod_in_elem2D":
            return out.reshape(self.N, self.max_nie)
        if name in ("area", "areasvol", "zbar_3d_n"):
            return out.reshape(self.N, self.nl)
        if name in ("hnode", "hnode_new", "Z_3d_n"):
            return out.reshape(self.N, self.nz)
        if name == "helem":
            return out.reshape(self.M, self.nz)
        return out

    def set_vertical(self, hnode=None, hnode_new=None, helem=None):
        """Replace the layer thicknesses (host and device)."""
        L = _lib.load()
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (hnode, hnode_new, helem)]
        ptrs = [None if a is None else a.ctypes.data_as(_lib._dp) for a in arrs]
        _lib.check(L.fgb_hmesh_set_vertical(self._h, *ptrs), "fgb_hmesh_set_vertical")
        if self._d is not None:
            _lib.check(L.fgb_mesh_update_vertical(self._d, self._h), "fgb_mesh_update_vertical")

    # ---- device ------------------------------------------------------------
    def upload(self):
        if self._d is not None:
            return self._d
        L = _lib.load()
        d = ctypes.c_void_p()
        _lib.check(L.fgb_mesh_create(self._h, ctypes.byref(d)), "fgb_mesh_create")
        self._d = d
        dims = (ctypes.c_int * 8)()
        _lib.check(L.fgb_mesh_dims(d, dims), "fgb_mesh_dims")
        self.LZ, self.LW, self.min_layers = int(dims[5]), int(dims[6]), int(dims[7])
        return d

    @property
    def handle(self):
        return self.upload()

    def wet_cells(self) -> int:
        """Layers summed over the node columns (the unit of tracer-cell updates)."""
        return int((self.get("nlevels_nod2D") - self.get("ulevels_nod2D")).sum())

    def close(self):
        L = _lib._lib
        if L is None:
            return
        if self._d is not None:
            L.fgb_mesh_free(self._d)
            self._d = None
        if self._h is not None:
            L.fgb_hmesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
