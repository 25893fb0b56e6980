"""ctypes wrapper of the CPU oracle (test infrastructure only).

Imported by tests/, ``__graft_entry__.smoke()`` and bench.py's cpu_baseline leg
as the checker. The product package never imports this module.

Arrays follow the reference's Fortran layout with the level/component index
fastest; numpy arrays are returned with shape ``(outer, inner)`` in C order,
i.e. ``a[node, level]`` for an ``(nl-1, nod2D)`` Fortran array.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfesom_oracle.so")

HOR = {"UPW1": 0, "MUSCL": 1, "MFCT": 2}
VER = {"UPW1": 0, "QR4C": 1, "CDIFF": 2, "PPM": 3}
LIM = {"NONE": 0, "FCT": 1}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.om_mesh_analytic.restype = ctypes.c_void_p
        L.om_mesh_analytic.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _dp, _ip]
        L.om_mesh_analytic2.restype = ctypes.c_void_p
        L.om_mesh_analytic2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, _dp, _ip]
        L.om_mesh_from_arrays.restype = ctypes.c_void_p
        L.om_mesh_from_arrays.argtypes = [ctypes.c_int] * 5 + [_dp, _ip, _ip, _ip, _ip, _ip, _dp, ctypes.c_int]
        L.om_mesh_free.argtypes = [ctypes.c_void_p]
        L.om_mesh_sizes.argtypes = [ctypes.c_void_p, _ip]
        L.om_mesh_get_int.restype = ctypes.c_long
        L.om_mesh_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _ip]
        L.om_mesh_get_dbl.restype = ctypes.c_long
        L.om_mesh_get_dbl.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        L.om_work_new.restype = ctypes.c_void_p
        L.om_work_new.argtypes = [ctypes.c_void_p]
        L.om_work_free.argtypes = [ctypes.c_void_p]
        L.om_work_get.restype = ctypes.c_long
        L.om_work_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        L.om_do_oce_adv_tra.restype = ctypes.c_int
        L.om_do_oce_adv_tra.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp,
                                        _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.om_analytic_step.restype = ctypes.c_int
        L.om_analytic_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                       _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp, _dp, ctypes.c_int, _dp]
        L.om_analytic_step_split.restype = ctypes.c_int
        L.om_analytic_step_split.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                             _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp, _ip, _ip, _ip, _dp, _dp,
                                             ctypes.c_int, ctypes.c_double, _dp]
        L.om_cabi_step.restype = ctypes.c_int
        L.om_cabi_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp, _dp,
                                   _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, _dp]
        L.om_init_dwarf_fields.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp, _dp]
        L.om_stats.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.om_set_threads.argtypes = [ctypes.c_int]
        L.om_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    """Threads of the oracle's parallel loops; results do not depend on it."""
    lib().om_set_threads(int(n))


def get_threads() -> int:
    return int(lib().om_get_threads())


def _p(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def read_fesom_dir(path):
    """The files of a FESOM mesh directory the reference reads at one
    partition (lib/oce_mesh.F90:98-806, :807-1001, :1617-1848), parsed as
    whitespace-separated tokens: nod2d.out, elem2d.out, aux3d.out (levels),
    edgenum.out, edges.out, edge_tri.out, elvls.out, nlvls.out."""
    def toks(name):
        with open(os.path.join(path, name)) as f:
            return f.read().split()

    t = toks("nod2d.out")
    N = int(t[0])
    nod = np.array(t[1:1 + 4 * N], dtype=np.float64).reshape(N, 4)
    t = toks("elem2d.out")
    M = int(t[0])
    elem = np.array(t[1:1 + 3 * M], dtype=np.int64).astype(np.int32).reshape(M, 3)
    t = toks("aux3d.out")
    nl = int(t[0])
    zbar = np.array(t[1:1 + nl], dtype=np.float64)
    t = toks("edgenum.out")
    E, E_in = int(t[0]), int(t[1])
    edges = np.array(toks("edges.out")[:2 * E], dtype=np.int64).astype(np.int32).reshape(E, 2)
    edge_tri = np.array(toks("edge_tri.out")[:2 * E], dtype=np.int64).astype(np.int32).reshape(E, 2)
    elvls = np.array(toks("elvls.out")[:M], dtype=np.int64).astype(np.int32)
    nlvls = np.array(toks("nlvls.out")[:N], dtype=np.int64).astype(np.int32)
    return dict(lonlat=np.ascontiguousarray(nod[:, 1:3]), coast=nod[:, 3].astype(np.int32), elem=elem, nl=nl,
                zbar=zbar, edge2D=E, edge2D_in=E_in, edges=edges, edge_tri=edge_tri, elvls=elvls, nlvls=nlvls)


class Mesh:
    """A mesh built by the oracle: the analytic mesh (lib/analytic_mesh.F90),
    or a FESOM mesh from its files (``from_files``)."""

    def __init__(self, nx, ny, nl, Lx=100000.0, Ly=100000.0, depth=1000.0, periodic=True,
                 cluster_full=False, zbar=None, elem_nlev=None, orient_left=False):
        L = lib()
        zb = _f64(zbar) if zbar is not None else None
        en = np.ascontiguousarray(elem_nlev, dtype=np.int32) if elem_nlev is not None else None
        self._zb, self._en = zb, en
        h = L.om_mesh_analytic2(nx, ny, nl, Lx, Ly, depth, int(periodic), int(cluster_full),
                                int(orient_left), _p(zb), _p(en, _ip))
        if not h:
            raise ValueError("invalid analytic mesh parameters")
        self._attach(h)
        self.Lx, self.Ly, self.periodic = Lx, Ly, periodic

    def _attach(self, h):
        self.h = ctypes.c_void_p(h)
        s = np.zeros(7, np.int32)
        lib().om_mesh_sizes(self.h, _p(s, _ip))
        (self.nod2D, self.nod2D_total, self.elem2D, self.edge2D, self.edge2D_in, self.nl,
         self.max_nie) = (int(v) for v in s)

    @classmethod
    def from_files(cls, path, rotate=True, euler_degrees=False, cyclic_2pi=False):
        """A FESOM mesh directory (read_fesom_dir) through om_mesh_from_arrays."""
        return cls.from_arrays(read_fesom_dir(path), rotate, euler_degrees, cyclic_2pi)

    @classmethod
    def from_arrays(cls, d, rotate=True, euler_degrees=False, cyclic_2pi=False):
        """om_mesh_from_arrays on a dict laid out as the files are: lonlat,
        elem, edges, edge_tri, elvls, nlvls, zbar, and edge2D / edge2D_in (or
        edgenum)."""
        d = dict(d)
        if "edgenum" in d:
            d["edge2D"], d["edge2D_in"] = int(d["edgenum"][0]), int(d["edgenum"][1])
        d["nl"] = len(d["zbar"])
        flags = (0 if rotate else 1) | (2 if euler_degrees else 0) | (4 if cyclic_2pi else 0)
        arrs = [np.ascontiguousarray(d[k], dtype=np.int32) for k in ("elem", "edges", "edge_tri", "elvls", "nlvls")]
        lonlat = _f64(d["lonlat"])
        zb = _f64(d["zbar"])
        h = lib().om_mesh_from_arrays(len(d["nlvls"]), len(d["elvls"]), d["edge2D"], d["edge2D_in"], d["nl"],
                                      _p(lonlat), *[_p(a, _ip) for a in arrs], _p(zb), flags)
        if not h:
            raise ValueError("invalid mesh files")
        self = cls.__new__(cls)
        self._attach(h)
        self.Lx = self.Ly = 0.0
        self.periodic = False
        return self

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.om_mesh_free(self.h)
            self.h = None

    _INT_SHAPES = {"elem2D_nodes": 3, "edges": 2, "edge_tri": 2, "edge_up_dn_tri": 2}
    _DBL_SHAPES = {"coord": 2, "edge_dxdy": 2, "edge_cross_dxdy": 4, "gradient_sca": 6}

    def geti(self, name):
        L = lib()
        n = L.om_mesh_get_int(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n, np.int32)
        L.om_mesh_get_int(self.h, name.encode(), _p(out, _ip))
        if name in self._INT_SHAPES:
            out = out.reshape(-1, self._INT_SHAPES[name])
        elif name == "nod_in_elem2D":
            out = out.reshape(-1, self.max_nie)
        return out

    def getd(self, name):
        L = lib()
        n = L.om_mesh_get_dbl(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n, np.float64)
        L.om_mesh_get_dbl(self.h, name.encode(), _p(out))
        if name in self._DBL_SHAPES:
            out = out.reshape(-1, self._DBL_SHAPES[name])
        elif name in ("area", "areasvol", "zbar_3d_n"):
            out = out.reshape(-1, self.nl)
        elif name in ("hnode", "hnode_new", "helem", "Z_3d_n"):
            out = out.reshape(-1, self.nl - 1)
        return out

    def dwarf_fields(self):
        nz = self.nl - 1
        T = np.zeros((self.nod2D, nz))
        S = np.zeros((self.nod2D, nz))
        lib().om_init_dwarf_fields(self.h, self.Lx, self.Ly, _p(T), _p(S))
        return T, S

    def stats(self, values):
        out = np.zeros(4)
        lib().om_stats(self.h, _p(_f64(values)), _p(out))
        return out


class Work:
    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        self.h = ctypes.c_void_p(lib().om_work_new(mesh.h))

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.om_work_free(self.h)
            self.h = None

    def get(self, name):
        L = lib()
        n = L.om_work_get(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        L.om_work_get(self.h, name.encode(), _p(out))
        m = self.mesh
        if name in ("adv_flux_ver", "adf_v_raw"):
            return out.reshape(m.nod2D, m.nl)
        if name in ("adv_flux_hor", "adf_h_raw"):
            return out.reshape(m.edge2D, m.nl - 1)
        if name == "edge_up_dn_grad":
            return out.reshape(m.edge2D, m.nl - 1, 4)
        if name == "tr_xy":
            return out.reshape(m.elem2D, m.nl - 1, 2)
        return out.reshape(m.nod2D, m.nl - 1)


def do_oce_adv_tra(mesh, work, dt, vel, w, ttf, ttfAB, hor="UPW1", ver="UPW1", lim="NONE",
                   ph=1.0, pv=1.0, wi=None, we=None):
    """One call of do_oce_adv_tra; returns (dttf_h, dttf_v) as (nod2D, nl-1).

    wi given switches w_split on: the FCT low-order solution gets the implicit
    vertical step with wi (adv_tra_vert_impl); we (default w) is the explicit
    vertical velocity of the low-order flux."""
    vel, w, ttf, ttfAB = _f64(vel), _f64(w), _f64(ttf), _f64(ttfAB)
    split = wi is not None
    wi = w if wi is None else _f64(wi)
    we = w if we is None else _f64(we)
    dh = np.zeros((mesh.nod2D, mesh.nl - 1))
    dv = np.zeros_like(dh)
    rc = lib().om_do_oce_adv_tra(mesh.h, work.h, dt, _p(vel), _p(w), _p(wi), _p(we), _p(ttf), _p(ttfAB),
                                 HOR[hor], VER[ver], LIM[lim], ph, pv, int(split), _p(dh), _p(dv))
    if rc != 0:
        raise RuntimeError(f"om_do_oce_adv_tra failed: {rc}")
    return dh, dv


def analytic_step(mesh, work, dt, vel, w, values, valuesAB, schemes, copy_ab=False, wi=None, we=None,
                  ab2_eps=None):
    """One driver step for all tracers, in place. schemes: list of (hor, ver, lim[, ph, pv]).
    wi / we as for do_oce_adv_tra. valuesAB afterwards: unchanged (copy_ab
    False), the new values (copy_ab True), or with ab2_eps given the
    second-order Adams-Bashforth level -(0.5+eps) old + (1.5+eps) new."""
    ntr = len(schemes)
    assert values.flags.c_contiguous and values.dtype == np.float64
    assert valuesAB.flags.c_contiguous and valuesAB.dtype == np.float64
    vel, w = _f64(vel), _f64(w)
    hor = np.array([HOR[s[0]] for s in schemes], np.int32)
    ver = np.array([VER[s[1]] for s in schemes], np.int32)
    lim = np.array([LIM[s[2]] for s in schemes], np.int32)
    ph = np.array([s[3] if len(s) > 3 else 1.0 for s in schemes])
    pv = np.array([s[4] if len(s) > 4 else 1.0 for s in schemes])
    del_ttf = np.zeros((mesh.nod2D, mesh.nl - 1))
    split = wi is not None
    wi = w if wi is None else _f64(wi)
    we = w if we is None else _f64(we)
    rc = lib().om_analytic_step_split(mesh.h, work.h, ntr, dt, _p(vel), _p(w), _p(wi), _p(we), int(split),
                                      _p(values), _p(valuesAB), _p(hor, _ip), _p(ver, _ip), _p(lim, _ip),
                                      _p(ph), _p(pv), 2 if ab2_eps is not None else int(copy_ab),
                                      0.0 if ab2_eps is None else float(ab2_eps), _p(del_ttf))
    if rc != 0:
        raise RuntimeError(f"om_analytic_step failed: {rc}")


def cabi_step(mesh, work, dt, vel, w, values, valuesAB, del_ttf, hor="UPW1", ver="UPW1", lim="NONE",
              ph=1.0, pv=1.0, wi=None, we=None):
    vel, w = _f64(vel), _f64(w)
    wi = np.zeros_like(w) if wi is None else _f64(wi)
    we = np.zeros_like(w) if we is None else _f64(we)
    rc = lib().om_cabi_step(mesh.h, work.h, dt, _p(vel), _p(w), _p(wi), _p(we), _p(values), _p(valuesAB),
                            HOR[hor], VER[ver], LIM[lim], ph, pv, _p(del_ttf))
    if rc != 0:
        raise RuntimeError(f"om_cabi_step failed: {rc}")
