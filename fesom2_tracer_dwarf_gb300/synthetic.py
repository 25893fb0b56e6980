"""Seeded synthetic inputs of the benchmark configurations.

No dataset is involved in the reference's measurements; the configurations
are analytic meshes with these fields:

- the analytic dwarf (src/fesom_analytic.F90:251-331): u=(0.1,0), W=0;
- streamfunction flows: a P1 streamfunction on nodes made of random-phase
  Fourier modes, decaying with depth; horizontal velocity on elements is its
  rotated element gradient (gradient_sca), scaled to a target horizontal CFL;
  on ragged meshes the vertical profile is normalised per element so the
  depth-integrated transport is non-divergent; W is diagnosed from the
  discrete continuity of the upwind flux of a uniform tracer;
- T: Gaussian blob of 20 on a background of 2 plus N(0, 0.1) noise;
  S: 35 + N(0, 0.3); passive tracers: random Gaussian blobs in [0, 1].
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh

R_EARTH = 6367500.0


def stretched_zbar(nz: int, top: float = 5.0, bottom: float = 250.0) -> np.ndarray:
    """Interface depths (0 at the surface, negative down) of nz layers whose
    thicknesses grow geometrically from top to bottom metres."""
    r = (bottom / top) ** (1.0 / (nz - 1)) if nz > 1 else 1.0
    h = top * r ** np.arange(nz)
    return np.concatenate([[0.0], -np.cumsum(h)])


def dwarf_velocity(m: Mesh):
    """u=(0.1, 0) m/s on every element, W=0 (src/fesom_analytic.F90:251-256)."""
    vel = np.zeros((m.M, m.nz, 2))
    vel[..., 0] = 0.1
    return vel, np.zeros((m.N, m.nl))


def node_xy(m: Mesh):
    c = m.get("coord")
    return c[:, 0] * R_EARTH, c[:, 1] * R_EARTH


def _xyL(m: Mesh):
    """Node coordinates (m) and the domain extent: the analytic mesh's Lx, Ly,
    or for meshes read from files the coordinates shifted to start at 0 and
    their span."""
    x, y = node_xy(m)
    if m.Lx:
        return x, y, m.Lx, m.Ly
    x, y = x - x.min(), y - y.min()
    return x, y, float(x.max()) or 1.0, float(y.max()) or 1.0


def random_field(m: Mesh, rng, K: int = 1) -> np.ndarray:
    """Smooth random tracer values (K, N, nz) for parity tests."""
    x, y, Lx, Ly = _xyL(m)
    out = np.zeros((K, m.N, m.nz))
    z = np.arange(m.nz) / max(m.nz - 1, 1)
    for t in range(K):
        a = rng.uniform(0.5, 2.0, 4)
        ph = rng.uniform(0, 2 * np.pi, 4)
        base = (a[0] * np.sin(2 * np.pi * x / Lx + ph[0]) * np.cos(2 * np.pi * y / Ly + ph[1])
                + a[1] * np.sin(4 * np.pi * x / Lx + ph[2]))
        out[t] = 10.0 + base[:, None] * (1.0 - 0.5 * z)[None, :] - 3.0 * z[None, :] + a[3] * np.cos(6 * z + ph[3])
        out[t] += rng.normal(0, 0.2, size=(m.N, m.nz))
    return out


def random_flow(m: Mesh, rng, umax: float = 0.3, wmax: float = 2e-3):
    """Random (non-solenoidal) horizontal and vertical velocities for parity
    tests; W is zero at each column's bottom interface."""
    vel = rng.uniform(-umax, umax, size=(m.M, m.nz, 2))
    w = rng.uniform(-wmax, wmax, size=(m.N, m.nl))
    nlev = m.get("nlevels_nod2D")
    for n in range(m.N):
        w[n, nlev[n] - 1:] = 0.0
    return vel, w


def _edge_vflux(m: Mesh, vel: np.ndarray, helem=None, levels=None) -> np.ndarray:
    """Volume flux through each edge's two segments, (E, nz), as the upwind
    flux of lib/oce_adv_tra_hor.F90:174-252 forms it."""
    ed_tri = m.get("edge_tri")
    cr = m.get("edge_cross_dxdy")
    helem = m.get("helem") if helem is None else helem
    lev = m.get("edge_lev")
    z = np.arange(1, (m.nz if levels is None else levels) + 1)[None, :]
    nu1, nl1, nu2, nl2 = (lev[:, i:i + 1] for i in range(4))
    nl12, nu12 = np.minimum(nl1, nl2), np.maximum(nu1, nu2)
    use1 = ((z >= nu1) & (z <= nu12 - 1)) | ((z >= nu12) & (z <= nl12)) | ((z > nl12) & (z <= nl1))
    use2 = (((nu2 > 0) & (z >= nu2) & (z <= nu12 - 1)) | ((z >= nu12) & (z <= nl12)) | ((z > nl12) & (z <= nl2)))
    e1 = ed_tri[:, 0]
    e2 = np.where(ed_tri[:, 1] >= 0, ed_tri[:, 1], 0)
    v1 = (-(vel[e1, :, 1] * cr[:, 0:1]) + vel[e1, :, 0] * cr[:, 1:2]) * helem[e1]
    v2 = (vel[e2, :, 1] * cr[:, 2:3] - vel[e2, :, 0] * cr[:, 3:4]) * helem[e2]
    return np.where(use1, v1, 0.0) + np.where(use2, v2, 0.0)


def _node_divergence(m: Mesh, vf: np.ndarray) -> np.ndarray:
    """Net inflow of a uniform tracer per node and layer, (N, nz)."""
    edges = m.get("edges")
    D = np.zeros((m.N,) + vf.shape[1:])
    np.add.at(D, edges[:, 0], -vf)
    np.add.at(D, edges[:, 1], vf)
    return D


def diagnose_w(m: Mesh, vel: np.ndarray) -> np.ndarray:
    """Vertical velocity (N, nl) from the discrete continuity of a uniform
    tracer: W(z) area(z) = D(z) + W(z+1) area(z+1), W = 0 at the bottom."""
    D = _node_divergence(m, _edge_vflux(m, vel))
    area = m.get("area")
    nlev = m.get("nlevels_nod2D")
    w = np.zeros((m.N, m.nl))
    for k in range(m.nz - 1, -1, -1):
        wet = k < nlev - 1
        below = w[:, k + 1] * area[:, k + 1]
        w[:, k] = np.where(wet, (D[:, k] + below) / np.where(area[:, k] > 0, area[:, k], 1.0), 0.0)
    return w


def max_cfl(m: Mesh, vel: np.ndarray, dt: float) -> float:
    """max over nodes and layers of dt * (upwind outflow) / (areasvol * hnode)."""
    out = _node_out(m, _edge_vflux(m, vel))
    vol = m.get("areasvol")[:, : m.nz] * m.get("hnode")
    nlev = m.get("nlevels_nod2D")
    wet = np.arange(m.nz)[None, :] < (nlev - 1)[:, None]
    return float(np.max(np.where(wet, dt * out / np.where(vol > 0, vol, 1.0), 0.0)))


def _flat(m: Mesh) -> bool:
    return bool(np.all(m.get("nlevels") == m.nl)) and bool(np.all(m.get("nlevels_nod2D") == m.nl))


def streamfunction_flow(m: Mesh, rng, dt: float, cfl: float = 0.4, nmodes: int = 8, kmax: int = 8,
                        efold: float = 500.0, psi_wall_zero: bool = False):
    """Horizontal velocity (M, nz, 2) = rotated P1 gradient of a random-phase
    Fourier streamfunction with a depth decay, scaled to the target CFL at dt,
    and W (N, nl) diagnosed from continuity."""
    x, y, Lx, Ly = _xyL(m)
    psi = np.zeros(m.N)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        psi += np.sin(2 * np.pi * (kx * x / Lx + ky * y / Ly) + ph) / np.hypot(kx, ky)
    if psi_wall_zero and not m.periodic:
        # closed basin: taper to zero on the walls
        psi *= np.sin(np.pi * x / Lx) * np.sin(np.pi * y / Ly)
    en = m.get("elem_nodes")
    gs = m.get("gradient_sca")
    dpx = (gs[:, 0:3] * psi[en]).sum(1)
    dpy = (gs[:, 3:6] * psi[en]).sum(1)
    zb = m.get("zbar")
    zmid = 0.5 * (zb[:-1] + zb[1:])
    h = zb[:-1] - zb[1:]
    s = np.exp(zmid / efold)
    if _flat(m):
        # One 2-D pass: vflux(e, z) = vflux2d(e) * s(z) * h(z), divergence likewise.
        vel2 = np.zeros((m.M, 1, 2))
        vel2[:, 0, 0] = -dpy
        vel2[:, 0, 1] = dpx
        vf2 = _edge_vflux(m, vel2, helem=np.ones((m.M, 1)), levels=1)[:, 0]
        out = _node_out(m, vf2)
        vol2 = m.get("areasvol")[:, 0]
        scale = cfl / float(np.max(dt * out[:, None] * (s * h)[None, :] / (vol2[:, None] * h[None, :])))
        vel = np.empty((m.M, m.nz, 2))
        vel[..., 0] = (-dpy * scale)[:, None] * s[None, :]
        vel[..., 1] = (dpx * scale)[:, None] * s[None, :]
        D2 = _node_divergence(m, vf2) * scale
        area = m.get("area")
        w = np.zeros((m.N, m.nl))
        for k in range(m.nz - 1, -1, -1):
            w[:, k] = (D2 * s[k] * h[k] + w[:, k + 1] * area[:, k + 1]) / area[:, k]
        return vel, w
    nlevel = m.get("nlevels")
    wet = np.arange(m.nz)[None, :] < (nlevel - 1)[:, None]
    full = (s * h).sum()
    col = np.where(wet, (s * h)[None, :], 0.0).sum(1)
    prof = np.where(wet, s[None, :] * (full / col)[:, None], 0.0)
    vel = np.zeros((m.M, m.nz, 2))
    vel[..., 0] = -dpy[:, None] * prof
    vel[..., 1] = dpx[:, None] * prof
    c = max_cfl(m, vel, dt)
    vel *= cfl / c
    w = diagnose_w(m, vel)
    return vel, w


def layered_flow(m: Mesh, rng, dt: float, cfl: float = 0.4, nmodes: int = 8, kmax: int = 8,
                 efold: float = 500.0, coast_taper: int = 3):
    """streamfunction_flow for large ragged meshes (ulevels = 1, helem the
    zbar thicknesses): velocity (M, 2) of the top layer and the depth profile
    s (nz) -- the layer-z velocity is u * s[z] -- and W (N, nl) from the
    discrete continuity of diagnose_w, computed per edge side with
    difference arrays over the layer breakpoints instead of per layer. The
    streamfunction is tapered to zero over `coast_taper` edge hops from the
    coast (nodes of edges with one element), so the rotated gradient's volume
    fluxes telescope around every dual cell and W comes from the bottom steps
    only. Scaled so that the largest horizontal and vertical Courant numbers
    at dt are cfl."""
    x, y, Lx, Ly = _xyL(m)
    psi = np.zeros(m.N)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        psi += np.sin(2 * np.pi * (kx * x / Lx + ky * y / Ly) + ph) / np.hypot(kx, ky)
    if coast_taper > 0:
        ed0, et0 = m.get("edges"), m.get("edge_tri")
        hops = np.full(m.N, coast_taper, np.int64)
        hops[ed0[et0[:, 1] < 0].reshape(-1)] = 0
        for _ in range(coast_taper):
            nb = np.minimum(hops[ed0[:, 0]], hops[ed0[:, 1]]) + 1
            np.minimum.at(hops, ed0[:, 0], nb)
            np.minimum.at(hops, ed0[:, 1], nb)
        psi *= np.minimum(hops, coast_taper) / coast_taper
    en = m.get("elem_nodes")
    gs = m.get("gradient_sca")
    u = np.stack([-(gs[:, 3:6] * psi[en]).sum(1), (gs[:, 0:3] * psi[en]).sum(1)], axis=1)
    zb = m.get("zbar")
    h = zb[:-1] - zb[1:]
    s = np.exp(0.5 * (zb[:-1] + zb[1:]) / efold)
    nz, N = m.nz, m.N
    ed, et, cr, lev = m.get("edges"), m.get("edge_tri"), m.get("edge_cross_dxdy"), m.get("edge_lev")
    has2 = et[:, 1] >= 0
    e1, e2 = et[:, 0], np.where(has2, et[:, 1], 0)
    # per-side 2-D volume flux factors (the v1, v2 of _edge_vflux without s h)
    c1 = -u[e1, 1] * cr[:, 0] + u[e1, 0] * cr[:, 1]
    c2 = np.where(has2, u[e2, 1] * cr[:, 2] - u[e2, 0] * cr[:, 3], 0.0)
    L1, L2 = lev[:, 1], np.where(has2, lev[:, 3], 0)  # deepest layer of each side
    # divergence: G[n, z] = sum over incident sides reaching layer z of +-c
    P = np.zeros((N, nz + 2))
    for col, sg in ((ed[:, 0], -1.0), (ed[:, 1], 1.0)):
        np.add.at(P, (col, L1), sg * c1)
        np.add.at(P, (col, L2), sg * c2)
    G = np.cumsum(P[:, ::-1], axis=1)[:, ::-1]
    D = G[:, 1:nz + 1] * (s * h)[None, :]
    del P, G
    area = m.get("area")
    nlev = m.get("nlevels_nod2D")
    w = np.zeros((N, m.nl))
    for k in range(nz - 1, -1, -1):
        wet = k < nlev - 1
        w[:, k] = np.where(wet, (D[:, k] + w[:, k + 1] * area[:, k + 1]) / np.where(area[:, k] > 0, area[:, k], 1.0),
                           0.0)
    del D
    # horizontal Courant numbers: upwind outflow, piecewise constant between
    # the two sides' bottoms
    lmin, lmax = np.minimum(L1, L2), np.maximum(L1, L2)
    cdeep = np.where(L1 >= L2, c1, c2)
    Q = np.zeros((N, nz + 2))
    for col, sg in ((ed[:, 0], 1.0), (ed[:, 1], -1.0)):
        a = np.maximum(sg * (c1 + c2), 0.0)
        b = np.maximum(sg * cdeep, 0.0)
        np.add.at(Q, (col, np.ones_like(lmin)), a)
        np.add.at(Q, (col, lmin + 1), b - a)
        np.add.at(Q, (col, lmax + 1), -b)
    out = np.cumsum(Q, axis=1)[:, 1:nz + 1] * s[None, :]
    del Q
    asv = m.get("areasvol")[:, :nz]
    wetl = np.arange(nz)[None, :] < (nlev - 1)[:, None]
    ch = float(np.max(np.where(wetl, dt * out / np.where(asv > 0, asv, 1.0), 0.0)))
    hmin = np.minimum(np.concatenate([h[:1], h[:-1]]), h)  # thinner layer at each interface k < nz
    cv = float(np.max(np.abs(w[:, :nz]) * dt / hmin[None, :]))
    scale = cfl / max(ch, cv, 1e-300)
    return u * scale, s, w * scale


def _node_out(m: Mesh, vf: np.ndarray) -> np.ndarray:
    edges = m.get("edges")
    out = np.zeros((m.N,) + vf.shape[1:])
    np.add.at(out, edges[:, 0], np.maximum(vf, 0.0))
    np.add.at(out, edges[:, 1], np.maximum(-vf, 0.0))
    return out


def gaussian_T(m: Mesh, rng) -> np.ndarray:
    x, y, Lx, Ly = _xyL(m)
    zmid = 0.5 * (m.get("zbar_3d_n")[0, :-1] + m.get("zbar_3d_n")[0, 1:])
    H = -m.get("zbar_3d_n")[0, -1]
    r2 = ((x - 0.5 * Lx) ** 2 + (y - 0.5 * Ly) ** 2) / (2 * (Lx / 8) ** 2)
    zz = (zmid + 0.25 * H) ** 2 / (2 * (0.25 * H) ** 2)
    return 2.0 + 20.0 * np.exp(-r2[:, None] - zz[None, :]) + rng.normal(0, 0.1, size=(m.N, m.nz))


def salinity(m: Mesh, rng) -> np.ndarray:
    return 35.0 + rng.normal(0, 0.3, size=(m.N, m.nz))


def passive_blob(m: Mesh, rng) -> np.ndarray:
    x, y, Lx, Ly = _xyL(m)
    zmid = 0.5 * (m.get("zbar_3d_n")[0, :-1] + m.get("zbar_3d_n")[0, 1:])
    H = -m.get("zbar_3d_n")[0, -1]
    cx, cy = rng.uniform(0, Lx), rng.uniform(0, Ly)
    sx, sy = rng.uniform(0.05, 0.2) * Lx, rng.uniform(0.05, 0.2) * Ly
    cz, sz = -rng.uniform(0, H), rng.uniform(0.1, 0.5) * H
    dx = np.abs(x - cx)
    dy = np.abs(y - cy)
    if m.periodic:
        dx = np.minimum(dx, Lx - dx)
        dy = np.minimum(dy, Ly - dy)
    return np.exp(-(dx / sx) ** 2 - (dy / sy) ** 2)[:, None] * np.exp(-((zmid - cz) / sz) ** 2)[None, :]


def bathymetry_levels(nx: int, ny: int, zbar: np.ndarray, rng, min_layers: int = 8) -> np.ndarray:
    """nlevels per element (2*(nx-1)*(ny-1)) from a smooth seeded bathymetry:
    depth between the depth of min_layers layers and the full depth."""
    nz = len(zbar) - 1
    xs = np.linspace(0, 1, nx)
    ys = np.linspace(0, 1, ny)
    X, Y = np.meshgrid(xs, ys)  # (ny, nx): node (i,j) -> [j, i]
    f = np.zeros_like(X)
    for _ in range(6):
        kx, ky = rng.integers(1, 5, size=2)
        f += rng.normal() * np.cos(np.pi * kx * X + rng.uniform(0, 6.3)) * np.cos(np.pi * ky * Y + rng.uniform(0, 6.3))
    f = (f - f.min()) / (f.max() - f.min() + 1e-30)
    dmin, dmax = -zbar[min_layers], -zbar[-1]
    depth = dmin + (dmax - dmin) * f
    # element depth = mean of its three node depths; layers whose top lies above it are wet
    q = depth[:-1, :-1], depth[:-1, 1:], depth[1:, 1:], depth[1:, :-1]  # (i,j),(i+1,j),(i+1,j+1),(i,j+1)
    lower = (q[0] + q[2] + q[1]) / 3.0
    upper = (q[0] + q[3] + q[2]) / 3.0
    el = np.stack([lower, upper], axis=-1).reshape(-1)  # quad order (j, i), lower then upper
    tops = -zbar[:-1]
    nlay = (tops[None, :] < el[:, None]).sum(1)
    nlay = np.clip(nlay, min_layers, nz)
    return (nlay + 1).astype(np.int32)


def flat_streamfunction_device(m: Mesh, rng, dt: float, dtype, device, cfl: float = 0.4, nmodes: int = 8,
                               kmax: int = 8, efold: float = 500.0):
    """streamfunction_flow for flat meshes, built directly as padded device
    tensors vel (M, LZ, 2) and w (N, LW) (large benchmark meshes)."""
    import torch

    assert _flat(m), "flat meshes only"
    x, y = node_xy(m)
    psi = np.zeros(m.N)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        psi += np.sin(2 * np.pi * (kx * x / m.Lx + ky * y / m.Ly) + ph) / np.hypot(kx, ky)
    en = m.get("elem_nodes")
    gs = m.get("gradient_sca")
    dpx = (gs[:, 0:3] * psi[en]).sum(1)
    dpy = (gs[:, 3:6] * psi[en]).sum(1)
    zb = m.get("zbar")
    zmid = 0.5 * (zb[:-1] + zb[1:])
    h = zb[:-1] - zb[1:]
    s = np.exp(zmid / efold)
    vel2 = np.zeros((m.M, 1, 2))
    vel2[:, 0, 0] = -dpy
    vel2[:, 0, 1] = dpx
    vf2 = _edge_vflux(m, vel2, helem=np.ones((m.M, 1)), levels=1)[:, 0]
    out = _node_out(m, vf2)
    vol2 = m.get("areasvol")[:, 0]
    scale = cfl / float(np.max(dt * out[:, None] * s[None, :] / vol2[:, None]))
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device)
    vel = torch.zeros(m.M, m.LZ, 2, dtype=dtype, device=device)
    sz = t(s)
    vel[:, : m.nz, 0] = (t(-dpy * scale)[:, None] * sz[None, :]).to(dtype)
    vel[:, : m.nz, 1] = (t(dpx * scale)[:, None] * sz[None, :]).to(dtype)
    D2 = t(_node_divergence(m, vf2) * scale)
    area = t(m.get("area"))
    w = torch.zeros(m.N, m.LW, dtype=torch.float64, device=device)
    for k in range(m.nz - 1, -1, -1):
        w[:, k] = (D2 * (s[k] * h[k]) + w[:, k + 1] * area[:, k + 1]) / area[:, k]
    return vel, w.to(dtype)


def tracers_device(m: Mesh, K: int, seed: int, dtype, device):
    """(K, N, LZ) padded tracers: T (Gaussian blob + noise), S (35 + noise),
    then passive Gaussian blobs in [0, 1]."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x, y = node_xy(m)
    zb = m.get("zbar")
    zmid = 0.5 * (zb[:-1] + zb[1:])
    H = -zb[-1]
    X = torch.as_tensor(x, dtype=torch.float64, device=device)[:, None]
    Y = torch.as_tensor(y, dtype=torch.float64, device=device)[:, None]
    Zm = torch.as_tensor(zmid, dtype=torch.float64, device=device)[None, :]
    out = torch.zeros(K, m.N, m.LZ, dtype=dtype, device=device)
    rng = np.random.default_rng(seed)
    for t in range(K):
        if t == 0:
            r2 = ((X - 0.5 * m.Lx) ** 2 + (Y - 0.5 * m.Ly) ** 2) / (2 * (m.Lx / 8) ** 2)
            zz = (Zm + 0.25 * H) ** 2 / (2 * (0.25 * H) ** 2)
            v = 2.0 + 20.0 * torch.exp(-r2 - zz)
            v = v + 0.1 * torch.randn(m.N, m.nz, generator=g, dtype=torch.float64, device=device)
        elif t == 1:
            v = 35.0 + 0.3 * torch.randn(m.N, m.nz, generator=g, dtype=torch.float64, device=device)
        else:
            cx, cy = rng.uniform(0, m.Lx), rng.uniform(0, m.Ly)
            sx, sy = rng.uniform(0.05, 0.2) * m.Lx, rng.uniform(0.05, 0.2) * m.Ly
            cz, sz = -rng.uniform(0, H), rng.uniform(0.1, 0.5) * H
            dx = (X - cx).abs()
            dy = (Y - cy).abs()
            if m.periodic:
                dx = torch.minimum(dx, m.Lx - dx)
                dy = torch.minimum(dy, m.Ly - dy)
            v = torch.exp(-(dx / sx) ** 2 - (dy / sy) ** 2) * torch.exp(-((Zm - cz) / sz) ** 2)
        out[t, :, : m.nz] = v.to(dtype)
    return out
