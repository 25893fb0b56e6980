"""Seeded inputs of the benchmark workloads on the oracle's own mesh, numpy only.

TEST INFRASTRUCTURE: bench.py's CPU legs (the reference arm and the CPU
baseline) build their workload with this module and the oracle, so no product
library is loaded on that path. The constructions are those of the benchmark
configurations:

- a doubly periodic analytic grid of n x n nodes (the dwarf's mesh generator
  with n + 1 grid points a side, lib/analytic_mesh.F90), dx = 1 km, nz layers
  whose thicknesses grow geometrically from 5 m to 250 m;
- horizontal velocity on elements: the rotated P1 gradient (gradient_sca,
  lib/oce_mesh.F90:2512-2534) of a streamfunction of 8 random-phase Fourier
  modes with wavenumbers 1..8, decaying as exp(z / 500 m), scaled so that the
  largest upwind outflow Courant number at dt is the target CFL;
- W from the discrete continuity of the upwind volume fluxes
  (lib/oce_adv_tra_hor.F90:174-252), zero at the bottom;
- T = 2 + 20 * Gaussian blob + N(0, 0.1); S = 35 + N(0, 0.3); passive
  tracers: Gaussian blobs in [0, 1].
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O

R_EARTH = 6367500.0  # lib/oce_modules.F90:24


def stretched_zbar(nz: int, top: float = 5.0, bottom: float = 250.0) -> np.ndarray:
    """Interface depths (0 at the surface, negative down) of nz layers whose
    thicknesses grow geometrically from top to bottom metres."""
    r = (bottom / top) ** (1.0 / (nz - 1)) if nz > 1 else 1.0
    return np.concatenate([[0.0], -np.cumsum(top * r ** np.arange(nz))])


def flat_mesh(n: int, nz: int) -> O.Mesh:
    """n x n nodes doubly periodic, dx = 1 km, nz stretched layers, edges
    oriented with the first element on the left (the benchmark meshes)."""
    zb = stretched_zbar(nz)
    L = n * 1000.0
    return O.Mesh(n + 1, n + 1, nz + 1, Lx=L, Ly=L, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb)


def _edge_sides(m: O.Mesh, u: np.ndarray) -> np.ndarray:
    """Depth-independent volume flux factor of every edge (both elements), for
    a velocity u (M, 2) on elements."""
    et = m.geti("edge_tri") - 1
    cr = m.getd("edge_cross_dxdy")
    e1 = et[:, 0]
    has2 = et[:, 1] >= 0
    e2 = np.where(has2, et[:, 1], 0)
    v1 = -(u[e1, 1] * cr[:, 0]) + u[e1, 0] * cr[:, 1]
    v2 = np.where(has2, u[e2, 1] * cr[:, 2] - u[e2, 0] * cr[:, 3], 0.0)
    return v1 + v2


def streamfunction_flow(m: O.Mesh, rng, dt: float, cfl: float = 0.4, nmodes: int = 8, kmax: int = 8,
                        efold: float = 500.0):
    """vel (M, nz, 2) and w (N, nl) of the streamfunction flow on a flat mesh."""
    c = m.getd("coord")
    x, y = c[:, 0] * R_EARTH, c[:, 1] * R_EARTH
    psi = np.zeros(m.nod2D)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, kmax + 1, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        psi += np.sin(2 * np.pi * (kx * x / m.Lx + ky * y / m.Ly) + ph) / np.hypot(kx, ky)
    en = m.geti("elem2D_nodes") - 1
    gs = m.getd("gradient_sca")
    dpx = (gs[:, 0:3] * psi[en]).sum(1)
    dpy = (gs[:, 3:6] * psi[en]).sum(1)
    zb = m.getd("zbar")
    h = zb[:-1] - zb[1:]
    s = np.exp(0.5 * (zb[:-1] + zb[1:]) / efold)
    vf2 = _edge_sides(m, np.stack([-dpy, dpx], axis=1))
    ed = m.geti("edges") - 1
    out = np.zeros(m.nod2D)
    np.add.at(out, ed[:, 0], np.maximum(vf2, 0.0))
    np.add.at(out, ed[:, 1], np.maximum(-vf2, 0.0))
    vol2 = m.getd("areasvol")[:, 0]
    scale = cfl / float(np.max(dt * out[:, None] * s[None, :] / vol2[:, None]))
    nz = m.nl - 1
    vel = np.empty((m.elem2D, nz, 2))
    vel[..., 0] = (-dpy * scale)[:, None] * s[None, :]
    vel[..., 1] = (dpx * scale)[:, None] * s[None, :]
    D2 = np.zeros(m.nod2D)
    np.add.at(D2, ed[:, 0], -vf2)
    np.add.at(D2, ed[:, 1], vf2)
    D2 *= scale
    area = m.getd("area")
    w = np.zeros((m.nod2D, m.nl))
    for k in range(nz - 1, -1, -1):
        w[:, k] = (D2 * (s[k] * h[k]) + w[:, k + 1] * area[:, k + 1]) / area[:, k]
    return vel, w


def tracers(m: O.Mesh, K: int, rng) -> np.ndarray:
    """(K, N, nz): T (blob + noise), S (35 + noise), then passive blobs."""
    c = m.getd("coord")
    x, y = c[:, 0] * R_EARTH, c[:, 1] * R_EARTH
    zb = m.getd("zbar")
    zmid = 0.5 * (zb[:-1] + zb[1:])
    H = -zb[-1]
    nz = m.nl - 1
    out = np.zeros((K, m.nod2D, nz))
    for t in range(K):
        if t == 0:
            r2 = ((x - 0.5 * m.Lx) ** 2 + (y - 0.5 * m.Ly) ** 2) / (2 * (m.Lx / 8) ** 2)
            zz = (zmid + 0.25 * H) ** 2 / (2 * (0.25 * H) ** 2)
            out[t] = 2.0 + 20.0 * np.exp(-r2[:, None] - zz[None, :]) + rng.normal(0, 0.1, size=(m.nod2D, nz))
        elif t == 1:
            out[t] = 35.0 + rng.normal(0, 0.3, size=(m.nod2D, nz))
        else:
            cx, cy = rng.uniform(0, m.Lx), rng.uniform(0, m.Ly)
            sx, sy = rng.uniform(0.05, 0.2) * m.Lx, rng.uniform(0.05, 0.2) * m.Ly
            cz, sz = -rng.uniform(0, H), rng.uniform(0.1, 0.5) * H
            dx, dy = np.abs(x - cx), np.abs(y - cy)
            dx, dy = np.minimum(dx, m.Lx - dx), np.minimum(dy, m.Ly - dy)
            out[t] = np.exp(-(dx / sx) ** 2 - (dy / sy) ** 2)[:, None] * np.exp(-((zmid - cz) / sz) ** 2)[None, :]
    return out


def flat_case(n: int, nz: int, K: int, dt: float, cfl: float = 0.4, seed: int = 20260301):
    """Mesh, vel, w and tracer values (K, N, nz) of an n x n periodic workload."""
    m = flat_mesh(n, nz)
    rng = np.random.default_rng(seed)
    vel, w = streamfunction_flow(m, rng, dt, cfl)
    return m, vel, w, np.ascontiguousarray(tracers(m, K, rng))
