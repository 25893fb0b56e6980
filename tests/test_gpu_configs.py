"""GPU against the oracle at the benchmark configurations' own sizes.

- 512 x 512 nodes doubly periodic, 48 layers stretched 5 -> 250 m, dx = 1 km,
  two tracers (T blob + noise, S = 35 + noise), streamfunction flow at CFL 0.4
  with W from continuity, QR4C vertical with upwind-FCT and MUSCL-FCT
  horizontal, three steps with copy-AB; and the same with a divergent
  component added to the flow, so that W is not zero and the vertical
  schemes see real fluxes (with a flat bottom the streamfunction flow alone
  has W = 0 up to rounding).
- 1024 x 1024 closed basin with seeded bathymetry (8..64 layers), the
  streamfunction vanishing on the walls, MUSCL-FCT + PPM, one step.

The FP64 form must equal the oracle bit for bit (do_oce_adv_tra,
lib/oce_adv_tra_driver.F90:23-294, in the reference's evaluation order); the
fast FP64 form is held to 1e-12 and the FP32 form (FP32 storage, and each
value with its rounding residual) to the FP32 bar of the other tests
(relative max-norm 1e-5) against the same oracle run. The oracle runs on every host core (its loops
are threaded without changing any result).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

REL_TOL_FP32 = 1e-5
REL_TOL_FAST64 = 1e-12


@pytest.fixture(scope="module")
def pkg(oracle_mod):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from fesom2_tracer_dwarf_gb300 import engine, mesh, synthetic

    before = oracle_mod.get_threads()
    oracle_mod.set_threads(os.cpu_count() or 1)
    yield mesh, engine, synthetic
    oracle_mod.set_threads(before)


def _divergent(m, synthetic, rng, vel, dt, frac=0.3, efold=500.0, cfl=0.4):
    """Add to the streamfunction flow (a 2-D field times the depth profile
    exp(z / efold)) the element gradient of a smooth potential of `frac` of
    its magnitude, rescale to the horizontal Courant number `cfl`, and
    diagnose W from continuity; all in 2-D, the flow being separable."""
    zb = m.get("zbar")
    h = zb[:-1] - zb[1:]
    s = np.exp(0.5 * (zb[:-1] + zb[1:]) / efold)
    x, y, Lx, Ly = synthetic._xyL(m)
    phi = np.zeros(m.N)
    for _ in range(4):
        kx, ky = rng.integers(1, 5, size=2)
        phi += np.cos(2 * np.pi * (kx * x / Lx + ky * y / Ly) + rng.uniform(0, 2 * np.pi))
    en, gs = m.get("elem_nodes"), m.get("gradient_sca")
    g = np.stack([(gs[:, 0:3] * phi[en]).sum(1), (gs[:, 3:6] * phi[en]).sum(1)], axis=1)
    u2 = vel[:, 0, :] / s[0]
    u2 = u2 + frac * np.abs(u2).max() / np.abs(g).max() * g
    vf2 = synthetic._edge_vflux(m, u2[:, None, :], helem=np.ones((m.M, 1)), levels=1)[:, 0]
    ch = float(np.max(dt * synthetic._node_out(m, vf2) * s[0] / m.get("areasvol")[:, 0]))
    D2 = synthetic._node_divergence(m, vf2)
    area = m.get("area")
    w = np.zeros((m.N, m.nl))
    for k in range(m.nz - 1, -1, -1):
        w[:, k] = (D2 * (s[k] * h[k]) + w[:, k + 1] * area[:, k + 1]) / area[:, k]
    hmin = np.minimum(h, np.concatenate([h[:1], h[:-1]]))  # thinner layer at each interface
    cv = float(np.max(np.abs(w[:, :-1]) * dt / hmin[None, :]))
    # the largest horizontal and vertical Courant numbers at most cfl
    scale = cfl / max(ch, cv)
    return (u2 * scale)[:, None, :] * s[None, :, None], w * scale


def _run(O, om, m, engine, vel, w, T, sch, steps, dt, precision, residual=False):
    eng = engine.TracerAdvection(m, T.shape[0], precision, *sch, copy_ab=True, residual=residual)
    eng.set_tracers(T)
    eng.set_velocity(vel, w)
    eng.step(dt, steps)
    torch.cuda.synchronize()
    return eng.values()


@pytest.fixture(scope="module")
def config2(pkg, oracle_mod):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    nz, n = 48, 512
    zb = synthetic.stretched_zbar(nz, 5.0, 250.0)
    kw = dict(Lx=n * 1e3, Ly=n * 1e3, depth=-zb[-1], periodic=True, orient_left=True, zbar=zb)
    om = O.Mesh(n + 1, n + 1, nz + 1, **kw)
    m = mesh_mod.Mesh(n + 1, n + 1, nz + 1, **kw)
    rng = np.random.default_rng(20260302)
    dt = 400.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4)
    T = np.stack([synthetic.gaussian_T(m, rng), synthetic.salinity(m, rng)])
    return O, om, m, engine, synthetic, rng, vel, w, T, dt


@pytest.mark.parametrize("hor", ["UPW1", "MUSCL"])
@pytest.mark.parametrize("flow", ["streamfunction", "divergent"])
def test_config2_512_fp64_bit_exact(config2, hor, flow):
    O, om, m, engine, synthetic, rng, vel, w, T, dt = config2
    if flow == "divergent":
        vel, w = _divergent(m, synthetic, np.random.default_rng(7), vel, dt)
        assert np.abs(w).max() > 1e-6
    sch = (hor, "QR4C", "FCT")
    steps = 3
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    W = O.Work(om)
    for _ in range(steps):
        O.analytic_step(om, W, dt, vel, w, vals, vab, [sch] * 2, copy_ab=True)
    got = _run(O, om, m, engine, vel, w, T, sch, steps, dt, "fp64")
    err = float(np.abs(got - vals).max())
    assert err == 0.0, f"512^2 x 48 {hor}-FCT/QR4C {flow}: max |GPU - oracle| = {err}"
    for residual in (False, True):
        got32 = _run(O, om, m, engine, vel, w, T, sch, steps, dt, "fp32", residual)
        for t in range(2):
            rel = float(np.abs(got32[t] - vals[t]).max() / np.abs(vals[t]).max())
            assert rel <= REL_TOL_FP32, f"FP32 form (residual={residual}), tracer {t}: {rel:.3g}"
    gotf = _run(O, om, m, engine, vel, w, T, sch, steps, dt, "fp64fast")
    for t in range(2):
        rel = float(np.abs(gotf[t] - vals[t]).max() / np.abs(vals[t]).max())
        assert rel <= REL_TOL_FAST64, f"fast FP64 form, tracer {t}: {rel:.3g}"


def test_config3_closed_1024_fp64_bit_exact(pkg, oracle_mod):
    mesh_mod, engine, synthetic = pkg
    O = oracle_mod
    nx, nz = 1025, 64
    rng = np.random.default_rng(20260303)
    zb = synthetic.stretched_zbar(nz, 5.0, 250.0)
    en = synthetic.bathymetry_levels(nx, nx, zb, rng, min_layers=8)
    kw = dict(Lx=1024e3, Ly=1024e3, depth=-zb[-1], periodic=False, orient_left=True, zbar=zb, elem_nlev=en)
    om = O.Mesh(nx, nx, nz + 1, **kw)
    m = mesh_mod.Mesh(nx, nx, nz + 1, **kw)
    lev = m.get("nlevels_nod2D") - 1
    assert lev.min() >= 8 and lev.max() == nz and lev.min() < lev.max()
    dt = 400.0
    vel, w = synthetic.streamfunction_flow(m, rng, dt, cfl=0.4, psi_wall_zero=True)
    assert np.abs(w).max() > 0.0  # the bottom steps make W non-zero
    T = np.stack([synthetic.gaussian_T(m, rng), synthetic.salinity(m, rng)])
    sch = ("MUSCL", "PPM", "FCT")
    vals = np.ascontiguousarray(T.copy())
    vab = vals.copy()
    O.analytic_step(om, O.Work(om), dt, vel, w, vals, vab, [sch] * 2, copy_ab=True)
    got = _run(O, om, m, engine, vel, w, T, sch, 1, dt, "fp64")
    wet = np.arange(nz)[None, :] < lev[:, None]
    err = float(np.abs(got - vals)[:, wet].max())
    assert err == 0.0, f"1024^2 closed MUSCL-FCT/PPM: max |GPU - oracle| = {err}"
    for residual in (False, True):
        got32 = _run(O, om, m, engine, vel, w, T, sch, 1, dt, "fp32", residual)
        for t in range(2):
            rel = float(np.abs(got32[t] - vals[t])[wet].max() / np.abs(vals[t][wet]).max())
            assert rel <= REL_TOL_FP32, f"FP32 form (residual={residual}), tracer {t}: {rel:.3g}"
