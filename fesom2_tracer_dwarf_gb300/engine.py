"""GPU engine of the tracer-advection step: device fields as torch tensors,
kernels launched through the C-ABI on torch's current CUDA stream.

``TracerAdvection`` advances K tracers of one mesh with do_oce_adv_tra
(lib/oce_adv_tra_driver.F90:23-294) followed by the analytic driver's
tendency update (src/fesom_analytic.F90:404-437). Tracer values live in a
(K, N, LZ) tensor (level index fastest, padded to LZ layers) in the FP64
form; the FP32 form groups V = 4 (or 2) tracers per node-layer, a
(K/V, N, LZ, V) tensor, so one vector load brings a group. ``to_layout`` and
``from_layout`` convert between (K, N, LZ) and the engine's layout.

valuesAB (the field the high-order fluxes read) is either frozen at the
values given to ``set_tracers`` -- the analytic dwarf, src/fesom_analytic.F90:335
-- or follows the values (``copy_ab=True``), or (``ab2_eps=eps``) is the
second-order Adams-Bashforth level -(0.5+eps) T_old + (1.5+eps) T_new that the
update stage writes for the next step (FESOM2's tracer AB2 with offset
epsilon; the reference declares epsilon = 0.1 at lib/oce_modules.F90:75).

Anomaly storage (``offsets``, opt-in, meant for the FP32 form): each tracer is
stored as T - c_t for a per-tracer reference value c_t (given; "mean": the
mean of the initial values; "auto": that mean only where it shrinks the stored
magnitude at least fourfold, else 0, so that fields touching zero such as
passive-tracer blobs keep exact zeros and stay non-negative), and c_t is added
back by ``values`` and ``stats``. Every
scheme of the step maps T + c to T' + c when a uniform field stays uniform,
i.e. when the velocities satisfy the discrete continuity of the step (as the
flows of the benchmark configurations do); then the stored anomalies advance
exactly as the full values would, and FP32 rounds them at their own, much
smaller magnitude (S ~ 35 +- 0.3 keeps ~2 more digits). For flows that do not
keep a uniform field uniform the offsets change the answer: leave them off.
The FCT limiter is shift-invariant only while values and anomalies stay
within +-1000: the reference bounds elements that are dry at a layer by
+-1e3 (bignumber, lib/oce_adv_tra_fct.F90:81,142-143).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .mesh import Mesh

_DT = {"fp64": torch.float64, "fp32": torch.float32, "fp64fast": torch.float64}
_PREC = {"fp64": _lib.FP64, "fp32": _lib.FP32, "fp64fast": _lib.FP64_FAST}


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("fesom2_tracer_dwarf_gb300 needs a CUDA GPU; there is no CPU path")


def anomaly_offsets(vals64, K, mode="mean"):
    """Per-tracer reference values of anomaly storage from (K, ...) values.

    "mean": each tracer's mean. "auto": the mean where max |T - mean| is at
    most a quarter of max |T| (the stored anomalies are then at least four
    times smaller than the values), else 0."""
    t = torch.as_tensor(vals64, dtype=torch.float64).reshape(K, -1)
    mean = t.mean(dim=1)
    if mode == "auto":
        spread = (t - mean[:, None]).abs().amax(dim=1)
        mean = torch.where(spread <= 0.25 * t.abs().amax(dim=1), mean, torch.zeros_like(mean))
    return mean.cpu().numpy()


class TracerAdvection:
    def __init__(self, mesh: Mesh, ntracers: int, precision: str = "fp64", hor: str = "UPW1",
                 ver: str = "UPW1", lim: str = "NONE", ph: float = 1.0, pv: float = 1.0,
                 copy_ab: bool = False, device: str = "cuda", tracer_vec: int | None = None,
                 ab2_eps: float | None = None, offsets=None, plain_sums=None, residual: bool = False):
        _require_cuda()
        if ab2_eps is not None and copy_ab:
            raise ValueError("copy_ab and ab2_eps are two choices of the valuesAB time level; give one")
        if precision not in _DT:
            raise ValueError(f"precision must be one of {list(_DT)}")
        self.mesh, self.K, self.precision = mesh, int(ntracers), precision
        self.dtype = _DT[precision]
        if tracer_vec is None:
            tracer_vec = 1 if precision != "fp32" else next(v for v in (4, 2, 1) if self.K % v == 0)
        if tracer_vec not in (1, 2, 4) or self.K % tracer_vec or (precision != "fp32" and tracer_vec != 1):
            raise ValueError("tracer_vec must be 1 (FP64 forms) or 1, 2, 4 dividing ntracers (FP32)")
        self.V = int(tracer_vec)
        self.G = self.K // self.V
        self.device = torch.device(device)
        self.set_schemes(hor, ver, lim, ph, pv)
        self.copy_ab = copy_ab
        self.ab2_eps = None if ab2_eps is None else float(ab2_eps)
        # FP32 form: plain FP32 sums instead of compensated ones (fgb_step_desc.fp32_plain_sums:
        # True = all, False = none, or the bit mask 1 LO fluxes, 2 update divergence, 4 FCT +/- sums).
        # None: by the form -- with the residual only the LO fluxes are compensated (the piece that keeps
        # the tracer sum to 1e-12), without it none (FP32 storage rounding dominates the sum's error)
        self.plain_sums = plain_sums
        # FP32 form with the FCT limiter: each value carries its FP32 rounding residual (self.Tlo)
        self.residual = bool(residual) and precision == "fp32" and lim == "FCT"
        if isinstance(offsets, str):
            if offsets not in ("mean", "auto"):
                raise ValueError('offsets must be None, "mean", "auto" or one value per tracer')
        elif offsets is not None:
            offsets = np.asarray(offsets, dtype=np.float64).reshape(self.K)
        self._offsets_req = offsets
        self.offsets = None  # per-tracer reference values of the stored anomalies (resolved at set_tracers)
        m = mesh
        m.upload()
        z = lambda *s: torch.zeros(*s, dtype=self.dtype, device=self.device)
        self.T = z(*self.layout_shape)
        self.Tlo = z(*self.layout_shape) if self.residual else None
        self.TA = None if copy_ab else z(*self.layout_shape)
        self.vel = z(m.M, m.LZ, 2)
        self.w = z(m.N, m.LW)
        self.we = self.w
        self.wi = None  # w_split off
        L = _lib.load()
        nbytes = L.fgb_workspace_bytes(m.handle, _PREC[precision], self.K)
        if nbytes < 0:
            raise RuntimeError(_lib.last_error())
        self.workspace = torch.zeros(int(nbytes), dtype=torch.uint8, device=self.device)
        self._stats_scratch = torch.zeros(int(L.fgb_stats_scratch_bytes(m.handle, self.K)), dtype=torch.uint8,
                                          device=self.device)
        self._stats_out = torch.zeros(self.K, 4, dtype=torch.float64, device=self.device)
        self.launches = 0
        self.cfg = [0] * _lib.NCFG  # launch configuration, see set_launch

    def set_residual(self, on: bool):
        """FP32 form with the FCT limiter: keep (allocate, zero) or drop the
        per-value rounding residual. Set the tracers afterwards to fill it."""
        on = bool(on) and self.precision == "fp32" and self.lim == "FCT"
        self.residual = on
        self.Tlo = torch.zeros_like(self.T) if on else None
        self._host_lo = None  # run_host's residual buffers follow the new one

    def set_launch(self, cfg):
        """Launch configuration (fgb_step_desc.cfg): a list of up to 12 ints or a
        dict with keys edge_warps, node_warps (lo, ratio, update), chunk (lo,
        ratio, update). Zeros pick the library defaults; results do not depend on it."""
        if isinstance(cfg, dict):
            nw = list(cfg.get("node_warps", (0, 0, 0)))
            kc = list(cfg.get("chunk", (0, 0, 0)))
            cfg = [int(cfg.get("edge_warps", 0)), *nw, *kc, 0]
        cfg = [int(c) for c in cfg] + [0] * (_lib.NCFG - len(cfg))
        if len(cfg) != _lib.NCFG:
            raise ValueError(f"a launch configuration has at most {_lib.NCFG} entries")
        self.cfg = cfg

    # ---- layout ------------------------------------------------------------
    @property
    def layout_shape(self):
        m = self.mesh
        return (self.K, m.N, m.LZ) if self.V == 1 else (self.G, m.N, m.LZ, self.V)

    def to_layout(self, x):
        """(K, N, LZ) tensor -> the engine's tracer layout (a view when V = 1)."""
        if self.V == 1:
            return x
        m = self.mesh
        return x.reshape(self.G, self.V, m.N, m.LZ).permute(0, 2, 3, 1).contiguous()

    def from_layout(self, x):
        """The engine's tracer layout -> (K, N, LZ)."""
        if self.V == 1:
            return x
        m = self.mesh
        return x.permute(0, 3, 1, 2).reshape(self.K, m.N, m.LZ)

    # ---- configuration -----------------------------------------------------
    def set_schemes(self, hor="UPW1", ver="UPW1", lim="NONE", ph=1.0, pv=1.0):
        for name, table, v in (("hor", _lib.HOR, hor), ("ver", _lib.VER, ver), ("lim", _lib.LIM, lim)):
            if v not in table:
                raise ValueError(f"unknown {name} scheme {v!r}")
        self.hor, self.ver, self.lim, self.ph, self.pv = hor, ver, lim, float(ph), float(pv)

    def _pad_nodes(self, a, width, ld):
        t = torch.as_tensor(np.asarray(a), dtype=self.dtype) if not torch.is_tensor(a) else a.to(self.dtype)
        out = torch.zeros(*t.shape[:-1], ld, dtype=self.dtype)
        out[..., :width] = t.cpu()
        return out.to(self.device)

    def _resolve_offsets(self, vals64):
        """vals64: (K, N, nz) float64 tensor or array of the initial values."""
        req = self._offsets_req
        if req is None:
            self.offsets = None
        elif isinstance(req, str):
            self.offsets = anomaly_offsets(vals64, self.K, req)
        else:
            self.offsets = req

    def _shifted(self, vals, ld, residual=False):
        """(K, N, nz) float64 values -> (K, N, ld) engine dtype on the host, minus the offsets
        (residual=True: the remainder those values leave after rounding to the engine dtype)."""
        m = self.mesh
        t = torch.as_tensor(np.asarray(vals) if not torch.is_tensor(vals) else vals.cpu(), dtype=torch.float64)
        t = t.reshape(self.K, m.N, -1)
        if self.offsets is not None:
            t = t - torch.as_tensor(self.offsets, dtype=torch.float64)[:, None, None]
        if residual:
            t = t - t.to(self.dtype).double()
        out = torch.zeros(self.K, m.N, ld, dtype=self.dtype)
        out[..., : t.shape[-1]] = t.to(self.dtype)
        return out.to(self.device)

    def set_tracers(self, values, values_ab=None):
        """values: (K, N, nz) array. values_ab defaults to values."""
        m = self.mesh
        self._resolve_offsets(values if torch.is_tensor(values) else np.asarray(values, dtype=np.float64))
        v = self.to_layout(self._shifted(values, m.LZ))
        self.T.copy_(v)
        if self.Tlo is not None:
            self.Tlo.copy_(self.to_layout(self._shifted(values, m.LZ, residual=True)))
        if self.TA is not None:
            self.TA.copy_(self.to_layout(self._shifted(values_ab, m.LZ)) if values_ab is not None else v)

    def set_velocity(self, vel, w, we=None, wi=None):
        """vel: (M, nz, 2) on elements; w, we, wi: (N, nl) at node interfaces.

        wi switches w_split on (dynamics%use_wsplit): under FCT the low-order
        solution gets the implicit vertical step with wi and the explicit
        low-order flux uses we (lib/oce_adv_tra_driver.F90:191-231). None
        switches it off."""
        m = self.mesh
        v = torch.zeros(m.M, m.LZ, 2, dtype=self.dtype)
        v[:, : m.nz, :] = torch.as_tensor(np.asarray(vel) if not torch.is_tensor(vel) else vel.cpu(), dtype=self.dtype)
        self.vel.copy_(v.to(self.device))
        self.w.copy_(self._pad_nodes(w, m.nl, m.LW))
        if we is None:
            self.we = self.w
        else:
            self.we = self._pad_nodes(we, m.nl, m.LW)
        self.wi = None if wi is None else self._pad_nodes(wi, m.nl, m.LW)

    def load_padded(self, T=None, TA=None, vel=None, w=None, we=None, wi=None):
        """Copy device tensors that already have the padded layouts
        (K,N,LZ), (M,LZ,2), (N,LW). wi (w_split) is kept until replaced."""
        m = self.mesh
        if T is not None:
            self._resolve_offsets(T[:, :, : m.nz].double())
            if self.offsets is not None:
                T = T.double() - torch.as_tensor(self.offsets, device=T.device)[:, None, None]
            self.T.copy_(self.to_layout(T.to(self.dtype)))
            if self.Tlo is not None:  # the remainder of wider values after rounding (0 for FP32 input)
                self.Tlo.copy_(self.to_layout((T.double() - T.to(self.dtype).double()).to(self.dtype)))
        if TA is not None and self.TA is not None:
            if self.offsets is not None:
                TA = TA.double() - torch.as_tensor(self.offsets, device=TA.device)[:, None, None]
            self.TA.copy_(self.to_layout(TA.to(self.dtype)))
        if vel is not None:
            self.vel.copy_(vel)
        if w is not None:
            self.w.copy_(w)
            self.we = self.w
        if we is not None:
            self.we = we.to(self.dtype).contiguous()
        if wi is not None:
            self.wi = wi.to(self.dtype).contiguous()

    # ---- step --------------------------------------------------------------
    def _desc(self, dt):
        d = _lib.StepDesc()
        d.precision = _PREC[self.precision]
        d.ntracers = self.K
        d.hor, d.ver, d.lim = _lib.HOR[self.hor], _lib.VER[self.ver], _lib.LIM[self.lim]
        d.ph, d.pv, d.dt = self.ph, self.pv, float(dt)
        m = self.mesh
        d.T = self.T.data_ptr()
        d.strideT = m.N * m.LZ * self.V
        d.TA = None if self.TA is None else self.TA.data_ptr()
        d.strideTA = m.N * m.LZ * self.V
        d.tracer_vec = self.V
        d.TAout = None
        if self.ab2_eps is not None:
            # the update stage writes the next step's AB2 level into TA
            d.TAout = self.TA.data_ptr()
            d.ab_order, d.ab_eps = 2, self.ab2_eps
        d.vel, d.w, d.we = self.vel.data_ptr(), self.w.data_ptr(), self.we.data_ptr()
        d.wi = None if self.wi is None else self.wi.data_ptr()
        d.del_ = None
        d.workspace = self.workspace.data_ptr()
        d.workspace_bytes = self.workspace.numel()
        ps = self.plain_sums
        if ps is None:
            ps = 6 if self.Tlo is not None else 7
        d.fp32_plain_sums = 7 if ps is True else (0 if ps is False else int(ps))
        d.Tlo = None if self.Tlo is None else self.Tlo.data_ptr()
        for i, c in enumerate(self.cfg):
            d.cfg[i] = c
        return d

    def step(self, dt: float, nsteps: int = 1, stages: int = _lib.STAGE_ALL):
        L = _lib.load()
        d = self._desc(dt)
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        for _ in range(nsteps):
            _lib.check(L.fgb_adv_stages(self.mesh.handle, ctypes.byref(d), stages, stream), "fgb_adv_stages")
            self.launches += L.fgb_last_launch_count()

    CHECK_BITS = {"T": 1, "TA": 2, "vel": 4, "w": 8, "we": 16, "wi": 32, "Tlo": 64}

    def check_inputs(self, dt: float = 1.0):
        """Names of the arrays a step would read that hold a NaN or an
        infinity (fgb_check_inputs: one device reduction per array, padding
        layers included); an empty list when every value is finite."""
        L = _lib.load()
        d = self._desc(dt)
        flags = ctypes.c_int()
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(L.fgb_check_inputs(self.mesh.handle, ctypes.byref(d), stream, ctypes.byref(flags)),
                   "fgb_check_inputs")
        return [k for k, bit in self.CHECK_BITS.items() if flags.value & bit]

    def run_host(self, host_in, host_out, dt: float, nsteps: int = 1, copy_streams: int = 1):
        """Advance independent batches of tracer fields that live in host
        memory: batch i is copied to the device from ``host_in[i]``, advanced
        ``nsteps`` steps, and copied back into ``host_out[i]`` (tensors of
        ``layout_shape`` and the engine's dtype, pinned for asynchronous
        copies; one tensor may serve several batches). An engine that keeps
        the FP32 rounding residual (residual=True) takes and returns each
        batch as a pair (values, residuals) of such tensors, the two halves of
        the FP64 field; a single tensor is then a batch of FP32 values, whose
        residual starts at zero and is not returned.

        Three device buffers take turns as the field being stepped, the next
        batch arriving and the previous batch leaving, so the host-to-device
        copy of batch i+1 and the device-to-host copy of batch i-1 run during
        the steps of batch i on the current stream. Each copy may be split into
        ``copy_streams`` chunks on as many streams per direction (which count
        is fastest depends on the host; one was on the machines measured).
        Needs a copy-AB engine (valuesAB follows the values). Returns
        on the host when every copy has been issued; synchronise the device
        before reading ``host_out``."""
        if self.TA is not None:
            raise ValueError("run_host needs copy_ab=True (valuesAB follows the values)")
        nb = len(host_in)
        if len(host_out) != nb:
            raise ValueError("host_in and host_out need one tensor per batch")

        def halves(x):
            x = tuple(x) if isinstance(x, (tuple, list)) else (x,)
            if len(x) not in (1, 2) or (len(x) == 2 and self.Tlo is None):
                raise ValueError("a batch is one tensor, or a (values, residuals) pair with residual=True")
            return x

        host_in = [halves(x) for x in host_in]
        host_out = [halves(x) for x in host_out]
        nc = max(1, int(copy_streams))
        main = torch.cuda.current_stream(self.device)
        if not hasattr(self, "_host_bufs"):
            self._host_bufs = [self.T] + [torch.empty_like(self.T) for _ in range(2)]
        if self.Tlo is not None and getattr(self, "_host_lo", None) is None:
            self._host_lo = [self.Tlo] + [torch.empty_like(self.Tlo) for _ in range(2)]
        if getattr(self, "_host_nc", None) != nc:
            self._h2d = [torch.cuda.Stream(self.device) for _ in range(nc)]
            self._d2h = [torch.cuda.Stream(self.device) for _ in range(nc)]
            self._host_nc = nc
        bufs = self._host_bufs
        lo = self._host_lo if self.Tlo is not None else None
        saved_t, saved_lo = self.T, self.Tlo
        numel = bufs[0].numel()
        bounds = [(c * numel) // nc for c in range(nc + 1)]
        free = [[torch.cuda.Event() for _ in range(nc)] for _ in range(3)]     # chunk no longer read by D2H
        arrived = [[torch.cuda.Event() for _ in range(nc)] for _ in range(3)]  # chunk copied in
        stepped = [torch.cuda.Event() for _ in range(3)]                        # steps on the buffer done
        for b in range(3):
            for c in range(nc):
                free[b][c].record(main)

        def device_halves(b):
            return (bufs[b],) if lo is None else (bufs[b], lo[b])

        def load(i):
            b = i % 3
            pairs = list(zip(host_in[i], device_halves(b)))
            for c in range(nc):
                st = self._h2d[c]
                with torch.cuda.stream(st):
                    st.wait_event(free[b][c])
                    for src, dst in pairs:
                        dst.view(-1)[bounds[c]:bounds[c + 1]].copy_(src.view(-1)[bounds[c]:bounds[c + 1]],
                                                                   non_blocking=True)
                    arrived[b][c].record(st)

        try:
            if nb:
                load(0)
            for i in range(nb):
                b = i % 3
                if i + 1 < nb:
                    load(i + 1)
                for c in range(nc):
                    main.wait_event(arrived[b][c])
                self.T = bufs[b]
                if lo is not None:
                    self.Tlo = lo[b]
                    if len(host_in[i]) == 1:  # FP32 values: no residual yet
                        self.Tlo.zero_()
                self.step(dt, nsteps)
                stepped[b].record(main)
                pairs = list(zip(device_halves(b), host_out[i]))
                for c in range(nc):
                    st = self._d2h[c]
                    with torch.cuda.stream(st):
                        st.wait_event(stepped[b])
                        for src, dst in pairs:
                            dst.view(-1)[bounds[c]:bounds[c + 1]].copy_(src.view(-1)[bounds[c]:bounds[c + 1]],
                                                                       non_blocking=True)
                        free[b][c].record(st)
            for b in range(3):
                for c in range(nc):
                    main.wait_event(free[b][c])
        finally:
            self.T, self.Tlo = saved_t, saved_lo
        return host_out

    def capture(self, dt: float, nsteps: int = 1):
        """Record ``nsteps`` steps as one CUDA graph (torch.cuda.CUDAGraph);
        ``graph.replay()`` then advances the tracers by nsteps steps with one
        launch of the graph. Capturing runs one eager step first (kernel
        attributes and lazy initialisation happen outside the capture), so the
        tracer values advance by one step: reset them before replaying if
        needed."""
        self.step(dt)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(dt, nsteps)
        return g

    # ---- outputs -----------------------------------------------------------
    def full_values(self):
        """(K, N, LZ) float64 tensor on the device: the stored values plus the
        rounding residuals (residual=True) plus the anomaly offsets."""
        v = self.from_layout(self.T).double()
        if self.Tlo is not None:
            v = v + self.from_layout(self.Tlo).double()
        if self.offsets is not None:
            v = v + torch.as_tensor(self.offsets, device=v.device)[:, None, None]
        return v

    def values(self) -> np.ndarray:
        """(K, N, nz) tracer values as float64."""
        return self.full_values()[:, :, : self.mesh.nz].cpu().numpy()

    def workspace_view(self, name: str):
        """One workspace array per tracer: vf (E,LZ), adfh (K,E,LZ), lo (K,N,LZ),
        adfv (K,N,LW), rp / rm (K,N,LZ). Views of the workspace in the FP64
        form; copies when the FP32 form groups tracers. The FP32 form stores the
        low-order solution as its increment LO - T: "lo" adds the current T back
        (read it before the update stage changes T), "lo_increment" is the
        stored increment."""
        if name == "lo" and self.precision == "fp32":
            return self.workspace_view("lo_increment") + self.from_layout(self.T)
        if name == "lo_increment":
            if self.precision != "fp32":
                raise ValueError("only the FP32 form stores the LO increment")
            name = "lo"
        m = self.mesh
        L = _lib.load()
        offs = (ctypes.c_longlong * 7)()
        _lib.check(L.fgb_workspace_offsets(m.handle, _PREC[self.precision], self.K, offs), "offsets")
        slot = {"vf": 0, "adfh": 2, "lo": 3, "adfv": 4, "rp": 5, "rm": 5}[name]
        G, V = self.G, self.V
        rows = {"vf": None, "adfh": (m.E, m.LZ), "lo": (m.N, m.LZ), "adfv": (m.N, m.LW), "rp": (m.N, m.LZ, 2),
                "rm": (m.N, m.LZ, 2)}[name]
        shape = (m.E, m.LZ) if rows is None else (G, *rows, V)
        n = int(np.prod(shape))
        es = self.T.element_size()
        v = self.workspace[offs[slot]: offs[slot] + n * es].view(self.dtype).view(shape)
        if rows is None:
            return v
        # (G, rows..., V) -> (K, rows...)
        v = v.movedim(-1, 1).reshape(self.K, *rows)
        if name == "rp":
            return v[..., 0]
        if name == "rm":
            return v[..., 1]
        return v

    def stats(self) -> np.ndarray:
        """(K, 4): min, max, plain sum, NaN count over all layers of the owned nodes."""
        L = _lib.load()
        m = self.mesh
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        if self.V == 1:
            _lib.check(L.fgb_tracer_stats(m.handle, _PREC[self.precision], ctypes.c_void_p(self.T.data_ptr()),
                                          m.N * m.LZ, self.K, ctypes.c_void_p(self._stats_scratch.data_ptr()),
                                          ctypes.c_void_p(self._stats_out.data_ptr()), stream), "fgb_tracer_stats")
        else:
            _lib.check(L.fgb_tracer_stats_grouped(m.handle, ctypes.c_void_p(self.T.data_ptr()), m.N * m.LZ * self.V,
                                                  self.K, self.V, ctypes.c_void_p(self._stats_scratch.data_ptr()),
                                                  ctypes.c_void_p(self._stats_out.data_ptr()), stream),
                       "fgb_tracer_stats_grouped")
        out = self._stats_out.cpu().numpy()
        if self.offsets is not None:
            out = out.copy()
            out[:, 0] += self.offsets
            out[:, 1] += self.offsets
            out[:, 2] += self.offsets * float(m.N * m.nz)
        return out
