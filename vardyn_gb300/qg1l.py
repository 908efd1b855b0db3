"""Torch-facing wrapper of the QG 1.5-layer plan of libvardyn_gb300.

A :class:`QG1LPlan` owns one ``vd_qg1l_plan`` (constant tables on the GPU)
and hands device pointers of torch tensors to the C ABI. Fields are torch
tensors of shape ``[ny, nx]`` or ``[batch, ny, nx]`` on the plan's device in
the plan's dtype. Workspaces come from the torch caching allocator; the C
calls allocate nothing and run on torch's current CUDA stream.
"""
import ctypes

import numpy as np
import torch

from . import _lib

SECONDS_PER_DAY = 3600.0 * 24.0


def build_mask(ny, nx, ssh=None):
    """Cell mask of the reference's Qgm (mapping/models/model_qg1l/jqgm.py:178-217):
    3 in the interior, 1 on the outer ring, 2 on the second ring and on rows /
    columns -3 (the reference marks -3 but not 2), and around land: 1 within
    one cell (Chebyshev distance), 2 within two cells, 0 on land (NaN SSH).
    The reference visits land points one by one; the result does not depend
    on the visiting order, so dilations give the same mask."""
    mask = np.full((ny, nx), 3, dtype=np.int8)
    mask[0, :] = 1
    mask[-1, :] = 1
    mask[:, 0] = 1
    mask[:, -1] = 1
    mask[1, 1:-1] = 2
    mask[-2, 1:-1] = 2
    mask[-3, 1:-1] = 2
    mask[1:-1, 1] = 2
    mask[1:-1, -2] = 2
    mask[1:-1, -3] = 2
    if ssh is not None:
        land = np.isnan(np.asarray(ssh, dtype=np.float64))
        if land.any():
            def dilate(b, r):
                pad = np.pad(b, r)
                out = np.zeros_like(b)
                for a in range(2 * r + 1):
                    for c in range(2 * r + 1):
                        out |= pad[a:a + ny, c:c + nx]
                return out
            d1 = dilate(land, 1)
            d2 = dilate(land, 2)
            new = mask.copy()
            new[d2 & (mask == 3)] = 2
            new[d1 & (mask >= 2)] = 1
            new[land] = 0
            mask = new
    return mask


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class QG1LPlan:
    """Constants of one QG 1.5-layer configuration on one GPU.

    Arguments mirror ``Qgm.__init__`` (jqgm.py:113-236) after its reductions:
    scalar ``dx``, ``dy``, ``f`` (mean Coriolis), ``c``; optional ``beta``
    (full-grid [ny, nx] array, rows 1..ny-2 used), ``fbathy`` (f times the
    bathymetry PV term), ``Kdiffus`` and ``mask`` (from :func:`build_mask`).
    """

    def __init__(self, ny, nx, dx, dy, dt, f, c, g=9.81, time_scheme="rk2",
                 dtype=torch.float32, Kdiffus=None, mask=None, beta=None, fbathy=None,
                 device=None, dst_engine="auto"):
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        self.device = torch.device(device if device is not None else "cuda")
        self.ny, self.nx = int(ny), int(nx)
        self.dtype = dtype
        self.dt = float(dt)
        self.time_scheme = time_scheme
        if time_scheme not in _lib.SCHEMES:
            raise ValueError(f"unknown time_scheme {time_scheme!r}")
        self.mask = (build_mask(ny, nx) if mask is None else np.ascontiguousarray(mask, dtype=np.int8))
        self._keep = []
        d = _lib.VdDesc()
        d.ny, d.nx = self.ny, self.nx
        d.dtype = _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32
        d.time_scheme = _lib.SCHEMES[time_scheme]
        d.dx, d.dy, d.dt = float(dx), float(dy), float(dt)
        d.g, d.f, d.c = float(g), float(f), float(c)
        if dst_engine not in ("auto", "fma"):
            raise ValueError("dst_engine is 'auto' (tensor cores for float32) or 'fma'")
        d.dst_engine = _lib.VD_DST_AUTO if dst_engine == "auto" else _lib.VD_DST_FMA
        self.dst_engine = dst_engine
        d.has_Kdiffus = 0 if Kdiffus is None else 1
        d.Kdiffus = 0.0 if Kdiffus is None else float(Kdiffus)
        m = np.ascontiguousarray(self.mask, dtype=np.int8)
        self._keep.append(m)
        d.mask_host = m.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))
        for name, arr in (("beta_host", beta), ("fbathy_host", fbathy)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64)
                if a.shape != (self.ny, self.nx):
                    raise ValueError(f"{name} must be [ny, nx]")
                self._keep.append(a)
                setattr(d, name, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self._desc = d
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("vd_qg1l_plan_create", ctypes.byref(handle), ctypes.byref(d))
        self._h = handle
        self._lib = _lib.load()
        self.nstage = self._lib.vd_qg1l_nstage(self._h)
        # float32 plans carry the PV state as a compensated pair (q, q_lo)
        self.compensated = dtype == torch.float32
        self._ws = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.vd_qg1l_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    # ---------------- launch schedule of the inversion ----------------
    SCHEDULE_KEYS = ("engine", "tc_group_fwd", "tc_group_inv", "fma_rows", "tridiag_rows", "tridiag_lean",
                     "stencil_loads")

    def schedule(self):
        """The inversion's launch schedule (vd_qg1l_schedule; 0 = built-in rule)."""
        s = _lib.VdQg1lSchedule()
        _lib.call("vd_qg1l_get_schedule", self._h, ctypes.byref(s))
        return {k: int(getattr(s, k)) for k in self.SCHEDULE_KEYS}

    def set_schedule(self, **kw):
        """Set schedule fields (the others keep their values); see
        vd_qg1l_set_schedule for the choices. Raises on a choice the plan
        cannot run."""
        cur = self.schedule()
        for k, v in kw.items():
            if k not in cur:
                raise KeyError(k)
            cur[k] = int(v)
        _lib.call("vd_qg1l_set_schedule", self._h, ctypes.byref(_lib.VdQg1lSchedule(**cur)))
        return cur

    # ---------------- buffers ----------------
    def workspace(self, batch):
        ws = self._ws.get(batch)
        if ws is None:
            nbytes = self._lib.vd_qg1l_workspace_bytes(self._h, batch)
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._ws[batch] = ws
        return ws

    def traj_bytes(self, batch, nstep):
        return int(self._lib.vd_qg1l_traj_bytes(self._h, batch, nstep))

    def new_traj(self, batch, nstep):
        esize = torch.empty((), dtype=self.dtype).element_size()
        n = self.traj_bytes(batch, nstep) // esize
        return torch.zeros(n, dtype=self.dtype, device=self.device)

    def field(self, batch=1, fill=0.0):
        return torch.full((batch, self.ny, self.nx), fill, dtype=self.dtype, device=self.device)

    def _as_batch(self, x, name):
        if not isinstance(x, torch.Tensor):
            raise TypeError(f"{name} must be a torch tensor")
        if x.device.type != "cuda" or x.dtype != self.dtype:
            raise TypeError(f"{name} must be a CUDA {self.dtype} tensor")
        if x.dim() == 2:
            x = x.unsqueeze(0)
        if x.shape[-2:] != (self.ny, self.nx):
            raise ValueError(f"{name} has shape {tuple(x.shape)}, grid is {(self.ny, self.nx)}")
        return x.contiguous()

    # ---------------- API mirrors of Qgm ----------------
    def h2pv(self, h, hb):
        h, hb = self._as_batch(h, "h"), self._as_batch(hb, "hb")
        q = torch.empty_like(h)
        _lib.call("vd_qg1l_h2pv", self._h, h.shape[0], _ptr(h), _ptr(hb), _ptr(q), _stream())
        return q

    def h2uv(self, h):
        h = self._as_batch(h, "h")
        u, v = torch.empty_like(h), torch.empty_like(h)
        _lib.call("vd_qg1l_h2uv", self._h, h.shape[0], _ptr(h), _ptr(u), _ptr(v), _stream())
        return u, v

    def rhs(self, u, v, q):
        u, v, q = self._as_batch(u, "u"), self._as_batch(v, "v"), self._as_batch(q, "q")
        r = torch.empty_like(q)
        _lib.call("vd_qg1l_rhs", self._h, q.shape[0], _ptr(u), _ptr(v), _ptr(q), _ptr(r), _stream())
        return r

    def pv2h(self, q, hb, qb):
        q, hb, qb = self._as_batch(q, "q"), self._as_batch(hb, "hb"), self._as_batch(qb, "qb")
        h = torch.empty_like(q)
        ws = self.workspace(q.shape[0])
        _lib.call("vd_qg1l_pv2h", self._h, q.shape[0], _ptr(q), _ptr(hb), _ptr(qb), _ptr(h),
                  _ptr(ws), ws.numel(), _stream())
        return h

    def step(self, h0, hb, nstep=1, traj=None, out=None):
        h0, hb = self._as_batch(h0, "h0"), self._as_batch(hb, "hb")
        B = h0.shape[0]
        out = torch.empty_like(h0) if out is None else out
        ws = self.workspace(B)
        _lib.call("vd_qg1l_step", self._h, B, _ptr(h0), _ptr(hb), int(nstep), _ptr(out),
                  _ptr(traj), _ptr(ws), ws.numel(), _stream())
        return out

    def step_tgl(self, dh0, h0, hb, nstep=1):
        dh0, h0, hb = (self._as_batch(dh0, "dh0"), self._as_batch(h0, "h0"),
                       self._as_batch(hb, "hb"))
        B = h0.shape[0]
        out = torch.empty_like(h0)
        ws = self.workspace(B)
        _lib.call("vd_qg1l_step_tgl", self._h, B, _ptr(dh0), _ptr(h0), _ptr(hb), int(nstep),
                  _ptr(out), _ptr(ws), ws.numel(), _stream())
        return out

    def step_adj(self, adh1, h0, hb, nstep=1, traj=None, traj_ready=False):
        adh1, h0, hb = (self._as_batch(adh1, "adh1"), self._as_batch(h0, "h0"),
                        self._as_batch(hb, "hb"))
        B = h0.shape[0]
        if traj is None:
            traj = self.new_traj(B, nstep)
            traj_ready = False
        out = torch.empty_like(h0)
        ws = self.workspace(B)
        _lib.call("vd_qg1l_step_adj", self._h, B, _ptr(adh1), _ptr(h0), _ptr(hb), int(nstep),
                  _ptr(out), _ptr(traj), int(bool(traj_ready)), _ptr(ws), ws.numel(), _stream())
        return out

    def rk_stage(self, hs, qs, qbase, k=(), c=(), cself=0.0, k_out=None):
        """One forward Runge-Kutta stage (vd_qg1l_rk_stage): returns
        q_out = qbase + sum c[t] k[t] + cself * rhs(h2uv(hs), qs)."""
        hs, qs, qbase = self._as_batch(hs, "hs"), self._as_batch(qs, "qs"), self._as_batch(qbase, "qbase")
        ks = [self._as_batch(x, "k") for x in k]
        kp = (ctypes.c_void_p * max(1, len(ks)))(*[x.data_ptr() for x in ks])
        cp = (ctypes.c_double * max(1, len(ks)))(*[float(x) for x in c])
        q_out = torch.empty_like(qs)
        _lib.call("vd_qg1l_rk_stage", self._h, qs.shape[0], _ptr(hs), _ptr(qs), _ptr(qbase), len(ks), kp, cp,
                  float(cself), _ptr(k_out), _ptr(q_out), _stream())
        return q_out

    def rk_stage_adj(self, hs, qs, g=(), c=(), acc=()):
        """Adjoint of one stage's tendency (vd_qg1l_rk_stage_adj): returns
        (adq, adh) for the stage cotangent sum c[t] g[t] plus the addends acc
        (on the tendency points)."""
        hs, qs = self._as_batch(hs, "hs"), self._as_batch(qs, "qs")
        gs = [self._as_batch(x, "g") for x in g]
        ac = [self._as_batch(x, "acc") for x in acc]
        gp = (ctypes.c_void_p * max(1, len(gs)))(*[x.data_ptr() for x in gs])
        cp = (ctypes.c_double * max(1, len(gs)))(*[float(x) for x in c])
        ap = (ctypes.c_void_p * max(1, len(ac)))(*[x.data_ptr() for x in ac])
        adq, adh = torch.empty_like(qs), torch.empty_like(qs)
        _lib.call("vd_qg1l_rk_stage_adj", self._h, qs.shape[0], _ptr(hs), _ptr(qs), len(gs), gp, cp, len(ac), ap,
                  _ptr(adq), _ptr(adh), _stream())
        return adq, adh

    # ---------------- state-level API (window engine) ----------------
    def new_qlo(self, batch):
        """Low-part buffer of the compensated PV state ([batch, ny, nx]), or
        None for float64 plans, which step with the reference's plain
        arithmetic."""
        return self.field(batch) if self.compensated else None

    def init_state(self, h, hb, q, qb, qlo=None):
        _lib.call("vd_qg1l_init_state", self._h, h.shape[0] if h.dim() == 3 else 1, _ptr(h),
                  _ptr(hb), _ptr(q), _ptr(qb), _ptr(qlo), _stream())

    def advance(self, batch, traj, traj_steps, first, nstep, hb, qb, qlo=None):
        ws = self.workspace(batch)
        _lib.call("vd_qg1l_advance", self._h, batch, _ptr(traj), int(traj_steps), int(first),
                  int(nstep), _ptr(hb), _ptr(qb), _ptr(qlo), _ptr(ws), ws.numel(), _stream())

    def advance_adj(self, batch, traj, traj_steps, first, nstep, adh, adq):
        ws = self.workspace(batch)
        _lib.call("vd_qg1l_advance_adj", self._h, batch, _ptr(traj), int(traj_steps), int(first),
                  int(nstep), _ptr(adh), _ptr(adq), _ptr(ws), ws.numel(), _stream())

    def init_state_adj(self, batch, h, adq, adh):
        _lib.call("vd_qg1l_init_state_adj", self._h, batch, _ptr(h), _ptr(adq), _ptr(adh), _stream())

    def finalize(self, batch, h, hb, out, forcing=None, coef=0.0):
        _lib.call("vd_qg1l_finalize", self._h, batch, _ptr(h), _ptr(hb), _ptr(forcing),
                  float(coef), _ptr(out), _stream())

    def scale(self, x, d):
        """out[b] = d * x[b] elementwise (d: [ny, nx] on the device)."""
        x = self._as_batch(x, "x")
        d = self._as_batch(d, "d")
        out = torch.empty_like(x)
        _lib.call("vd_diag_axpy", _lib.VD_F64 if self.dtype == torch.float64 else _lib.VD_F32,
                  ctypes.c_longlong(x.numel()), ctypes.c_longlong(self.ny * self.nx), _ptr(d), _ptr(x), None,
                  _ptr(out), _stream())
        return out

    def traj_view(self, traj, batch, nstep):
        """[nstep*nstage+1, 2, batch, ny, nx] view of a trajectory buffer."""
        return traj.view(nstep * self.nstage + 1, 2, batch, self.ny, self.nx)
