"""Masked multigrid Helmholtz solver on the GPU with the interface of the
reference's MG_Helmholtz (mapping/models/model_qgsw/helmholtz_multigrid.py
156-419):

    solver = MG_Helmholtz(dx, dy, nx, ny, coef_ugrid, coef_vgrid, lambd=lam,
                          mask=mask, niter_bottom=-1, max_ite=20)
    f = solver.solve(rhs)            # div(c grad f) - lambda f = rhs

Arrays keep the reference's (nl, nx, ny) layout (axis -2 with spacing dx,
axis -1 with spacing dy); ``lambd`` holds one value per system (the
reference's lambd of shape (nl, 1, 1)). NumPy inputs give NumPy outputs,
CUDA tensors give tensors. The whole solve (full-multigrid start and the
max_ite V-cycles) runs in the library's kernels on torch's current stream.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class MG_Helmholtz:
    def __init__(self, dx, dy, nx, ny, coef_ugrid, coef_vgrid, n_levels=None, lambd=None, tol=1e-8, max_ite=20,
                 dtype=torch.float64, device=None, mask=None, niter_bottom=-1, use_compilation=True):
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        if isinstance(dtype, str):
            dtype = torch.float64 if dtype == "float64" else torch.float32
        if dtype not in (torch.float32, torch.float64):
            dtype = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
        self.dtype = dtype
        dev = torch.device(device if isinstance(device, (str, torch.device)) and str(device) != "cpu" else "cuda")
        self.device = torch.device("cuda", dev.index if dev.index is not None else torch.cuda.current_device())
        self.nx, self.ny, self.dx, self.dy = int(nx), int(ny), float(dx), float(dy)
        self.lambd = np.zeros(1) if lambd is None else np.asarray(_np(lambd), dtype=np.float64).reshape(-1)
        self.n_levels_req = 0 if n_levels is None else int(n_levels)
        self.max_ite, self.niter_bottom, self.tol = int(max_ite), int(niter_bottom), tol
        self.mask = None if mask is None else np.ascontiguousarray(_np(mask), dtype=np.float64).reshape(nx, ny)
        self.lib = _lib.load()
        self._h = None
        self._build(coef_ugrid, coef_vgrid)

    def _build(self, coef_ugrid, coef_vgrid):
        cu = np.ascontiguousarray(_np(coef_ugrid), dtype=np.float64).reshape(self.nx + 1, self.ny)
        cv = np.ascontiguousarray(_np(coef_vgrid), dtype=np.float64).reshape(self.nx, self.ny + 1)
        dptr = ctypes.POINTER(ctypes.c_double)
        lam = np.ascontiguousarray(self.lambd)
        d = _lib.VdMgDesc(self.nx, self.ny, lam.size, _lib.VD_F64 if self.dtype == torch.float64 else _lib.VD_F32,
                          self.dx, self.dy, lam.ctypes.data_as(dptr),
                          self.mask.ctypes.data_as(dptr) if self.mask is not None else None,
                          cu.ctypes.data_as(dptr), cv.ctypes.data_as(dptr), self.n_levels_req, self.max_ite,
                          self.niter_bottom)
        self._destroy()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.vd_mg_plan_create(ctypes.byref(h), ctypes.byref(d)), "vd_mg_plan_create")
        self._h = h
        self.n_levels = int(self.lib.vd_mg_levels(h))
        n = int(self.lib.vd_mg_workspace_bytes(h))
        self._ws = torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)

    def _destroy(self):
        if self._h is not None and self._h.value:
            try:
                self.lib.vd_mg_plan_destroy(self._h)
            except Exception:
                pass
        self._h = None

    def __del__(self):
        self._destroy()

    def _in(self, rhs):
        is_t = isinstance(rhs, torch.Tensor)
        r = rhs if is_t else torch.as_tensor(np.asarray(rhs, dtype=np.float64))
        r = r.to(device=self.device, dtype=self.dtype)
        shape = r.shape
        r = r.reshape(-1, self.nx, self.ny)
        if r.shape[0] != self.lambd.size:
            raise ValueError(f"rhs holds {r.shape[0]} systems, lambd {self.lambd.size}")
        return r.contiguous(), shape, is_t

    def solve(self, rhs, coef_ugrid=None, coef_vgrid=None):
        """FMG_Helmholtz (helmholtz_multigrid.py:300-304, 380-419)."""
        if coef_ugrid is not None and coef_vgrid is not None:
            self._build(coef_ugrid, coef_vgrid)
        r, shape, is_t = self._in(rhs)
        f = torch.empty_like(r)
        _lib.check(self.lib.vd_mg_solve(self._h, _ptr(r), _ptr(f), _ptr(self._ws), self._ws.numel(), _stream()),
                   "vd_mg_solve")
        f = f.reshape(shape)
        return f if is_t else f.double().cpu().numpy()

    def residual(self, f, rhs):
        """rhs - H f on the finest level (helmholtz_multigrid.py:102-114)."""
        r, shape, is_t = self._in(rhs)
        ff, _, _ = self._in(f)
        out = torch.empty_like(r)
        _lib.check(self.lib.vd_mg_residual(self._h, _ptr(ff), _ptr(r), _ptr(out), _stream()), "vd_mg_residual")
        out = out.reshape(shape)
        return out if is_t else out.double().cpu().numpy()


def _np(x):
    if isinstance(x, torch.Tensor):
        return x.detach().double().cpu().numpy()
    return np.asarray(x)


class MaskedDirichletMG:
    """Multigrid solve of the masked Dirichlet Helmholtz problems of the
    multilayer QG PV inversion (qg.py:222-298, which the reference solves by
    DST plus capacitance matrices): per mode m on n0 x n1 interior nodes,
    lap5(u) - lambda_m u = b where mask != 0, u = 0 on land and beyond the
    walls (vd_mgd_*). ``solve(b)`` takes [nmode][batch][n0][n1] tensors, or
    the interior of padded fields through ``ld`` / ``fs`` strides; each system
    stops at the relative residual ``tol`` (float64 norms)."""

    def __init__(self, n0, n1, d0, d1, lambdas, mask=None, dtype=torch.float64, tol=1e-8, max_cycles=24,
                 device=None, graphs=True):
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        self.n0, self.n1, self.dtype = int(n0), int(n1), dtype
        self.device = torch.device(device if device is not None else "cuda")
        self.lambdas = np.ascontiguousarray(np.asarray(lambdas, dtype=np.float64).reshape(-1))
        self.nmode = self.lambdas.size
        self.tol = float(tol)
        self.mask = None if mask is None else np.ascontiguousarray(np.asarray(mask, dtype=np.float64)
                                                                   .reshape(self.n0, self.n1))
        dptr = ctypes.POINTER(ctypes.c_double)
        d = _lib.VdMgdDesc(self.n0, self.n1, self.nmode, _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32,
                           float(d0), float(d1), self.lambdas.ctypes.data_as(dptr),
                           self.mask.ctypes.data_as(dptr) if self.mask is not None else None, int(max_cycles),
                           self.tol)
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.vd_mgd_plan_create(ctypes.byref(h), ctypes.byref(d)), "vd_mgd_plan_create")
        self._h = h
        self.levels = int(self.lib.vd_mgd_levels(h))
        self.coarse_unknowns = int(self.lib.vd_mgd_coarse_unknowns(h))
        self._ws = {}
        self.rel = None
        self.graphs = bool(graphs)
        self._graphs = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.vd_mgd_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def workspace(self, batch):
        ws = self._ws.get(batch)
        if ws is None:
            n = int(self.lib.vd_mgd_workspace_bytes(self._h, batch))
            ws = torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)
            self._ws[batch] = ws
            self.rel = torch.zeros(self.nmode * batch, dtype=torch.float64, device=self.device)
        return ws

    def _raw(self, batch, b, ldb, fsb, u, ldu, fsu, rel):
        ws = self.workspace(batch)
        _lib.check(self.lib.vd_mgd_solve(self._h, int(batch), _ptr(b), int(ldb), int(fsb), _ptr(u), int(ldu),
                                         int(fsu), _ptr(rel), _ptr(ws), ws.numel(), _stream()), "vd_mgd_solve")

    def _graph(self, batch):
        """The whole solve of ``batch`` windows captured once on owned
        buffers (a solve is some thousands of short launches); replayed by
        :meth:`solve_strided` between a copy in and a copy out."""
        gr = self._graphs.get(batch)
        if gr is None:
            shape = (self.nmode, batch, self.n0, self.n1)
            bin_ = torch.zeros(shape, dtype=self.dtype, device=self.device)
            uout = torch.zeros(shape, dtype=self.dtype, device=self.device)
            rel = torch.zeros(self.nmode * batch, dtype=torch.float64, device=self.device)
            fs = self.n0 * self.n1
            self._raw(batch, bin_, self.n1, fs, uout, self.n1, fs, rel)      # warm-up outside the capture
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            st = torch.cuda.Stream(self.device)
            st.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(st):
                with torch.cuda.graph(g, stream=st):
                    self._raw(batch, bin_, self.n1, fs, uout, self.n1, fs, rel)
            torch.cuda.current_stream(self.device).wait_stream(st)
            gr = (g, bin_, uout, rel)
            self._graphs[batch] = gr
        return gr

    def solve_strided(self, batch, b, ldb, fsb, u, ldu, fsu):
        """In-place form: b / u point at element (0, 0) of system 0 (tensor
        views whose data_ptr is that element) with the given strides. Outside
        stream capture the solve replays a captured graph."""
        self.workspace(batch)
        if self.rel is None or self.rel.numel() != self.nmode * batch:
            self.rel = torch.zeros(self.nmode * batch, dtype=torch.float64, device=self.device)
        if not self.graphs or torch.cuda.is_current_stream_capturing():
            self._raw(batch, b, ldb, fsb, u, ldu, fsu, self.rel)
            return u
        g, bin_, uout, rel = self._graph(batch)
        n = self.nmode * batch
        bview = torch.as_strided(b, (n, self.n0, self.n1), (fsb, ldb, 1))
        uview = torch.as_strided(u, (n, self.n0, self.n1), (fsu, ldu, 1))
        bin_.view(n, self.n0, self.n1).copy_(bview)
        g.replay()
        uview.copy_(uout.view(n, self.n0, self.n1))
        self.rel.copy_(rel)
        return u

    def solve(self, b):
        """u [nmode][batch][n0][n1] = A^-1 b."""
        if b.dtype != self.dtype or b.device.type != "cuda" or b.shape[-2:] != (self.n0, self.n1):
            raise ValueError("b must be a CUDA tensor [nmode][batch][n0][n1] of the plan dtype")
        b = b.reshape(self.nmode, -1, self.n0, self.n1).contiguous()
        u = torch.empty_like(b)
        fs = self.n0 * self.n1
        return self.solve_strided(b.shape[1], b, self.n1, fs, u, self.n1, fs)

