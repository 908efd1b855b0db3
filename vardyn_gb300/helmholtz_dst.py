"""Spectral (DST-I) Helmholtz solvers of the multi-layer QG model, on the GPU.

Drop-in for mapping/models/model_qgsw/helmholtz.py:

  compute_laplace_dstI            129-135
  solve_helmholtz_dstI            138-143
  compute_capacitance_matrices    146-169
  solve_helmholtz_dstI_cmm        172-184

Axis convention of the reference: fields are ``[..., nx+1, ny+1]`` with the
first spatial axis along x (spacing dx); right-hand sides are the
``[..., nx-1, ny-1]`` interiors and the last non-spatial axis indexes the
``nl`` modes of ``helm = laplace_dstI - f0**2 * lambd`` (qg.py:74-78).

Every operator of the reference has that form, which separates: the solve of
one mode is the QG plan's pv2h (orthonormal x-DST-I, y-tridiagonal solve,
inverse x-DST-I) on a plan built with g = f = 1 and c = 1/sqrt(shift),
whose operator is exactly laplace_dstI - shift. :class:`HelmholtzDST` holds
one such plan per mode; the functional drop-ins recover (dx, dy, shift) from
a ``helm`` array and refuse arrays of any other form.
"""
import weakref

import numpy as np
import torch

from . import _lib
from .qg1l import QG1LPlan, _ptr, _stream

__all__ = ["HelmholtzDST", "compute_laplace_dstI", "solve_helmholtz_dstI",
           "compute_capacitance_matrices", "solve_helmholtz_dstI_cmm"]


def compute_laplace_dstI(nx, ny, dx, dy, dtype=torch.float64, device=None):
    """DST-I eigenvalues of the 5-point Laplacian (helmholtz.py:129-135),
    shape [nx-1, ny-1]."""
    x, y = np.meshgrid(np.arange(1, nx, dtype=np.float64), np.arange(1, ny, dtype=np.float64), indexing="ij")
    lap = 2 * (np.cos(np.pi / nx * x) - 1) / dx ** 2 + 2 * (np.cos(np.pi / ny * y) - 1) / dy ** 2
    return torch.as_tensor(lap, dtype=dtype, device=device)


class HelmholtzDST:
    """Solver of ``div grad u - shift[l] u = rhs`` on an (nx+1) x (ny+1) grid
    with u = 0 on the walls before edge padding, one mode per entry of
    ``shift`` (the reference's ``f0**2 * lambd``).

    Output fields are ``[..., nl, nx+1, ny+1]`` with the walls edge-padded,
    as solve_helmholtz_dstI returns them. ``dtype`` float64 runs the FMA DST;
    float32 runs the tensor-core DST (3xTF32)."""

    CHUNK = 256  # unit solves per batch when building capacitance matrices

    def __init__(self, nx, ny, dx, dy, shift, dtype=torch.float64, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        self.nx, self.ny = int(nx), int(ny)
        self.dx, self.dy = float(dx), float(dy)
        self.shift = [float(s) for s in np.asarray(shift, dtype=np.float64).ravel()]
        if not self.shift:
            raise ValueError("shift needs at least one mode")
        if any(s < 0 for s in self.shift):
            raise ValueError("shift must be >= 0 (the operator is laplace_dstI - shift)")
        self.nl = len(self.shift)
        self.dtype = dtype
        self.device = torch.device(device if device is not None else "cuda")
        self._dt = _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32
        # plan rows run along the reference's x axis: plan (ny, nx, dx, dy) =
        # reference (nx+1, ny+1, dy, dx)
        self.plans = [QG1LPlan(self.nx + 1, self.ny + 1, self.dy, self.dx, 1.0, 1.0,
                               1.0 / np.sqrt(s) if s > 0 else 1e150, g=1.0, dtype=dtype, device=self.device)
                      for s in self.shift]

    # ---------------- internals ----------------
    @property
    def field_shape(self):
        return (self.nx + 1, self.ny + 1)

    def _modes_first(self, rhs):
        """[..., nl, nx-1, ny-1] -> zero-walled [nl, nb, nx+1, ny+1] and the
        leading shape."""
        rhs = torch.as_tensor(rhs, device=self.device)
        if rhs.shape[-2:] != (self.nx - 1, self.ny - 1):
            raise ValueError(f"rhs interior {tuple(rhs.shape[-2:])} does not match {(self.nx - 1, self.ny - 1)}")
        lead = tuple(rhs.shape[:-2])
        if self.nl == 1:
            r = rhs.reshape(1, -1, self.nx - 1, self.ny - 1)
        else:
            if rhs.dim() < 3 or rhs.shape[-3] != self.nl:
                raise ValueError(f"rhs needs {self.nl} modes on axis -3, got shape {tuple(rhs.shape)}")
            r = rhs.reshape(-1, self.nl, self.nx - 1, self.ny - 1).transpose(0, 1)
        nb = r.shape[1]
        pad = torch.zeros((self.nl, nb) + self.field_shape, dtype=self.dtype, device=self.device)
        pad[:, :, 1:-1, 1:-1] = r
        return pad, lead

    def _modes_last(self, f, lead):
        return f.transpose(0, 1).reshape(lead + self.field_shape)

    def _solve_modes(self, q, out):
        """out[l] = (laplace - shift[l])^-1 q[l] on the interiors, zero walls."""
        for l, p in enumerate(self.plans):
            nb = q.shape[1]
            if nb == 0:
                continue
            ws = p.workspace(nb)
            _lib.call("vd_qg1l_pv2h", p.handle, nb, _ptr(q[l]), None, None, _ptr(out[l]),
                      _ptr(ws), ws.numel(), _stream())
        return out

    def _edge_pad(self, src, dst, mask=None):
        n = src.shape[0] * src.shape[1]
        _lib.call("vd_edge_pad", self._dt, n, self.nx + 1, self.ny + 1, _ptr(src), _ptr(mask), _ptr(dst),
                  _stream())
        return dst

    def _bidx(self, bound_xids, bound_yids):
        bx = np.asarray(bound_xids, dtype=np.int64).ravel()
        by = np.asarray(bound_yids, dtype=np.int64).ravel()
        if bx.shape != by.shape:
            raise ValueError("bound_xids and bound_yids differ in length")
        if bx.size and (bx.min() < 0 or bx.max() >= self.nx - 1 or by.min() < 0 or by.max() >= self.ny - 1):
            raise ValueError("boundary points must lie in the [nx-1, ny-1] interior")
        flat = (bx + 1) * (self.ny + 1) + (by + 1)
        return torch.as_tensor(flat.astype(np.int32), device=self.device)

    # ---------------- API ----------------
    def solve(self, rhs):
        """solve_helmholtz_dstI (helmholtz.py:138-143)."""
        q, lead = self._modes_first(rhs)
        sol = torch.empty_like(q)
        self._solve_modes(q, sol)
        self._edge_pad(sol, sol)
        return self._modes_last(sol, lead)

    def capacitance_matrices(self, bound_xids, bound_yids):
        """compute_capacitance_matrices (helmholtz.py:146-169): for every mode
        the inverse of G[i][m] = (unit solve at boundary point m) at point i.
        The unit solves run on the GPU in batches; the M x M inversions run
        on the host in float64 (set-up, like the plan tables)."""
        bidx = self._bidx(bound_xids, bound_yids)
        M = bidx.numel()
        fs = (self.nx + 1) * (self.ny + 1)
        G = np.zeros((self.nl, M, M))
        for m0 in range(0, M, self.CHUNK):
            m1 = min(M, m0 + self.CHUNK)
            q = torch.zeros((self.nl, m1 - m0, fs), dtype=self.dtype, device=self.device)
            q[:, torch.arange(m1 - m0, device=self.device), bidx[m0:m1].long()] = 1
            q = q.view((self.nl, m1 - m0) + self.field_shape)
            sol = torch.empty_like(q)
            self._solve_modes(q, sol)
            G[:, :, m0:m1] = sol.view(self.nl, m1 - m0, fs)[:, :, bidx.long()].transpose(1, 2).double().cpu().numpy()
        cap = np.stack([np.linalg.inv(G[l]) for l in range(self.nl)]) if M else G
        return torch.as_tensor(cap, dtype=self.dtype, device=self.device)

    def solve_cmm(self, rhs, cap_matrices, bound_xids, bound_yids, mask):
        """solve_helmholtz_dstI_cmm (helmholtz.py:172-184): the first solve,
        the capacitance correction at the irregular boundary, the second
        solve, edge padding and the mask."""
        bidx = self._bidx(bound_xids, bound_yids)
        M = bidx.numel()
        cap = torch.as_tensor(cap_matrices, device=self.device).to(self.dtype)
        if cap.numel() != self.nl * M * M:
            raise ValueError(f"cap_matrices must hold {self.nl} matrices of {M} x {M}")
        cap = cap.reshape(self.nl, M, M).contiguous()
        mask = torch.as_tensor(mask, device=self.device).to(self.dtype)
        if tuple(mask.shape[-2:]) != self.field_shape or mask.numel() != np.prod(self.field_shape):
            raise ValueError(f"mask must be {self.field_shape}")
        mask = mask.reshape(self.field_shape).contiguous()
        q, lead = self._modes_first(rhs)
        sol = torch.empty_like(q)
        self._solve_modes(q, sol)
        fs = (self.nx + 1) * (self.ny + 1)
        _lib.call("vd_cmm_correct", self._dt, self.nl, q.shape[1], M, fs, _ptr(cap), _ptr(bidx), _ptr(sol),
                  _ptr(q), _ptr(q), _stream())
        self._solve_modes(q, sol)
        out = torch.empty_like(sol)
        self._edge_pad(sol, out, mask)
        return self._modes_last(out, lead)


# ---------------- functional drop-ins ----------------

def _infer(helm):
    """(nx, ny, dx, dy, shifts) with helm == laplace_dstI(nx, ny, dx, dy) -
    shift[l], from a [..., nl, nx-1, ny-1] array; ValueError otherwise."""
    single = (helm.dtype == torch.float32) if torch.is_tensor(helm) else (np.asarray(helm).dtype == np.float32)
    h = helm.detach().double().cpu().numpy() if torch.is_tensor(helm) else np.asarray(helm, dtype=np.float64)
    if h.ndim < 2 or h.shape[-2] < 2 or h.shape[-1] < 2:
        raise ValueError("helm needs at least 2 x 2 interior points")
    nx, ny = h.shape[-2] + 1, h.shape[-1] + 1
    modes = h.reshape(-1, nx - 1, ny - 1)
    h0 = modes[0]
    # a(k) = 2 (cos(pi k / nx) - 1) / dx^2: the full range a(nx-1) - a(1) is
    # -4 cos(pi / nx) / dx^2, well conditioned for any nx
    dx2 = -4 * np.cos(np.pi / nx) / (h0[-1, 0] - h0[0, 0])
    dy2 = -4 * np.cos(np.pi / ny) / (h0[0, -1] - h0[0, 0])
    if not (dx2 > 0 and dy2 > 0):
        raise ValueError("helm is not laplace_dstI - shift")
    dx, dy = float(np.sqrt(dx2)), float(np.sqrt(dy2))
    lap = compute_laplace_dstI(nx, ny, dx, dy).numpy()
    scale = np.abs(lap).max()
    shifts = []
    for m in modes:
        s = float(np.mean(lap - m))
        if abs(s) <= 1e-13 * scale:
            s = 0.0
        err = np.abs(lap - s - m).max()
        tol = (1e-5 if single else 1e-9) * scale
        if err > tol or s < 0:
            raise ValueError("helm is not laplace_dstI - shift with shift >= 0: the GPU solve needs that form")
        shifts.append(s)
    return nx, ny, dx, dy, shifts


_cache = {}


def _solver_for(helm, dtype, device):
    """Solver for a helm array, cached per array object (torch tensors: the
    same tensor at the same version; NumPy arrays: the same bytes)."""
    if torch.is_tensor(helm):
        key = ("t", id(helm), helm._version, dtype, str(device))
        hit = _cache.get(key)
        if hit is not None and hit[0]() is helm:
            return hit[1]
    else:
        a = np.ascontiguousarray(helm, dtype=np.float64)
        key = ("n", a.shape, a.tobytes(), dtype, str(device))
        hit = _cache.get(key)
        if hit is not None:
            return hit[1]
    nx, ny, dx, dy, shifts = _infer(helm)
    solver = HelmholtzDST(nx, ny, dx, dy, shifts, dtype=dtype, device=device)
    if len(_cache) > 32:
        _cache.clear()
    _cache[key] = (weakref.ref(helm) if torch.is_tensor(helm) else (lambda: None), solver)
    return solver


def _dtype_device(rhs):
    if torch.is_tensor(rhs) and rhs.is_cuda:
        return (rhs.dtype if rhs.dtype in (torch.float32, torch.float64) else torch.float64), rhs.device
    return torch.float64, torch.device("cuda")


def solve_helmholtz_dstI(rhs, helmholtz_dstI):
    """Drop-in for helmholtz.py:138-143 (GPU; returns a CUDA tensor)."""
    dtype, device = _dtype_device(rhs)
    return _solver_for(helmholtz_dstI, dtype, device).solve(rhs)


def compute_capacitance_matrices(helmholtz_dstI, bound_xids, bound_yids, dtype=torch.float64, device=None):
    """Drop-in for helmholtz.py:146-169 (GPU unit solves, host inversion)."""
    device = torch.device(device if device is not None else "cuda")
    return _solver_for(helmholtz_dstI, dtype, device).capacitance_matrices(bound_xids, bound_yids)


def solve_helmholtz_dstI_cmm(rhs, helmholtz_dstI, cap_matrices, bound_xids, bound_yids, mask):
    """Drop-in for helmholtz.py:172-184 (GPU)."""
    dtype, device = _dtype_device(rhs)
    return _solver_for(helmholtz_dstI, dtype, device).solve_cmm(rhs, cap_matrices, bound_xids, bound_yids, mask)
