"""Spectral Helmholtz solver with Neumann boundaries, on the GPU.

Drop-in for mapping/models/model_qgsw/helmholtz.py:

  compute_laplace_dctII      22-30
  HelmholtzNeumannSolver     187-303 on a rectangular (all-ocean) domain,
                             where ``solve`` is the fast diagonalisation G
                             alone (solve_helmholtz_dctII, 81-87)

The solve is the library's vd_neumann_solve: the unnormalised DCT-II pair
along each axis through FFTs in shared memory (vardyn_gb300/csrc/vd_neumann.cu).
The shallow-water model's barotropic filter uses the same solve inside its
right-hand side (vardyn_gb300/sw.py, ``barotropic_filter``).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .qg1l import _ptr, _stream

__all__ = ["HelmholtzNeumannSolver", "compute_laplace_dctII"]


def compute_laplace_dctII(nx, ny, dx, dy, dtype=torch.float64, device=None):
    """DCT-II eigenvalues of the 5-point Laplacian (helmholtz.py:22-30),
    shape [nx, ny] (dx, dy scalars or [nx, ny] arrays)."""
    x, y = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
    lap = 2 * (np.cos(np.pi / nx * x) - 1) / np.asarray(dx, dtype=np.float64) ** 2 \
        + 2 * (np.cos(np.pi / ny * y) - 1) / np.asarray(dy, dtype=np.float64) ** 2
    return torch.as_tensor(lap, dtype=dtype, device=device)


def _flat(a, nx, ny):
    """(array, spatial flag) of a scalar or an [..., nx, ny]-broadcastable field."""
    a = np.asarray(a, dtype=np.float64)
    if a.size == 1:
        return np.array(a.reshape(1)), 0
    return np.array(np.broadcast_to(a.reshape(a.shape[-2:]), (nx, ny))), 1


class HelmholtzNeumannSolver:
    """HelmholtzNeumannSolver(nx, ny, dx, dy, lambd, dtype, mask) of
    helmholtz.py:187-225: solves ``div grad w - lambd w = rhs`` with Neumann
    boundaries on [..., nx, ny] fields. ``dx``, ``dy`` and ``lambd`` are
    scalars or [nx, ny] fields (the reference broadcasts them into its
    eigenvalue table). Masks with land raise: the capacitance correction of
    irregular domains (232-303) is not built, and the reference's one caller
    (the shallow-water filter) cannot construct it (254)."""

    def __init__(self, nx, ny, dx, dy, lambd, dtype=torch.float64, mask=None, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("vardyn_gb300 needs a CUDA device (no CPU path)")
        if mask is not None and np.any(np.asarray(mask, dtype=np.float64) < 0.5):
            raise NotImplementedError("Neumann solve on a masked domain (capacitance correction, "
                                      "helmholtz.py:232-303)")
        self.nx, self.ny = int(nx), int(ny)
        self.dtype = dtype
        self.device = torch.device(device if device is not None else "cuda")
        self.lambd = lambd
        dxa, sdx = _flat(dx, self.nx, self.ny)
        dya, sdy = _flat(dy, self.nx, self.ny)
        if sdx or sdy:   # one flag covers both spacings
            dxa = np.array(np.broadcast_to(dxa if sdx else dxa[0], (self.nx, self.ny)))
            dya = np.array(np.broadcast_to(dya if sdy else dya[0], (self.nx, self.ny)))
            sdx = 1
        lam, slam = _flat(lambd, self.nx, self.ny)
        self.helmholtz_dctII = (compute_laplace_dctII(self.nx, self.ny, dxa if sdx else float(dxa[0]),
                                                      dya if sdx else float(dya[0]), dtype, self.device)
                                - torch.as_tensor(lam if slam else float(lam[0]), dtype=dtype, device=self.device))
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("vd_neumann_plan_create", ctypes.byref(handle), self.nx, self.ny,
                      _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32, dxa.ctypes.data, dya.ctypes.data, sdx,
                      lam.ctypes.data, slam)
        self._h = handle
        self._lib = _lib.load()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.vd_neumann_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def solve(self, rhs):
        """HelmholtzNeumannSolver.solve (296-303) of rhs [..., nx, ny]."""
        numpy_in = not torch.is_tensor(rhs)
        r = torch.as_tensor(np.asarray(rhs) if numpy_in else rhs, device=self.device)
        if r.shape[-2:] != (self.nx, self.ny):
            raise ValueError(f"rhs must end in ({self.nx}, {self.ny}), got {tuple(r.shape)}")
        out_dtype = r.dtype
        x = r.to(self.dtype).contiguous().reshape(-1, self.nx, self.ny)
        out = torch.empty_like(x)
        with torch.cuda.device(self.device):
            for s in range(0, x.shape[0], 65535):
                n = min(65535, x.shape[0] - s)
                _lib.call("vd_neumann_solve", self._h, n, _ptr(x[s:s + n]), _ptr(out[s:s + n]), _stream())
        out = out.reshape(r.shape).to(out_dtype)
        return out.cpu().numpy() if numpy_in else out
