"""Drop-in multilayer QG model class (mapping/models/model_qgsw/qg.py QG,
19-345) backed by the GB300 kernels: the shallow-water tendencies projected
by P = G o (Q o G)^-1 o Q at every RK3-SSP stage.

``QG(param)`` keeps the reference's constructor and the attributes its
callers read (``A``, ``lambd``, ``Cl2m``, ``Cm2l``, ``helmholtz_dstI``,
``cap_matrices``, ``homsol_wgrid``, ``masks``) and the methods ``step``,
``step_tgl``, ``step_adj``, ``project_qg`` and ``compute_time_derivatives``. ``QG.step`` fails in the reference as shipped
(``SW.step`` passes ``ref_vals`` and wind arguments that QG's overrides do not
accept); here those arguments are passed through, which is the only way the
class can step. Background-SSH boundary handling (``set_boundary_ssh``,
qg.py:100-188, which plots with matplotlib in its body) is not supported.
"""
import numpy as np
import torch

from vardyn_gb300.model_qgsw.sw import SW
from vardyn_gb300.qg_ml import QGPlan


class QG(SW):
    """QG(param) of qg.py:22-43."""

    def _make_plan(self, H, h_wind=None):
        if H is not None:
            raise NotImplementedError("QG needs H constant in space; a per-call H perturbation is not supported")
        if h_wind is not None:
            raise NotImplementedError("h_wind: the QG wind forcing divides by the top layer's H (qg.py:190-193)")
        p = self.param
        kw = self._plan_kwargs()
        kw.pop("rho_water")
        kw.pop("h_wind")
        # the barotropic filter is SW's only (sw.py:307-309); open boundaries
        # would also have to open the projector's face masks, not built
        for k in ("barotropic_filter", "bf_lambd"):
            kw.pop(k)
        if kw.pop("flag_obc"):
            raise NotImplementedError("open boundaries in the QG model (the projector's masks)")
        H = np.asarray(self.H)
        if H.shape[-2:] != (1, 1):
            raise ValueError(f"H must be constant in space for the qg approximation, got shape {H.shape}")
        return QGPlan(self.nx, self.ny, self.nl, p["dx"], p["dy"], p["f"], H, p["g_prime"], p["dt"], **kw)

    def __init__(self, param):
        super().__init__(param)
        q = self._base
        self.A = q.A
        self.lambd = q.lambd.reshape(1, self.nl, 1, 1)
        self.Cl2m, self.Cm2l = q.Cl2m, q.Cm2l
        self.cap_matrices = q.cap if q.cmm else None
        self.homsol_wgrid = q.homsol[None]
        self.homsol_wgrid_mean = q.hmean.reshape(1, self.nl, 1, 1)
        nx, ny = self.nx, self.ny
        x, y = np.meshgrid(np.arange(1, nx), np.arange(1, ny), indexing="ij")
        lap = (2 * (np.cos(np.pi / nx * x) - 1) / q.dx ** 2 + 2 * (np.cos(np.pi / ny * y) - 1) / q.dy ** 2)
        self.helmholtz_dstI = lap[None, None] - q.f0 ** 2 * self.lambd

    def project_qg(self, u, v, h):
        """P = G o (Q o G)^-1 o Q (qg.py:310-312) of model-space fields."""
        sw = self._swplan()
        x = [self._in(a) for a in (u, v, h)]
        r = self._base.project(*sw._uvh(*x, sw._batch(x[0])))
        return tuple(self._out(u, a) for a in r)

    def compute_time_derivatives(self, u, v, h, ref_vals=None, taux=None, tauy=None, h_wind=None):
        """qg.py:335-345: projected shallow-water tendencies."""
        if ref_vals is not None:
            raise NotImplementedError("ref_vals")
        if h_wind is not None:
            raise NotImplementedError("h_wind: the QG wind forcing divides by the top layer's H (qg.py:190-193)")
        r = self._base.rhs(self._in(u), self._in(v), self._in(h), *self._tau(taux, tauy))
        return tuple(self._out(u, a) for a in r)
