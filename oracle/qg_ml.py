"""Oracle (test infrastructure only): float64 NumPy restatement of the
multilayer QG model of mapping/models/model_qgsw/qg.py (QG as projected SW).

  compute_auxillary_matrices   qg.py:45-98 (A, modes, Helmholtz, homsol)
  G                            qg.py:198-219
  QoG_inv (no background)      qg.py:222-298
  Q                            qg.py:300-308
  project_qg                   qg.py:310-312
  compute_time_derivatives     qg.py:335-345

The projector is pinned against outputs of the reference's own qg.py
(tests/golden/gen_golden_sw.py). ``QG.step`` cannot run in the reference as
shipped (SW.step passes ref_vals / wind arguments that QG's overrides do not
accept); the step here is SW.step with the projected tendencies and those
arguments passed through, QG's wind term ``taux / H[0] * dx`` on the
interior u faces: parity of the step is unpinned by reference outputs.
"""
import numpy as np

from oracle.helmholtz_dst import (compute_capacitance_matrices, compute_laplace_dstI, solve_helmholtz_dstI,
                                  solve_helmholtz_dstI_cmm)
from oracle.sw import SWOracle, interp_TP


def layer_matrix(H, gp):
    """A operator (qg.py:47-59)."""
    H, gp = np.asarray(H, float).ravel(), np.asarray(gp, float).ravel()
    nl = H.size
    A = np.zeros((nl, nl))
    if nl == 1:
        A[0, 0] = 1. / (H[0] * gp[0])
        return A
    A[0, 0] = 1. / (H[0] * gp[0]) + 1. / (H[0] * gp[1])
    A[0, 1] = -1. / (H[0] * gp[1])
    for i in range(1, nl - 1):
        A[i, i - 1] = -1. / (H[i] * gp[i])
        A[i, i] = 1. / H[i] * (1 / gp[i + 1] + 1 / gp[i])
        A[i, i + 1] = -1. / (H[i] * gp[i + 1])
    A[-1, -1] = 1. / (H[nl - 1] * gp[nl - 1])
    A[-1, -2] = -1. / (H[nl - 1] * gp[nl - 1])
    return A


def modes(A):
    """Layer/mode matrices (qg.py:62-70)."""
    lr, R = np.linalg.eig(A)
    ll, L = np.linalg.eig(A.T)
    R, L = R.real, L.real
    Cl2m = np.diag(1. / np.diag(L.T @ R)) @ L.T
    return lr.real, Cl2m, R


class QGOracle(SWOracle):
    def __init__(self, param):
        super().__init__(param)
        self.dxs = float(np.asarray(param["dx"]).ravel()[0])
        self.dys = float(np.asarray(param["dy"]).ravel()[0])
        self.Hc = np.asarray(param["H"], float).reshape(-1)
        nl, nx, ny = self.nl, self.nx, self.ny
        self.A = layer_matrix(self.Hc, self.gp)
        lam, self.Cl2m, self.Cm2l = modes(self.A)
        self.lambd = lam
        self.helm = (compute_laplace_dstI(nx, ny, self.dxs, self.dys)[None]
                     - self.f0 ** 2 * lam.reshape(nl, 1, 1))
        m = self.masks
        self.cmm = m.irr_x.size > 0
        cst = np.ones((nl, nx + 1, ny + 1))
        if self.cmm:
            self.cap = compute_capacitance_matrices(self.helm[None], m.irr_x, m.irr_y)
            sol = solve_helmholtz_dstI_cmm((cst * m.psi)[..., 1:-1, 1:-1], self.helm, self.cap, m.irr_x, m.irr_y,
                                           m.psi)
        else:
            sol = solve_helmholtz_dstI(cst[..., 1:-1, 1:-1], self.helm)
        self.homsol = cst + sol * self.f0 ** 2 * lam.reshape(nl, 1, 1)
        self.homsol_mean = self.homsol.mean((-1, -2), keepdims=True)
        self.area_s = self.dxs * self.dys

    def G(self, p):
        m = self.masks
        dx, dy, f0 = self.dxs, self.dys, self.f0
        p_i = interp_TP(p)
        u = -np.diff(p, axis=-1) / dy / f0 * dx * m.u
        v = np.diff(p, axis=-2) / dx / f0 * dy * m.v
        u = np.where(np.isnan(u), 0, u)
        v = np.where(np.isnan(v), 0, v)
        u[..., :, 0] = 0
        v[..., 0, :] = 0
        h = self.Hc.reshape(-1, 1, 1) * np.einsum("lm,...mxy->...lxy", self.A, p_i) * self.area_s * m.h
        return u, v, np.where(np.isnan(h), 0, h)

    def Q(self, u, v, h):
        om = np.diff(v[..., 1:-1], axis=-2) - np.diff(u[..., 1:-1, :], axis=-1)
        return (om - self.f0 * interp_TP(h) / self.Hc.reshape(-1, 1, 1)) * (self.f0 / self.area_s)

    def QoG_inv(self, rhs):
        m = self.masks
        hr = np.einsum("lm,...mxy->...lxy", self.Cl2m, rhs)
        if self.cmm:
            pm = solve_helmholtz_dstI_cmm(hr * m.psi[1:-1, 1:-1], self.helm, self.cap, m.irr_x, m.irr_y, m.psi)
        else:
            pm = solve_helmholtz_dstI(hr, self.helm)
        alpha = -pm.mean((-1, -2), keepdims=True) / self.homsol_mean
        pm = pm + alpha * self.homsol
        p = np.einsum("lm,...mxy->...lxy", self.Cm2l, pm)
        return p, interp_TP(p)

    def project(self, u, v, h):
        return self.G(self.QoG_inv(self.Q(u, v, h))[0])

    def wind(self, refv, taux, tauy):
        """QG.add_wind_forcing (qg.py:190-193) on the interior faces."""
        H0 = self.Hc[0]
        return (np.where(self.masks.u[1:-1, :] > 0.5, taux / H0 * self.dx_u[1:-1, :], 0.0),
                np.where(self.masks.v[:, 1:-1] > 0.5, tauy / H0 * self.dy_v[:, 1:-1], 0.0))

    def rhs(self, u, v, h, refv, taux, tauy):
        return self.project(*super().rhs(u, v, h, refv, taux, tauy))
