"""Multilayer quasi-geostrophic model as projected shallow water
(mapping/models/model_qgsw/qg.py ``QG``) on the GPU.

Every right-hand side is the shallow-water tendency (vd_sw_*) projected by
P = G o (Q o G)^-1 o Q (qg.py:310-345): Q and G are the vd_qgp kernels, the
inversion solves one Helmholtz problem per vertical mode with the spectral
solvers of :mod:`vardyn_gb300.helmholtz_dst` (capacitance-matrix method when
the psi mask has irregular boundary points), followed by the homogeneous
correction. P is linear, so the tangent linear projects the tangent
tendency and the adjoint applies P^T = Q^T (Q o G)^-T G^T: the DST solve is
symmetric, edge padding and the capacitance correction are transposed
explicitly.

``inversion="multigrid"`` replaces the DST + capacitance inversion by a
masked Dirichlet multigrid (vd_mgd_*) solving the same discrete problem per
mode: on domains with many irregular boundary points (20 % land) the
capacitance set-up, one DST solve per point and an M x M inverse, is out of
reach.

Deviations needed to run at all (``QG.step`` fails in the reference as
shipped, see oracle/qg_ml.py): the SW step passes its reference values and
wind arguments through QG's overrides, and QG's wind term
``taux / H[0] * dx`` acts on the interior u / v faces.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .helmholtz_dst import HelmholtzDST
from .helmholtz_mg import MaskedDirichletMG
from .qg1l import _ptr, _stream
from .sw import SWPlan


def layer_matrix(H, g_prime):
    """A operator (qg.py:47-59)."""
    H, gp = np.asarray(H, float).ravel(), np.asarray(g_prime, float).ravel()
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


def mode_matrices(A):
    """Eigen-decomposition into layer-to-mode / mode-to-layer matrices
    (qg.py:62-70), on the host in float64 (set-up)."""
    lr, R = np.linalg.eig(A)
    _, L = np.linalg.eig(A.T)
    R, L = R.real, L.real
    return lr.real, np.diag(1. / np.diag(L.T @ R)) @ L.T, R


def _scalar_metric(a, name):
    a = np.asarray(a, dtype=np.float64)
    if a.size > 1 and not np.all(a == a.ravel()[0]):
        raise ValueError(f"the QG operators need a uniform {name} (qg.py:198-308 use it as a scalar)")
    return float(a.ravel()[0])


class QGPlan:
    """QG(param) of qg.py; arguments as :class:`vardyn_gb300.sw.SWPlan`,
    with H constant in space and uniform dx, dy."""

    def __init__(self, nx, ny, nl, dx, dy, f, H, g_prime, dt, mask=None, slip_coef=1.0, bottom_drag_coef=0.0,
                 h_min=0.1, h_min_sharpness=10.0, visc_coef=0.0, diff_coef=0.0, sponge_coef=0.0, flag_linear=False,
                 forcing_momentum="direct", taux=0.0, tauy=0.0, sponge_u=None, sponge_v=None, sponge_h=None,
                 dtype=torch.float64, device=None, inversion="spectral", mg_tol=1e-8, mg_max_cycles=24,
                 mg_dtype=None):
        self.nx, self.ny, self.nl = int(nx), int(ny), int(nl)
        nx, ny, nl = self.nx, self.ny, self.nl
        Hc = np.asarray(H, dtype=np.float64)
        if Hc.size != nl:
            raise ValueError("H must be constant in space for the QG approximation (shape (nl, 1, 1))")
        self.Hc = Hc.reshape(nl)
        self.dx, self.dy = _scalar_metric(dx, "dx"), _scalar_metric(dy, "dy")
        self.dtype = dtype
        fa = np.asarray(f, dtype=np.float64)
        self.f0 = float(fa.mean())
        # QG's wind term taux / H[0] * dx: the SW wind with rho = 1, depth H[0]
        self.sw = SWPlan(nx, ny, nl, self.dx, self.dy, fa, self.Hc, g_prime, dt, mask=mask, slip_coef=slip_coef,
                         bottom_drag_coef=bottom_drag_coef, rho_water=1.0, h_min=h_min,
                         h_min_sharpness=h_min_sharpness, visc_coef=visc_coef, diff_coef=diff_coef,
                         sponge_coef=sponge_coef, flag_linear=flag_linear, forcing_momentum=forcing_momentum,
                         h_wind=float(self.Hc[0]), taux=taux, tauy=tauy, sponge_u=sponge_u, sponge_v=sponge_v,
                         sponge_h=sponge_h, dtype=dtype, device=device)
        self.device = self.sw.device
        self.masks = self.sw.masks
        self.A = layer_matrix(self.Hc, g_prime)
        self.lambd, self.Cl2m, self.Cm2l = mode_matrices(self.A)
        self.helm = HelmholtzDST(nx, ny, self.dx, self.dy, self.f0 ** 2 * self.lambd, dtype=dtype,
                                 device=self.device)
        m = self.masks
        if inversion not in ("spectral", "multigrid"):
            raise ValueError("inversion is 'spectral' (DST + capacitance matrices, the reference's) or 'multigrid'")
        self.inversion = inversion
        self.masked = m.psi_irrbound_xids.size > 0
        # the capacitance branch only for the spectral inversion; the
        # multigrid solves the masked Dirichlet problem directly
        self.cmm = self.masked and inversion == "spectral"
        self.mg = None
        if inversion == "multigrid":
            self.mg = MaskedDirichletMG(nx - 1, ny - 1, self.dx, self.dy, self.f0 ** 2 * self.lambd,
                                        mask=np.asarray(m.psi, dtype=np.float64)[1:-1, 1:-1],
                                        dtype=dtype if mg_dtype is None else mg_dtype, tol=mg_tol,
                                        max_cycles=mg_max_cycles, device=self.device)
        self._dt = _lib.VD_F64 if dtype == torch.float64 else _lib.VD_F32
        X, Y = nx + 1, ny + 1
        self.psi = torch.as_tensor(m.psi, dtype=dtype, device=self.device).contiguous()
        if self.cmm:
            self.cap = self.helm.capacitance_matrices(m.psi_irrbound_xids, m.psi_irrbound_yids).contiguous()
            self.capT = self.cap.transpose(1, 2).contiguous()
            self.bidx = self.helm._bidx(m.psi_irrbound_xids, m.psi_irrbound_yids)
        # C plan of the Q / G / mixing kernels
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (self.Hc, self.A, self.Cl2m, self.Cm2l)]
        mk = None if mask is None else np.ascontiguousarray(np.asarray(mask, dtype=np.float64))
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d = _lib.VdQgpDesc()
        d.nx, d.ny, d.nl, d.dtype = nx, ny, nl, self._dt
        d.dx, d.dy, d.f0 = self.dx, self.dy, self.f0
        d.H_host, d.A_host, d.Cl2m_host, d.Cm2l_host = (dp(a) for a in keep)
        d.mask_host = None if mk is None else dp(mk)
        d.cmm = 1 if self.masked else 0          # Q masks the modal rhs on land
        h = ctypes.c_void_p()
        _lib.call("vd_qgp_plan_create", ctypes.byref(h), ctypes.byref(d))
        self._q = h
        self._lib = _lib.load()
        # homogeneous solutions (qg.py:87-98)
        q = torch.zeros((nl, 1, X, Y), dtype=dtype, device=self.device)
        q[..., 1:-1, 1:-1] = self.psi[1:-1, 1:-1] if self.masked else 1.0
        sol = self._solve(q)[:, 0]
        shift = torch.as_tensor(self.f0 ** 2 * self.lambd, dtype=dtype, device=self.device).reshape(nl, 1, 1)
        self.homsol = (1.0 + sol * shift).contiguous()
        self.hmean = self.homsol.double().mean((-1, -2)).contiguous()

    def __del__(self):
        h = getattr(self, "_q", None)
        if h is not None and h.value:
            try:
                self._lib.vd_qgp_plan_destroy(h)
            except Exception:
                pass
            self._q = None

    # ---------------- projector pieces ----------------
    def _op(self, op, B, *args):
        arr = (ctypes.c_void_p * len(args))(*[None if a is None else a.data_ptr() for a in args])
        _lib.call("vd_qgp_op", self._q, op, B, arr, _stream())

    def _S(self, q):
        out = torch.empty_like(q)
        self.helm._solve_modes(q, out)
        return out

    def _mg_interior(self, src, dst):
        """dst interior = multigrid solve of src interior ([nl][B][X][Y], in
        place on the padded fields: system m*B + b)."""
        X, Y = self.nx + 1, self.ny + 1
        if self.mg.dtype != src.dtype:
            # float32 model, float64 inversion (a 1e-8 relative residual is
            # below float32 resolution)
            s64, d64 = src.to(self.mg.dtype), torch.zeros(dst.shape, dtype=self.mg.dtype, device=dst.device)
            self.mg.solve_strided(src.shape[1], s64[:, :, 1:, 1:], Y, X * Y, d64[:, :, 1:, 1:], Y, X * Y)
            return dst.copy_(d64)
        self.mg.solve_strided(src.shape[1], src[:, :, 1:, 1:], Y, X * Y, dst[:, :, 1:, 1:], Y, X * Y)
        return dst

    def _solve(self, q):
        """Modal solutions of QoG_inv (qg.py:272-280), [nl][B][nx+1][ny+1]
        edge-padded (times psi in the capacitance branch and, on a masked
        domain, in the multigrid branch)."""
        nl, B = q.shape[0], q.shape[1]
        if self.inversion == "multigrid":
            s = self._mg_interior(q, torch.zeros_like(q))
            out = torch.empty_like(s)
            self.helm._edge_pad(s, out, self.psi if self.masked else None)
            return out
        s = self._S(q)
        if not self.cmm:
            self.helm._edge_pad(s, s)
            return s
        fs = (self.nx + 1) * (self.ny + 1)
        q2 = torch.empty_like(q)
        _lib.call("vd_cmm_correct", self._dt, nl, B, self.bidx.numel(), fs, _ptr(self.cap), _ptr(self.bidx),
                  _ptr(s), _ptr(q), _ptr(q2), _stream())
        s2 = self._S(q2)
        out = torch.empty_like(s2)
        self.helm._edge_pad(s2, out, self.psi)
        return out

    def _solve_adj(self, ad):
        nl, B = ad.shape[0], ad.shape[1]
        X, Y = self.nx + 1, self.ny + 1
        g0 = torch.empty_like(ad)
        _lib.call("vd_edge_pad_adj", self._dt, nl * B, X, Y, _ptr(ad), _ptr(self.psi if self.masked else None),
                  _ptr(g0), _stream())
        if self.inversion == "multigrid":
            # the masked Dirichlet operator is symmetric: its inverse is its
            # own transpose (to the solve's tolerance)
            return self._mg_interior(g0, torch.zeros_like(g0))
        g = self._S(g0)
        if not self.cmm:
            return g
        z = torch.zeros_like(g)
        _lib.call("vd_cmm_correct", self._dt, nl, B, self.bidx.numel(), X * Y, _ptr(self.capT), _ptr(self.bidx),
                  _ptr(g), _ptr(z), _ptr(z), _stream())
        return g.add_(self._S(z))

    def project(self, u, v, h):
        """project_qg (qg.py:310-312) of model-space fields [B][nl][..]."""
        B = u.shape[0]
        nl, X, Y = self.nl, self.nx + 1, self.ny + 1
        modes = torch.empty((nl, B, X, Y), dtype=self.dtype, device=self.device)
        self._op(0, B, u, v, h, modes)
        pm = self._solve(modes)
        sums = torch.empty(nl * B * 65, dtype=torch.float64, device=self.device)
        self._op(2, B, pm, None, sums)
        pqg = torch.empty((B, nl, X, Y), dtype=self.dtype, device=self.device)
        self._op(3, B, pm, sums, self.hmean, self.homsol, pqg)
        Pu, Pv, Ph = torch.empty_like(u), torch.empty_like(v), torch.empty_like(h)
        self._op(6, B, pqg, Pu, Pv, Ph)
        return Pu, Pv, Ph

    def project_adj(self, au, av, ah):
        B = au.shape[0]
        nl, X, Y = self.nl, self.nx + 1, self.ny + 1
        apqg = torch.empty((B, nl, X, Y), dtype=self.dtype, device=self.device)
        self._op(7, B, au.contiguous(), av.contiguous(), ah.contiguous(), apqg)
        apm = torch.empty((nl, B, X, Y), dtype=self.dtype, device=self.device)
        self._op(4, B, apqg, apm)
        sums = torch.empty(nl * B * 65, dtype=torch.float64, device=self.device)
        self._op(2, B, apm, self.homsol, sums)
        self._op(5, B, sums, self.hmean, apm)
        aq = self._solve_adj(apm)
        adu, adv, adh = torch.empty_like(au), torch.empty_like(av), torch.empty_like(ah)
        self._op(1, B, aq, adu, adv, adh)
        return adu, adv, adh

    # ---------------- model ----------------
    def rhs(self, u, v, h, taux=None, tauy=None):
        """compute_time_derivatives (qg.py:335-345) of model-space fields."""
        return self.project(*self.sw.rhs(u, v, h, taux, tauy))

    def _prep(self, u0, v0, h0, ub, vb, hb, Fu, Fv, Fh):
        sw = self.sw
        B = sw._batch(u0)
        x0 = sw._uvh(u0, v0, h0, B)
        x = tuple(torch.empty_like(a) for a in x0)
        sw.scale(B, False, x0, x)
        bsrc = sw._uvh(ub, vb, hb, B, "b_") if ub is not None else x0
        xb = tuple(torch.empty_like(a) for a in x0)
        sw.scale(B, False, bsrc, xb)
        F = None
        Fp = sw._fill_forcing(Fu, Fv, Fh, B)
        if Fp[0] is not None:
            F = tuple(torch.empty_like(a) for a in x0)
            sw.scale(B, False, Fp, F)
        return B, x, xb, F

    def _stages(self, B, x, xb, F, tau, store=None):
        """One RK3-SSP step in place on x; returns the stage states."""
        sw = self.sw
        mc = sw.forcing_momentum == "mass_consistent"
        new = lambda: tuple(torch.empty_like(a) for a in x)
        x1, x2, k0, k1 = new(), new(), new(), new()
        x3 = new() if mc else x
        cur = x
        stages = [tuple(a.clone() for a in x)]
        for stg in range(3):
            r = self.rhs(*cur, *tau)
            nxt = (x1, x2, x3)[stg]
            sw.stage(B, stg, cur, r, k0 if stg > 0 else None, k1 if stg > 1 else None, xb,
                     F if (stg == 2 and not mc) else None, (k0, k1, None)[stg], nxt)
            cur = nxt
            if stg < 2:
                stages.append(nxt)
        if mc:
            Fz = F if F is not None else tuple(torch.zeros_like(a) for a in x)
            stages.append(tuple(a.clone() for a in x3))
            sw.force_mc(B, x3, Fz, x)
        return stages

    def step(self, u0, v0, h0, nstep=1, ub=None, vb=None, hb=None, Fu=None, Fv=None, Fh=None, taux=None,
             tauy=None):
        B, x, xb, F = self._prep(u0, v0, h0, ub, vb, hb, Fu, Fv, Fh)
        tau = self.sw._tau(taux, tauy)
        for _ in range(int(nstep)):
            self._stages(B, x, xb, F, tau)
        out = tuple(torch.empty_like(a) for a in x)
        self.sw.scale(B, True, x, out)
        return out

    def step_tgl(self, u0, v0, h0, du0, dv0, dh0, nstep=1, ub=None, vb=None, hb=None, dub=None, dvb=None, dhb=None,
                 Fu=None, Fv=None, Fh=None, dFu=None, dFv=None, dFh=None, taux=None, tauy=None):
        sw = self.sw
        if sw.forcing_momentum == "mass_consistent":
            raise NotImplementedError("tangent linear of the QG model with mass-consistent forcing")
        B, x, xb, F = self._prep(u0, v0, h0, ub, vb, hb, Fu, Fv, Fh)
        _, dx, dxb, dF = self._prep(du0, dv0, dh0, dub if ub is not None else None, dvb, dhb, dFu, dFv, dFh)
        if ub is not None and dub is None:
            dxb = tuple(torch.zeros_like(a) for a in dx)
        tau = sw._tau(taux, tauy)
        if F is not None and dF is None:
            dF = tuple(torch.zeros_like(a) for a in dx)
        if dF is not None and F is None:
            F = tuple(torch.zeros_like(a) for a in x)
        new = lambda: tuple(torch.empty_like(a) for a in x)
        for _ in range(int(nstep)):
            x1, x2, k0, k1 = new(), new(), new(), new()
            d1, d2, dk0, dk1 = new(), new(), new(), new()
            cur, dcur = x, dx
            for stg in range(3):
                r, dr = sw.rhs_tgl(*cur, *dcur, *tau)
                r, dr = self.project(*r), self.project(*dr)
                nxt, dnxt = (x1, x2, x)[stg], (d1, d2, dx)[stg]
                sw.stage(B, stg, cur, r, k0 if stg > 0 else None, k1 if stg > 1 else None, xb,
                         F if stg == 2 else None, (k0, k1, None)[stg], nxt)
                sw.stage(B, stg, dcur, dr, dk0 if stg > 0 else None, dk1 if stg > 1 else None, dxb,
                         dF if stg == 2 else None, (dk0, dk1, None)[stg], dnxt)
                cur, dcur = nxt, dnxt
        out = tuple(torch.empty_like(a) for a in dx)
        sw.scale(B, True, dx, out)
        return out

    def step_adj(self, u0, v0, h0, adu1, adv1, adh1, nstep=1, ub=None, vb=None, hb=None, Fu=None, Fv=None, Fh=None,
                 taux=None, tauy=None, want_bc=False, want_forcing=False):
        sw = self.sw
        mc = sw.forcing_momentum == "mass_consistent"
        B, x, xb, F = self._prep(u0, v0, h0, ub, vb, hb, Fu, Fv, Fh)
        tau = sw._tau(taux, tauy)
        traj = []
        for _ in range(int(nstep)):
            traj.append(tuple(a.clone() for a in x))
            self._stages(B, x, xb, F, tau)
        ad = tuple(torch.empty_like(a) for a in x)
        sw.scale(B, True, sw._uvh(adu1, adv1, adh1, B, "ad"), ad)
        zeros = lambda: tuple(torch.zeros_like(a) for a in x)
        adb, adF = zeros(), zeros()
        adk = tuple(torch.empty_like(a) for a in x)
        Fz = F if F is not None else zeros()
        for n in range(int(nstep) - 1, -1, -1):
            xs = tuple(a.clone() for a in traj[n])
            stages = self._stages(B, xs, xb, F, tau)
            for a, b in zip(adF, ad):
                a.add_(b, alpha=sw.dt)
            if mc:
                sw.force_mc_adj(B, stages[3], Fz[2], ad, adF[2])
            a0, a1 = zeros(), zeros()
            for stg in (2, 1, 0):
                sw.stage_adj(B, stg, ad, adk, a0, a1, adb)
                ar = self.project_adj(*adk)
                sw.rhs_adj(*stages[stg], *ar, ad)
        if ub is None:
            for a, b in zip(ad, adb):
                a.add_(b)
        out = {}
        res = tuple(torch.empty_like(a) for a in ad)
        sw.scale(B, False, ad, res)
        out["u0"], out["v0"], out["h0"] = res
        if want_bc and ub is not None:
            r2 = tuple(torch.empty_like(a) for a in ad)
            sw.scale(B, False, adb, r2)
            out["ub"], out["vb"], out["hb"] = r2
        if want_forcing:
            r3 = tuple(torch.empty_like(a) for a in ad)
            sw.scale(B, False, adF, r3)
            out["Fu"], out["Fv"], out["Fh"] = r3
        return out

