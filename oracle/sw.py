"""Oracle (test infrastructure only): float64 NumPy restatement of the
multilayer rotating shallow-water model of mapping/models/model_qgsw/sw.py
and its helpers.

  masks                    masks.py:57-158 (avg_pool2d: tools.py:9-67)
  reconstructions          reconstruction.py:17-169 (WENO_EPS = 1e-4)
  flux                     flux.py:39-90
  interp_TP, comp_ke, div  finite_diff.py:6-52
  smooth_clamp             sw.py:27-33
  reference values         sw.py:385-418
  omega                    sw.py:678-696
  diagnostics              sw.py:698-718
  advection_h              sw.py:468-481
  advection_momentum       sw.py:483-511
  diffusion (u, v / h)     sw.py:513-568
  wind / bottom drag       sw.py:570-669
  RK3-SSP step, sponge,
  forcing                  sw.py:752-904

Arrays follow the reference's layout: [n_ens, nl, x, y] with u on
(nx+1, ny), v on (nx, ny+1), h on (nx, ny), vorticity on (nx+1, ny+1).
Pinned against outputs of the reference's own sw.py (tests/golden/
gen_golden_sw.py).
"""
import numpy as np

WENO_EPS = 1e-4


# ---------------------------------------------------------------- masks
def _pool_sum(x, kx, ky, px, py):
    """Window sums of a 2-D array over kx x ky windows, zero padding px/py."""
    xp = np.pad(x, ((px, px), (py, py)))
    nxo, nyo = xp.shape[0] - kx + 1, xp.shape[1] - ky + 1
    out = np.zeros((nxo, nyo))
    for a in range(kx):
        for b in range(ky):
            out += xp[a:a + nxo, b:b + nyo]
    return out


class SWMasks:
    """Staggered masks and WENO stencil-width selectors (masks.py:57-158).
    Window averages are compared through their integer sums."""

    def __init__(self, mask_h):
        h = np.asarray(mask_h, dtype=np.float64)
        self.h = h
        self.u = (_pool_sum(h, 2, 1, 1, 0) == 2).astype(float)
        self.v = (_pool_sum(h, 1, 2, 0, 1) == 2).astype(float)
        w4 = _pool_sum(h, 2, 2, 1, 1)
        self.w = (w4 >= 1).astype(float)
        self.psi = (w4 == 4).astype(float)
        n_v = _pool_sum(self.v, 2, 1, 1, 0) == 1
        n_u = _pool_sum(self.u, 1, 2, 0, 1) == 1
        w = self.w > 0
        self.w_vertical_bound = (w & n_v & ~n_u).astype(float)
        self.w_horizontal_bound = (w & n_u & ~n_v).astype(float)
        self.w_cornerout_bound = (w & n_u & n_v).astype(float)
        self.w_valid = (w & ~(n_v & ~n_u) & ~(n_u & ~n_v) & ~(n_u & n_v)).astype(float)
        nb = _pool_sum(self.psi, 3, 3, 0, 0)
        self.irr_x, self.irr_y = np.where((self.psi[1:-1, 1:-1] == 0) & (nb > 0))
        u, v = self.u > 0, self.v > 0
        # h stencils along x on the u grid
        eq2 = (_pool_sum(h, 2, 1, 1, 0) == 2) & (_pool_sum(h, 4, 1, 2, 0) < 4) & u
        gt4 = ~eq2 & u
        eq4 = (_pool_sum(h, 6, 1, 3, 0) < 6) & gt4
        self.u_hx = (eq2, eq4, ~eq4 & gt4)
        # vorticity stencils along y on the u grid; the reference passes
        # u_sten_wy_gt4 (not gt6) as its 6-point mask (sw.py:296-305)
        eq2 = (_pool_sum(self.w, 1, 2, 0, 0) == 2) & (_pool_sum(self.w, 1, 4, 0, 1) < 4) & u
        gt4 = ~eq2 & u
        eq4 = (_pool_sum(self.w, 1, 6, 0, 2) < 6) & gt4
        self.u_wy = (eq2, eq4, gt4)
        self.u_wy_gt6 = ~eq4 & gt4
        # h stencils along y on the v grid
        eq2 = (_pool_sum(h, 1, 2, 0, 1) == 2) & (_pool_sum(h, 1, 4, 0, 2) < 4) & v
        gt4 = ~eq2 & v
        eq4 = (_pool_sum(h, 1, 6, 0, 3) < 6) & gt4
        self.v_hy = (eq2, eq4, ~eq4 & gt4)
        # vorticity stencils along x on the v grid
        eq2 = (_pool_sum(self.w, 2, 1, 0, 0) == 2) & (_pool_sum(self.w, 4, 1, 1, 0) < 4) & v
        gt4 = ~eq2 & v
        eq4 = (_pool_sum(self.w, 6, 1, 2, 0) < 6) & gt4
        self.v_wx = (eq2, eq4, ~eq4 & gt4)


# ---------------------------------------------------------------- reconstructions
def smooth_abs(x):
    return np.sqrt(x * x + WENO_EPS ** 2)


def wenoz4(qmm, qm, qp, qpp):
    q1 = -0.5 * qmm + 1.5 * qm
    q2 = 0.5 * (qm + qp)
    b1, b2 = (qm - qmm) ** 2, (qp - qm) ** 2
    tau = smooth_abs(b2 - b1)
    w1 = (1. / 3.) * (1. + tau / (b1 + WENO_EPS))
    w2 = (2. / 3.) * (1. + tau / (b2 + WENO_EPS))
    return (w1 * q1 + w2 * q2) / (w1 + w2)


def wenoz6(q0, q1, q2, q3, q4, q5):
    r1 = 1. / 3. * q0 - 7. / 6. * q1 + 11. / 6. * q2
    r2 = -1. / 6. * q1 + 5. / 6. * q2 + 1. / 3. * q3
    r3 = 1. / 3. * q2 + 5. / 6. * q3 - 1. / 6. * q4
    k1, k2 = 13. / 12., 0.25
    b1 = k1 * (q0 - 2 * q1 + q2) ** 2 + k2 * (q0 - 4 * q1 + 3 * q2) ** 2
    b2 = k1 * (q1 - 2 * q2 + q3) ** 2 + k2 * (q1 - q3) ** 2
    b3 = k1 * (q2 - 2 * q3 + q4) ** 2 + k2 * (3 * q2 - 4 * q3 + q4) ** 2
    tau = smooth_abs(b1 - b3)
    w1 = 0.1 * (1 + tau / (b1 + WENO_EPS))
    w2 = 0.6 * (1 + tau / (b2 + WENO_EPS))
    w3 = 0.3 * (1 + tau / (b3 + WENO_EPS))
    return (w1 * r1 + w2 * r2 + w3 * r3) / (w1 + w2 + w3)


def weno_flux(q, vel, axis, m2, m4, m6):
    """Upwind-biased flux of q across the interior faces along ``axis``
    (length n-1) with 2/4/6-point reconstructions selected by masks;
    the 4- and 6-point values are 0 within 1 / 2 faces of the ends."""
    q = np.moveaxis(q, axis, -1)
    vel, m2, m4, m6 = (np.moveaxis(np.broadcast_to(a, vel.shape), axis, -1) for a in (vel, m2, m4, m6))
    n = q.shape[-1]
    s = [q[..., k:n - 5 + k] for k in range(6)]
    pos2 = 0.5 * (q[..., :-1] + q[..., 1:])
    pos4 = np.zeros_like(pos2)
    neg4 = np.zeros_like(pos2)
    pos6 = np.zeros_like(pos2)
    neg6 = np.zeros_like(pos2)
    t = [q[..., k:n - 3 + k] for k in range(4)]
    pos4[..., 1:-1] = wenoz4(t[0], t[1], t[2], t[3])
    neg4[..., 1:-1] = wenoz4(t[3], t[2], t[1], t[0])
    pos6[..., 2:-2] = wenoz6(*s)
    neg6[..., 2:-2] = wenoz6(*s[::-1])
    up = np.maximum(vel, 0)
    un = vel - up
    out = up * (m2 * pos2 + m4 * pos4 + m6 * pos6) + un * (m2 * pos2 + m4 * neg4 + m6 * neg6)
    return np.moveaxis(out, -1, axis)


def smooth_clamp(x, xmin, sharp):
    return xmin + np.logaddexp((x - xmin) * sharp, 0.0) / sharp


def interp_TP(f):
    return 0.25 * (f[..., 1:, 1:] + f[..., 1:, :-1] + f[..., :-1, 1:] + f[..., :-1, :-1])


def div_noflux(fx, fy):
    """Divergence with the reference's edge-padded fluxes (finite_diff.py:
    44-52): the first and last cells along each axis get no contribution."""
    dx = np.zeros(fx.shape[:-2] + (fx.shape[-2] + 1, fx.shape[-1]))
    dx[..., 1:-1, :] = np.diff(fx, axis=-2)
    dy = np.zeros(fy.shape[:-1] + (fy.shape[-1] + 1,))
    dy[..., 1:-1] = np.diff(fy, axis=-1)
    return dx + dy


def _edge_avg(a, axis):
    """0.5 * (neighbours) of an edge-padded array: n -> n+1 along axis."""
    pad = [(0, 0)] * a.ndim
    pad[axis] = (1, 1)
    p = np.pad(a, pad, mode="edge")
    sl0 = [slice(None)] * a.ndim
    sl1 = [slice(None)] * a.ndim
    sl0[axis] = slice(1, None)
    sl1[axis] = slice(None, -1)
    return 0.5 * (p[tuple(sl0)] + p[tuple(sl1)])


# ---------------------------------------------------------------- model
class SWOracle:
    """SW(param) restated; ``param`` takes the reference's keys."""

    def __init__(self, param):
        self.nx, self.ny, self.nl = param["nx"], param["ny"], param["nl"]
        nx, ny = self.nx, self.ny
        self.dx = np.asarray(param["dx"], dtype=np.float64)
        self.dy = np.asarray(param["dy"], dtype=np.float64)
        assert self.dx.shape == (nx, ny) and self.dy.shape == (nx, ny)
        self.dx_u, self.dy_u = _edge_avg(self.dx, 0), _edge_avg(self.dy, 0)
        self.dx_v, self.dy_v = _edge_avg(self.dx, 1), _edge_avg(self.dy, 1)
        self.area = self.dx * self.dy
        self.area_u, self.area_v = self.dx_u * self.dy_u, self.dx_v * self.dy_v
        self.slip = float(param.get("slip_coef", 1.0))
        self.masks = SWMasks(param["mask"] if "mask" in param else np.ones((nx, ny)))
        # open boundaries (sw.py:353-371): the u masks of the west / east
        # faces and the v masks of the south / north faces are set to 1 after
        # the other masks are built; the boundary arrays allocated there are
        # never read
        if param.get("flag_obc", False):
            self.masks.u = self.masks.u.copy()
            self.masks.u[0, :] = 1.0
            self.masks.u[-1, :] = 1.0
            self.masks.v = self.masks.v.copy()
            self.masks.v[:, 0] = 1.0
            self.masks.v[:, -1] = 1.0
        f = np.asarray(param["f"], dtype=np.float64)
        self.f0 = f.mean()
        self.fstar_u = 0.5 * (f[:, 1:] + f[:, :-1]) * self.area_u
        self.fstar_v = 0.5 * (f[1:, :] + f[:-1, :]) * self.area_v
        self.gp = np.asarray(param["g_prime"], dtype=np.float64).reshape(-1, 1, 1)
        self.taux, self.tauy = param["taux"], param["tauy"]
        self.drag = float(param["bottom_drag_coef"])
        self.rho = float(param.get("rho_water", 1025.0))
        self.h_wind = param.get("h_wind", None)
        self.h_min = float(param.get("h_min", 0.1))
        self.sharp = float(param.get("h_min_sharpness", 10.0))
        self.visc = float(param.get("visc_coef", 0.0) or 0.0)
        self.diff = float(param.get("diff_coef", 0.0) or 0.0)
        self.dt = float(param["dt"])
        self.linear = bool(param.get("flag_linear", False))
        self.sponge_coef = float(param.get("sponge_coef", 0.0))
        self.sponge_u = np.zeros((nx + 1, ny))
        self.sponge_v = np.zeros((nx, ny + 1))
        self.sponge_h = np.zeros((nx, ny))
        self.forcing_momentum = param.get("forcing_momentum", "direct")
        self.H = np.asarray(param["H"], dtype=np.float64)
        # barotropic filter, spectral form (sw.py:305-320): a Neumann Helmholtz
        # solve diagonalised by one DCT-II per direction (helmholtz.py:20-87)
        self.barotropic_filter = bool(param.get("barotropic_filter", False))
        if self.barotropic_filter:
            if not param.get("barotropic_filter_spectral", False):
                raise NotImplementedError("the exact (multigrid) barotropic filter is work in progress in the "
                                          "reference (sw.py:712-719)")
            if np.any(self.masks.h < 0.5):
                raise NotImplementedError("the reference's spectral filter solver does not construct with land "
                                          "(helmholtz.py:254 divides a face-grid difference by the [nx, ny] "
                                          "spacing)")
            self.tau = 2 * self.dt
            self.g = float(self.gp.reshape(-1)[0])
            lambd = 1.0 / (self.g * self.dt * self.tau * self.H.sum(axis=-3, keepdims=True))
            xg, yg = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
            self.helm_dct = (2 * (np.cos(np.pi / nx * xg) - 1) / self.dx ** 2
                             + 2 * (np.cos(np.pi / ny * yg) - 1) / self.dy ** 2) - lambd

    # reference values (sw.py:385-410), as functions of H_total
    def ref_values(self, H):
        h_ref = H * self.area
        eta_ref = -H.sum(axis=-3) + (H[::-1].cumsum(axis=-3))[::-1]
        p_ref = np.cumsum(self.gp * eta_ref, axis=-3)
        h_ref_u = _edge_avg(h_ref, -2)
        h_ref_v = _edge_avg(h_ref, -1)
        dxp = np.diff(p_ref, axis=-2) if H.shape[-2] != 1 else 0.0
        dyp = np.diff(p_ref, axis=-1) if H.shape[-1] != 1 else 0.0
        return h_ref, h_ref_u, h_ref_v, dxp, dyp

    # ---- barotropic filter, spectral form (sw.py:695-725) ----
    def neumann_solve(self, rhs):
        """HelmholtzNeumannSolver.solve without land (helmholtz.py:80-86,
        296-303): unnormalised DCT-II along y then x, division by the
        operator's eigenvalues, the inverse transforms."""
        import scipy.fft as sf
        r = sf.dct(sf.dct(rhs, type=2, axis=-1), type=2, axis=-2)
        return sf.idct(sf.idct(r / self.helm_dct, type=2, axis=-1), type=2, axis=-2)

    def filter_barotropic(self, du, dv, dh, u, v, htu, htv):
        m = self.masks
        us = (u + self.dt * du) / self.dx_u
        vs = (v + self.dt * dv) / self.dy_v
        ub = (us * htu).sum(axis=-3, keepdims=True) / htu.sum(axis=-3, keepdims=True)
        vb = (vs * htv).sum(axis=-3, keepdims=True) / htv.sum(axis=-3, keepdims=True)
        rhs = 1.0 / (self.g * self.dt * self.tau) * (np.diff(ub, axis=-2) / self.dx + np.diff(vb, axis=-1) / self.dy)
        w = self.neumann_solve(rhs)
        pad_u = [(0, 0)] * (w.ndim - 2) + [(1, 1), (0, 0)]
        pad_v = [(0, 0)] * (w.ndim - 2) + [(0, 0), (1, 1)]
        fu = np.pad(-self.g * self.tau * np.diff(w, axis=-2), pad_u) * m.u
        fv = np.pad(-self.g * self.tau * np.diff(w, axis=-1), pad_v) * m.v
        return du + fu, dv + fv, dh

    def to_model(self, u, v, h):
        m = self.masks
        return u * m.u * self.dx_u, v * m.v * self.dy_v, h * m.h * self.area

    def omega(self, u, v):
        m = self.masks
        up = np.pad(u, [(0, 0)] * (u.ndim - 1) + [(1, 1)])
        vp = np.pad(v, [(0, 0)] * (v.ndim - 2) + [(1, 1), (0, 0)])
        dxv = np.diff(vp, axis=-2)
        dyu = np.diff(up, axis=-1)
        curl = dxv - dyu
        a = 2 * (1 - self.slip)
        return (m.w_valid * curl + m.w_cornerout_bound * (1 - self.slip) * curl
                + m.w_vertical_bound * a * dxv - m.w_horizontal_bound * a * dyu)

    def wind(self, refv, taux, tauy):
        m = self.masks
        hw = self.h_wind
        if hw is not None:
            hw = np.asarray(hw, dtype=np.float64)
            if hw.ndim >= 2:
                Hu = np.maximum(0.5 * (hw[:-1, :] + hw[1:, :]), self.h_min)
                Hv = np.maximum(0.5 * (hw[:, :-1] + hw[:, 1:]), self.h_min)
            else:
                Hu = Hv = np.maximum(hw, self.h_min)
        else:
            # the model's own reference thickness, not the one of a perturbed H
            # passed to step (sw.py:622-630 read self.h_ref_ugrid / _vgrid)
            base = self.ref_values(self.H)
            H0u, H0v = base[1][0], base[2][0]
            if H0u.shape[0] > 1:
                H0u = H0u[1:-1, :]
            if H0v.shape[1] > 1:
                H0v = H0v[:, 1:-1]
            Hu = np.maximum(H0u / self.area_u[1:-1, :], self.h_min)
            Hv = np.maximum(H0v / self.area_v[:, 1:-1], self.h_min)
        wu = np.where(m.u[1:-1, :] > 0.5, taux / (self.rho * Hu) * self.dx_u[1:-1, :], 0.0)
        wv = np.where(m.v[:, 1:-1] > 0.5, tauy / (self.rho * Hv) * self.dy_v[:, 1:-1], 0.0)
        return wu, wv

    def rhs(self, u, v, h, refv, taux, tauy):
        """compute_time_derivatives (sw.py:727-750), with the spectral
        barotropic filter when the model has it."""
        m = self.masks
        h_ref, _, _, dxp, dyp = refv
        om = self.omega(u, v)
        eta = (h / self.area)[..., ::-1, :, :].cumsum(axis=-3)[..., ::-1, :, :]
        p = np.cumsum(self.gp * eta, axis=-3)
        U, V = u / self.dx_u ** 2, v / self.dy_v ** 2
        Um, Vm = interp_TP(U), interp_TP(V)
        usq, vsq = u * U, v * V
        ke = 0.25 * (usq[..., 1:, :] + usq[..., :-1, :] + vsq[..., 1:] + vsq[..., :-1]) * m.h
        # thickness
        if self.linear:
            htot = h_ref * np.ones_like(h)
        else:
            htot = smooth_clamp(h_ref + h, self.h_min * self.area, self.sharp)
        fy = weno_flux(htot, V[..., 1:-1], -1, *(a[:, 1:-1] for a in m.v_hy))
        fx = weno_flux(htot, U[..., 1:-1, :], -2, *(a[1:-1, :] for a in m.u_hx))
        dth = -div_noflux(fx, fy) * m.h
        if self.diff > 0:
            hp = np.pad(h / self.area, [(0, 0)] * (h.ndim - 2) + [(1, 1), (1, 1)], mode="edge")
            lap = ((hp[..., 2:, 1:-1] - 2 * hp[..., 1:-1, 1:-1] + hp[..., :-2, 1:-1]) / self.dx ** 2
                   + (hp[..., 1:-1, 2:] - 2 * hp[..., 1:-1, 1:-1] + hp[..., 1:-1, :-2]) / self.dy ** 2)
            dth = dth + self.diff * lap * self.area * m.h
        # momentum
        oVm = weno_flux(om[..., 1:-1, :], Vm, -1, *(a[1:-1, :] for a in m.u_wy))
        oUm = weno_flux(om[..., 1:-1], Um, -2, *(a[:, 1:-1] for a in m.v_wx))
        du = oVm + self.fstar_u[1:-1, :] * Vm
        dv = -(oUm + self.fstar_v[:, 1:-1] * Um)
        kp = ke + p
        du = du - (np.diff(kp, axis=-2) + dxp)
        dv = dv - (np.diff(kp, axis=-1) + dyp)
        wu, wv = self.wind(refv, taux, tauy)
        du[..., 0, :, :] += wu
        dv[..., 0, :, :] += wv
        du[..., -1, :, :] -= self.drag * u[..., -1, 1:-1, :]
        dv[..., -1, :, :] -= self.drag * v[..., -1, :, 1:-1]
        if self.visc > 0:
            upad = np.pad(u, [(0, 0)] * (u.ndim - 1) + [(1, 1)], mode="edge")
            vpad = np.pad(v, [(0, 0)] * (v.ndim - 2) + [(1, 1), (0, 0)], mode="edge")
            up = upad / np.pad(self.dx_u, ((0, 0), (1, 1)), mode="edge")
            vp = vpad / np.pad(self.dy_v, ((1, 1), (0, 0)), mode="edge")
            dxu, dyu = self.dx_u[1:-1, :], self.dy_u[1:-1, :]
            lu = ((up[..., 2:, 1:-1] - 2 * up[..., 1:-1, 1:-1] + up[..., :-2, 1:-1]) / dxu ** 2
                  + (up[..., 1:-1, 2:] - 2 * up[..., 1:-1, 1:-1] + up[..., 1:-1, :-2]) / dyu ** 2)
            dxv, dyv = self.dx_v[:, 1:-1], self.dy_v[:, 1:-1]
            lv = ((vp[..., 2:, 1:-1] - 2 * vp[..., 1:-1, 1:-1] + vp[..., :-2, 1:-1]) / dxv ** 2
                  + (vp[..., 1:-1, 2:] - 2 * vp[..., 1:-1, 1:-1] + vp[..., 1:-1, :-2]) / dyv ** 2)
            du = du + self.visc * lu * dxu
            dv = dv + self.visc * lv * dyv
        pad_u = [(0, 0)] * (du.ndim - 2) + [(1, 1), (0, 0)]
        pad_v = [(0, 0)] * (dv.ndim - 2) + [(0, 0), (1, 1)]
        du, dv = np.pad(du, pad_u) * m.u, np.pad(dv, pad_v) * m.v
        if self.barotropic_filter:
            # total thickness on the faces (sw.py:688-692)
            _, h_ref_u, h_ref_v, _, _ = refv
            hu, hv = self._h_on_uv(h)
            htu = smooth_clamp(h_ref_u + hu, self.h_min * self.area_u, self.sharp)
            htv = smooth_clamp(h_ref_v + hv, self.h_min * self.area_v, self.sharp)
            du, dv, dth = self.filter_barotropic(du, dv, dth, u, v, htu, htv)
        return du, dv, dth

    def _h_on_uv(self, h):
        """replicate_pad then face averages (sw.py:36-48, 711-713)."""
        m = self.masks.h
        hp = np.pad(h, [(0, 0)] * (h.ndim - 2) + [(1, 1), (1, 1)], mode="edge")
        mp = np.pad(m, ((1, 1), (1, 1)), mode="edge")
        ms = _pool_sum(_pool_sum(mp, 3, 1, 1, 0), 1, 3, 0, 1)
        flat = hp.reshape((-1,) + hp.shape[-2:])
        fs = np.stack([_pool_sum(_pool_sum(a, 3, 1, 1, 0), 1, 3, 0, 1) for a in flat]).reshape(hp.shape)
        hr = mp * hp + (1 - mp) * (fs / np.maximum(1.0, ms))
        return 0.5 * (hr[..., 1:, 1:-1] + hr[..., :-1, 1:-1]), 0.5 * (hr[..., 1:-1, 1:] + hr[..., 1:-1, :-1])

    def step(self, u0, v0, h0, H=None, nstep=1, u_b=None, v_b=None, h_b=None, Fu=None, Fv=None, Fh=None,
             taux=None, tauy=None):
        """SW.step (sw.py:752-904): physical in, physical out."""
        u, v, h = self.to_model(u0, v0, h0)
        ub, vb, hb = self.to_model(u0 if u_b is None else u_b, v0 if v_b is None else v_b,
                                   h0 if h_b is None else h_b)
        zu, zv, zh = np.zeros_like(u0), np.zeros_like(v0), np.zeros_like(h0)
        fu, fv, fh = self.to_model(zu if Fu is None else Fu, zv if Fv is None else Fv, zh if Fh is None else Fh)
        refv = self.ref_values(self.H if H is None else self.H + H)
        taux = self.taux if taux is None else taux
        tauy = self.tauy if tauy is None else tauy
        g = self.sponge_coef / self.dt
        gu, gv, gh = g * self.sponge_u, g * self.sponge_v, g * self.sponge_h
        dt = self.dt
        for _ in range(nstep):
            k0 = self.rhs(u, v, h, refv, taux, tauy)
            k0 = (k0[0] + gu * (ub - u), k0[1] + gv * (vb - v), k0[2] + gh * (hb - h))
            u1, v1, h1 = u + dt * k0[0], v + dt * k0[1], h + dt * k0[2]
            k1 = self.rhs(u1, v1, h1, refv, taux, tauy)
            k1 = (k1[0] + gu * (ub - u1), k1[1] + gv * (vb - v1), k1[2] + gh * (hb - h1))
            u2 = u1 + dt / 4 * (k1[0] - 3 * k0[0])
            v2 = v1 + dt / 4 * (k1[1] - 3 * k0[1])
            h2 = h1 + dt / 4 * (k1[2] - 3 * k0[2])
            k2 = self.rhs(u2, v2, h2, refv, taux, tauy)
            k2 = (k2[0] + gu * (ub - u2), k2[1] + gv * (vb - v2), k2[2] + gh * (hb - h2))
            u = u2 + dt / 12 * (8 * k2[0] - k1[0] - k0[0])
            v = v2 + dt / 12 * (8 * k2[1] - k1[1] - k0[1])
            h = h2 + dt / 12 * (8 * k2[2] - k1[2] - k0[2])
            if self.forcing_momentum == "mass_consistent":
                hu, hv = self._h_on_uv(h)
                htu = smooth_clamp(refv[1] + hu, self.h_min * self.area_u, self.sharp)
                htv = smooth_clamp(refv[2] + hv, self.h_min * self.area_v, self.sharp)
                fhu, fhv = self._h_on_uv(fh)
                u = u + dt * (-u / htu * fhu)
                v = v + dt * (-v / htv * fhv)
            u, v, h = u + dt * fu, v + dt * fv, h + dt * fh
        return u / self.dx_u, v / self.dy_v, h / self.area
