"""Oracle (test infrastructure only): restatement of the reference's masked
multigrid Helmholtz solver (mapping/models/model_qgsw/helmholtz_multigrid.py)
in float64 NumPy.

Solves  div(c grad u) - lambda u = rhs  on cell centres of a masked domain
embedded in an n0 x n1 rectangle, homogeneous Neumann walls on cell edges;
axis 0 has spacing d0 (the reference's x), axis 1 spacing d1. A batch of
systems shares the grid and the coefficient; system b uses lambda[b]
(the reference's lambd of shape (nl, 1, 1)).

  compute_nlevels            helmholtz_multigrid.py:27-33
  compute_mask_uvgrids       36-48   (avg_pool2d: model_qgsw/tools.py:9-69)
  compute_helmholtz_matrix   51-70
  jacobi_smoothing           73-99   (6 damped sweeps)
  residual                   102-114
  prolong / restrict         117-151
  hierarchies                248-293
  V_cycle / FMG_Helmholtz    322-419

Parity status: pinned to solutions of the reference's own
helmholtz_multigrid.py run with a NumPy stand-in for jax
(tests/golden/gen_golden_mg.py, ≤1e-12), and to the solution of the
assembled operator (scipy spsolve) after convergence.
"""
import numpy as np


def compute_nlevels(n):
    if n <= 8:
        return 1
    h = int(np.log2(n & (~(n - 1))))
    while n // 2 ** h < 8:
        h -= 1
    return 1 + h


def _pad(f):
    return np.pad(f, [(0, 0)] * (f.ndim - 2) + [(1, 1), (1, 1)])


def pool_u(m):
    """Sum of the two cells either side of every axis-0 edge (zero outside):
    avg_pool2d(m, (2, 1), padding (1, 0), divisor 1)."""
    p = np.pad(m, [(0, 0)] * (m.ndim - 2) + [(1, 1), (0, 0)])
    return p[..., 1:, :] + p[..., :-1, :]


def pool_v(m):
    p = np.pad(m, [(0, 0)] * (m.ndim - 2) + [(0, 0), (1, 1)])
    return p[..., :, 1:] + p[..., :, :-1]


def mask_uvgrids(mask):
    return (pool_u(mask) > 1.5).astype(mask.dtype), (pool_v(mask) > 1.5).astype(mask.dtype)


def helmholtz(f, d0, d1, lam, mask, cu, cv):
    f_ = _pad(f)
    dx_f = np.diff(f_[..., 1:-1], axis=-2)
    dy_f = np.diff(f_[..., 1:-1, :], axis=-1)
    return (np.diff(cu * dx_f, axis=-2) / d0 ** 2 + np.diff(cv * dy_f, axis=-1) / d1 ** 2 - lam * f) * mask


def jacobi_smoothing(f, rhs, d0, d1, mask, cu, cv, omega, lam):
    dxm2, dym2 = 1. / d0 ** 2, 1. / d1 ** 2
    factor = mask / (lam + dxm2 * (cu[..., 1:, :] + cu[..., :-1, :]) + dym2 * (cv[..., 1:] + cv[..., :-1]))
    for _ in range(6):
        f_ = _pad(f)
        f = omega * factor * (dxm2 * (cu[..., 1:, :] * f_[..., 2:, 1:-1] + cu[..., :-1, :] * f_[..., :-2, 1:-1])
                              + dym2 * (cv[..., 1:] * f_[..., 1:-1, 2:] + cv[..., :-1] * f_[..., 1:-1, :-2])
                              - rhs) + (1 - omega) * f
    return f


def residual(f, rhs, d0, d1, mask, cu, cv, lam):
    return rhs - helmholtz(f, d0, d1, lam, mask, cu, cv)


def prolong(v, divisor=16):
    n0, n1 = v.shape[-2:]
    v_ = _pad(v)
    c = v_[..., 1:-1, 1:-1]
    q00 = 9 * c + 3 * (v_[..., 1:-1, 0:-2] + v_[..., 0:-2, 1:-1]) + v_[..., 0:-2, 0:-2]
    q10 = 9 * c + 3 * (v_[..., 1:-1, 0:-2] + v_[..., 2:, 1:-1]) + v_[..., 2:, 0:-2]
    q01 = 9 * c + 3 * (v_[..., 1:-1, 2:] + v_[..., 0:-2, 1:-1]) + v_[..., 0:-2, 2:]
    q11 = 9 * c + 3 * (v_[..., 2:, 1:-1] + v_[..., 1:-1, 2:]) + v_[..., 2:, 2:]
    out = np.zeros(v.shape[:-2] + (2 * n0, 2 * n1))
    out[..., 0::2, 0::2] = q00
    out[..., 1::2, 0::2] = q10
    out[..., 0::2, 1::2] = q01
    out[..., 1::2, 1::2] = q11
    return out / divisor


def restrict(v, divisor=4):
    return (v[..., :-1:2, :-1:2] + v[..., 1::2, :-1:2] + v[..., ::2, 1::2] + v[..., 1::2, 1::2]) / divisor


class MGOracle:
    """MG_Helmholtz (helmholtz_multigrid.py:156-419) in float64."""

    def __init__(self, d0, d1, n0, n1, coef_u, coef_v, lam, mask=None, n_levels=None, max_ite=20,
                 niter_bottom=-1):
        self.lam = np.asarray(lam, dtype=np.float64).reshape(-1, 1, 1)
        if n_levels is None:
            n_levels = min(compute_nlevels(n0), compute_nlevels(n1))
        N = 2 ** (n_levels - 1)
        assert n0 % N == 0 and n1 % N == 0
        self.n0, self.n1, self.d0, self.d1 = n0, n1, float(d0), float(d1)
        self.omega = 0.95
        self.n_levels, self.max_ite, self.niter_bottom = n_levels, max_ite, niter_bottom
        mask = np.ones((n0, n1)) if mask is None else np.asarray(mask, dtype=np.float64)
        mask = mask[None]
        mu, mv = mask_uvgrids(mask)
        self.masks, self.masks_u, self.masks_v = [mask], [mu], [mv]
        for _ in range(1, n_levels):
            m = (restrict(self.masks[-1]) > 0.5).astype(np.float64)
            mu, mv = mask_uvgrids(m)
            self.masks.append(m)
            self.masks_u.append(mu)
            self.masks_v.append(mv)
        self.div_r = [None]
        for n in range(1, n_levels):
            d = restrict(self.masks[n - 1], divisor=1)
            self.div_r.append(np.maximum(d, np.ones_like(d)))
        self.div_p = []
        for n in range(n_levels - 1):
            d = prolong(self.masks[n + 1], divisor=1)
            self.div_p.append(np.maximum(d, np.ones_like(d)))
        self.div_p.append(None)
        cu = np.asarray(coef_u, dtype=np.float64)
        cv = np.asarray(coef_v, dtype=np.float64)
        coef = 0.25 * (cu[1:, :] + cu[:-1, :] + cv[:, 1:] + cv[:, :-1])[None]
        self.cu = [cu[None] * self.masks_u[0]]
        self.cv = [cv[None] * self.masks_v[0]]
        for i in range(1, n_levels):
            coef = restrict(coef, self.div_r[i]) * self.masks[i]
            self.cu.append(pool_u(coef) / 2 * self.masks_u[i])
            self.cv.append(pool_v(coef) / 2 * self.masks_v[i])
        if niter_bottom <= 0:
            s = 2 ** (n_levels - 1)
            mb = self.masks[-1][0]
            self.i_s, self.j_s = np.where(mb)
            Nb = self.i_s.size
            self.binv = []
            for b in range(self.lam.shape[0]):
                H = np.zeros((Nb, Nb))
                for k in range(Nb):
                    x = np.zeros((1,) + mb.shape)
                    x[0, self.i_s[k], self.j_s[k]] = 1
                    Hx = helmholtz(x, self.d0 * s, self.d1 * s, self.lam[b], self.masks[-1], self.cu[-1],
                                   self.cv[-1])
                    H[:, k] = Hx[0, self.i_s, self.j_s]
                self.binv.append(np.linalg.pinv(H))

    def _bottom(self, f, rhs, d0, d1):
        if self.niter_bottom <= 0:
            f = np.zeros_like(rhs)
            for b in range(rhs.shape[0]):
                f[b, self.i_s, self.j_s] = rhs[b, self.i_s, self.j_s] @ self.binv[b]
            return f
        for _ in range(self.niter_bottom):
            f = jacobi_smoothing(f, rhs, d0, d1, self.masks[-1], self.cu[-1], self.cv[-1], self.omega, self.lam)
        return f

    def V_cycle(self, f, rhs, d0, d1, level=0):
        if level == self.n_levels - 1:
            return self._bottom(f, rhs, d0, d1)
        m, cu, cv = self.masks[level], self.cu[level], self.cv[level]
        f = jacobi_smoothing(f, rhs, d0, d1, m, cu, cv, self.omega, self.lam)
        res = residual(f, rhs, d0, d1, m, cu, cv, self.lam)
        rc = restrict(res, self.div_r[level + 1]) * self.masks[level + 1]
        ec = self.V_cycle(np.zeros_like(rc), rc, d0 * 2, d1 * 2, level + 1)
        f = f + prolong(ec, self.div_p[level]) * m
        return jacobi_smoothing(f, rhs, d0, d1, m, cu, cv, self.omega, self.lam)

    def solve(self, rhs):
        rhs = np.asarray(rhs, dtype=np.float64)
        rl = [rhs]
        for i in range(1, self.n_levels):
            rl.append(restrict(rl[-1], self.div_r[i]) * self.masks[i])
        k = 2 ** (self.n_levels - 1)
        f = self._bottom(np.zeros_like(rl[-1]), rl[-1], k * self.d0, k * self.d1)
        for i in range(2, self.n_levels + 1):
            k = 2 ** (self.n_levels - i)
            f = prolong(f, self.div_p[-i]) * self.masks[-i]
            f = self.V_cycle(f, rl[-i], k * self.d0, k * self.d1, level=self.n_levels - i)
        for _ in range(self.max_ite):
            f = self.V_cycle(f, rhs, self.d0, self.d1)
        return f

    def operator_matrix(self, b=0):
        """The assembled fine-level operator on the masked cells (for an
        exact reference solution)."""
        import scipy.sparse as sp
        m = self.masks[0][0]
        i_s, j_s = np.where(m)
        idx = -np.ones(m.shape, dtype=np.int64)
        idx[i_s, j_s] = np.arange(i_s.size)
        cu, cv = self.cu[0][0], self.cv[0][0]
        rows, cols, vals = [], [], []
        for k, (i, j) in enumerate(zip(i_s, j_s)):
            diag = -self.lam[b, 0, 0]
            for (ii, jj, c, dd) in ((i + 1, j, cu[i + 1, j], self.d0), (i - 1, j, cu[i, j], self.d0),
                                    (i, j + 1, cv[i, j + 1], self.d1), (i, j - 1, cv[i, j], self.d1)):
                diag -= c / dd ** 2
                if 0 <= ii < m.shape[0] and 0 <= jj < m.shape[1] and idx[ii, jj] >= 0 and c != 0:
                    rows.append(k)
                    cols.append(idx[ii, jj])
                    vals.append(c / dd ** 2)
            rows.append(k)
            cols.append(k)
            vals.append(diag)
        return sp.csr_matrix((vals, (rows, cols)), shape=(i_s.size, i_s.size)), i_s, j_s
