"""Outer 4D-Var minimisation on the GPU: L-BFGS without bounds for a batch
of independent windows (the quasi-Newton loop of mapping/src/inv.py:309-414,
which calls ``scipy.optimize.minimize(method='L-BFGS-B')`` without bounds).

The iteration follows L-BFGS-B 3.0 (Byrd, Lu, Nocedal, Zhu 1995; Morales,
Nocedal 2011) on an unconstrained problem, the algorithm of scipy's
``L-BFGS-B`` (scipy is a third-party dependency of the reference, not vendored
there):

- first direction (and after a restart) ``-g / theta`` with theta = 1; later
  directions ``-H g`` with the limited-memory inverse Hessian of the m last
  pairs, initial scaling s'y / y'y (what the compact form of L-BFGS-B
  computes, here by the two-loop recursion on the device);
- line search: the Moré-Thuente ``dcsrch`` / ``dcstep`` of MINPACK-2
  (ftol 1e-3, gtol 0.9, xtol 0.1), first step min(1/||d||, 1e10) on the first
  iteration and 1 afterwards, at most ``maxls`` evaluations, a failed search
  restarting from steepest descent (abnormal termination when already
  there);
- pair update skipped when s'y <= eps * (-g'd * stp) with s'y formed as
  (g_new - g_old)'d * stp;
- stops: max|g| <= gtol, (f_old - f) <= ftol * max(|f_old|, |f|, 1),
  maxiter, maxfun.

Vectors, the pair history and the two-loop recursion stay on the device in
float64 (vd_bdot_f64, vd_baxpy_f64, vd_bxpay_f64: coefficients are device
arrays, so the recursion needs no host round trip); per evaluation only the
cost and g'd of each window come back to the host for the line search.
"""
import ctypes

import numpy as np
import torch

from . import _lib

EPSMCH = np.finfo(np.float64).eps


# ------------------------------------------------------------------ line search
def dcstep(stx, fx, dx, sty, fy, dy, stp, fp, dp, brackt, stpmin, stpmax):
    """Safeguarded step of Moré & Thuente (1994), MINPACK-2 ``dcstep``."""
    sgnd = dp * (dx / abs(dx))
    if fp > fx:
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp < stx:
            gamma = -gamma
        p = (gamma - dx) + theta
        q = ((gamma - dx) + gamma) + dp
        r = p / q
        stpc = stx + r * (stp - stx)
        stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx)
        stpf = stpc if abs(stpc - stx) < abs(stpq - stx) else stpc + (stpq - stpc) / 2.0
        brackt = True
    elif sgnd < 0.0:
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = ((gamma - dp) + gamma) + dx
        r = p / q
        stpc = stp + r * (stx - stp)
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
        brackt = True
    elif abs(dp) < abs(dx):
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * np.sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = (gamma + (dx - dp)) + gamma
        r = p / q
        if r < 0.0 and gamma != 0.0:
            stpc = stp + r * (stx - stp)
        elif stp > stx:
            stpc = stpmax
        else:
            stpc = stpmin
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        if brackt:
            stpf = stpc if abs(stpc - stp) < abs(stpq - stp) else stpq
            if stp > stx:
                stpf = min(stp + 0.66 * (sty - stp), stpf)
            else:
                stpf = max(stp + 0.66 * (sty - stp), stpf)
        else:
            stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
            stpf = min(stpmax, stpf)
            stpf = max(stpmin, stpf)
    else:
        if brackt:
            theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp
            s = max(abs(theta), abs(dy), abs(dp))
            gamma = s * np.sqrt((theta / s) ** 2 - (dy / s) * (dp / s))
            if stp > sty:
                gamma = -gamma
            p = (gamma - dp) + theta
            q = ((gamma - dp) + gamma) + dy
            r = p / q
            stpf = stp + r * (sty - stp)
        elif stp > stx:
            stpf = stpmax
        else:
            stpf = stpmin
    if fp > fx:
        sty, fy, dy = stp, fp, dp
    else:
        if sgnd < 0.0:
            sty, fy, dy = stx, fx, dx
        stx, fx, dx = stp, fp, dp
    return stx, fx, dx, sty, fy, dy, stpf, brackt


class LineSearch:
    """Moré-Thuente line search of MINPACK-2 ``dcsrch`` as a state machine:
    ``start(f, g, stp)`` then ``step(f, g, stp)`` until the task is not
    'FG'."""

    XTRAPL, XTRAPU = 1.1, 4.0

    def __init__(self, ftol=1e-3, gtol=0.9, xtol=0.1, stpmin=0.0, stpmax=1e10):
        self.ftol, self.gtol, self.xtol = ftol, gtol, xtol
        self.stpmin, self.stpmax = stpmin, stpmax

    def start(self, f, g, stp):
        if stp < self.stpmin:
            return "ERROR: STP .LT. STPMIN", stp
        if stp > self.stpmax:
            return "ERROR: STP .GT. STPMAX", stp
        if g >= 0.0:
            return "ERROR: INITIAL G .GE. ZERO", stp
        self.brackt = False
        self.stage = 1
        self.finit, self.ginit = f, g
        self.gtest = self.ftol * g
        self.width = self.stpmax - self.stpmin
        self.width1 = self.width / 0.5
        self.stx, self.fx, self.gx = 0.0, f, g
        self.sty, self.fy, self.gy = 0.0, f, g
        self.stmin = 0.0
        self.stmax = stp + self.XTRAPU * stp
        return "FG", stp

    def step(self, f, g, stp):
        ftest = self.finit + stp * self.gtest
        if self.stage == 1 and f <= ftest and g >= 0.0:
            self.stage = 2
        task = None
        if self.brackt and (stp <= self.stmin or stp >= self.stmax):
            task = "WARNING: ROUNDING ERRORS PREVENT PROGRESS"
        if self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax:
            task = "WARNING: XTOL TEST SATISFIED"
        if stp == self.stpmax and f <= ftest and g <= self.gtest:
            task = "WARNING: STP = STPMAX"
        if stp == self.stpmin and (f > ftest or g >= self.gtest):
            task = "WARNING: STP = STPMIN"
        if f <= ftest and abs(g) <= self.gtol * (-self.ginit):
            task = "CONVERGENCE"
        if task is not None:
            return task, stp
        if self.stage == 1 and f <= self.fx and f > ftest:
            gt = self.gtest
            fm, fxm, fym = f - stp * gt, self.fx - self.stx * gt, self.fy - self.sty * gt
            gm, gxm, gym = g - gt, self.gx - gt, self.gy - gt
            (self.stx, fxm, gxm, self.sty, fym, gym, stp, self.brackt) = dcstep(
                self.stx, fxm, gxm, self.sty, fym, gym, stp, fm, gm, self.brackt, self.stmin, self.stmax)
            self.fx, self.fy = fxm + self.stx * gt, fym + self.sty * gt
            self.gx, self.gy = gxm + gt, gym + gt
        else:
            (self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, self.brackt) = dcstep(
                self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, f, g, self.brackt, self.stmin,
                self.stmax)
        if self.brackt:
            if abs(self.sty - self.stx) >= 0.66 * self.width1:
                stp = self.stx + 0.5 * (self.sty - self.stx)
            self.width1 = self.width
            self.width = abs(self.sty - self.stx)
        if self.brackt:
            self.stmin = min(self.stx, self.sty)
            self.stmax = max(self.stx, self.sty)
        else:
            self.stmin = stp + self.XTRAPL * (stp - self.stx)
            self.stmax = stp + self.XTRAPU * (stp - self.stx)
        stp = max(stp, self.stpmin)
        stp = min(stp, self.stpmax)
        if (self.brackt and (stp <= self.stmin or stp >= self.stmax)) or \
                (self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax):
            stp = self.stx
        return "FG", stp


# ------------------------------------------------------------------ batched L-BFGS
class _Vec:
    """Device float64 batched vector ops through the C ABI."""

    def __init__(self, B, n, device):
        self.B, self.n = B, n
        self.work = torch.empty(max(8, _lib.load().vd_bdot_workspace_bytes(B, n) // 8), dtype=torch.float64,
                                device=device)
        self.device = device

    @staticmethod
    def _p(t):
        return None if t is None else ctypes.c_void_p(t.data_ptr())

    def _st(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def dot(self, x, y, out, c0=None, c1=None):
        _lib.call("vd_bdot_f64", self.B, self.n, self._p(x), self._p(y), self._p(c0), self._p(c1), self._p(out),
                  self._p(self.work), self.work.numel() * 8, self._st())
        return out

    def axpy(self, scale, coef, x, beta, y):
        _lib.call("vd_baxpy_f64", self.B, self.n, float(scale), self._p(coef), self._p(x), float(beta), self._p(y),
                  self._st())

    def xpay(self, x, coef, y, z):
        _lib.call("vd_bxpay_f64", self.B, self.n, self._p(x), self._p(coef), self._p(y), self._p(z), self._st())


class BatchedLBFGS:
    """L-BFGS-B without bounds for B independent problems of size n.

    ``fun(x)`` takes a [B, n] float64 CUDA tensor and returns (f [B],
    g [B, n]) (f a host array or tensor, g a CUDA tensor of any float type).
    Options and stopping rules are scipy's ``L-BFGS-B`` ones: ``m``
    (maxcor), ``ftol``, ``gtol`` (on max|g|), ``maxiter``, ``maxfun``,
    ``maxls``."""

    def __init__(self, fun, B, n, m=10, ftol=2.220446049250313e-09, gtol=1e-5, maxiter=15000, maxfun=15000,
                 maxls=20, device="cuda", callback=None):
        self.fun, self.B, self.n, self.m = fun, int(B), int(n), int(m)
        self.ftol, self.gtol = float(ftol), np.broadcast_to(np.asarray(gtol, dtype=np.float64), (self.B,)).copy()
        self.maxiter, self.maxfun, self.maxls = int(maxiter), int(maxfun), int(maxls)
        self.device = torch.device(device)
        self.callback = callback
        self.vec = _Vec(self.B, self.n, self.device)

    def _eval(self, x, status):
        out = self.fun(x)
        f, g = out[0], out[1]
        f = np.asarray(f.detach().cpu().numpy() if torch.is_tensor(f) else f, dtype=np.float64).reshape(self.B)
        if len(out) > 2:
            stop = np.asarray(out[2], dtype=bool) & (status < 0)
            status[stop] = 3
        return f, g.to(torch.float64).reshape(self.B, self.n)

    def _direction(self, g, S, Y, rho, nrho, gamma, order):
        """d = -H g by the two-loop recursion on the device; pairs with
        rho = 0 contribute nothing, ``order`` lists ring slots newest first."""
        B, dev, vec = self.B, self.device, self.vec
        q = torch.empty_like(g)
        vec.axpy(-1.0, None, g, 0.0, q)              # q = -g
        alpha = torch.zeros((self.m, B), dtype=torch.float64, device=dev)
        for k in order:                              # newest -> oldest
            vec.dot(S[k], q, alpha[k], c1=rho[k])    # alpha = rho s'q
            vec.axpy(-1.0, alpha[k], Y[k], 1.0, q)   # q -= alpha y
        r = torch.empty_like(g)
        vec.axpy(1.0, gamma, q, 0.0, r)              # r = gamma q
        coef = torch.empty(B, dtype=torch.float64, device=dev)
        for k in reversed(order):                    # oldest -> newest
            vec.dot(Y[k], r, coef, c0=alpha[k], c1=nrho[k])   # alpha - rho y'r
            vec.axpy(1.0, coef, S[k], 1.0, r)        # r += s (alpha - beta)
        return r

    def minimize(self, x0, active=None):
        """Run all windows to termination. ``active`` (bool [B]) leaves the
        other windows untouched (status 4). ``fun`` may return a third item,
        a bool [B] mask of windows to stop at once (status 3)."""
        B, n, m, dev, vec = self.B, self.n, self.m, self.device, self.vec
        x = torch.as_tensor(x0, dtype=torch.float64, device=dev).reshape(B, n).clone()
        status = np.full(B, -1, dtype=np.int64)   # -1 running, 0 converged, 1 stop, 2 abnormal, 3 stopped, 4 inactive
        message = [""] * B
        if active is not None:
            status[~np.asarray(active, dtype=bool)] = 4
        f, g = self._eval(x, status)
        g = g.clone()
        nfev = np.ones(B, dtype=np.int64)
        nit = np.zeros(B, dtype=np.int64)
        S = torch.zeros((m, B, n), dtype=torch.float64, device=dev)
        Y = torch.zeros((m, B, n), dtype=torch.float64, device=dev)
        rho_h = np.zeros((m, B))
        col = np.zeros(B, dtype=np.int64)
        head = np.zeros(B, dtype=np.int64)          # ring slot of the next pair
        theta = np.ones(B)
        sbg = torch.amax(torch.abs(g), dim=1).cpu().numpy()
        for b in range(B):
            if status[b] < 0 and sbg[b] <= self.gtol[b]:
                status[b], message[b] = 0, "CONVERGENCE: NORM OF PROJECTED GRADIENT <= PGTOL"
        need_dir = status < 0
        d = torch.zeros_like(x)
        t = x.clone()
        r = g.clone()
        fold = f.copy()
        stp = np.zeros(B)
        gdold = np.zeros(B)
        ls = [LineSearch() for _ in range(B)]
        ifun = np.zeros(B, dtype=np.int64)
        iback = np.zeros(B, dtype=np.int64)
        gd_dev = torch.empty(B, dtype=torch.float64, device=dev)
        while np.any(status < 0):
            act = status < 0
            # ---- new directions for the windows that start an iteration
            nd = need_dir & act
            if np.any(nd):
                rho = torch.as_tensor(rho_h, device=dev)
                gam = torch.as_tensor(np.where(col > 0, 1.0 / theta, 1.0), device=dev)
                dn = self._direction_batched(g, S, Y, rho, gam, self._orders(head))
                sel = torch.as_tensor(nd, device=dev)[:, None]
                d = torch.where(sel, dn, d)
                dd = torch.empty(B, dtype=torch.float64, device=dev)
                vec.dot(d, d, dd)
                dnorm = np.sqrt(dd.cpu().numpy())
                for b in np.nonzero(nd)[0]:
                    stp[b] = min(1.0 / dnorm[b], 1e10) if nit[b] == 0 else 1.0
                    fold[b] = f[b]
                    ifun[b], iback[b] = 0, 0
                t = torch.where(sel, x, t)
                r = torch.where(sel, g, r)
                need_dir[:] = False
            # ---- line search step of every running window
            vec.dot(g, d, gd_dev)
            gd_h = gd_dev.cpu().numpy()
            trial = np.zeros(B, dtype=bool)
            done_ls = np.zeros(B, dtype=bool)
            failed = np.zeros(B, dtype=bool)
            for b in np.nonzero(act)[0]:
                if ifun[b] == 0:
                    gdold[b] = gd_h[b]
                    if gd_h[b] >= 0.0:
                        failed[b] = True      # the directional derivative is >= 0
                        continue
                    task, stp[b] = ls[b].start(f[b], gd_h[b], stp[b])
                else:
                    task, stp[b] = ls[b].step(f[b], gd_h[b], stp[b])
                if task.startswith("CONV") or task.startswith("WARN"):
                    done_ls[b] = True
                elif task.startswith("FG"):
                    ifun[b] += 1
                    iback[b] = ifun[b] - 1
                    if iback[b] >= self.maxls:
                        failed[b] = True
                    else:
                        trial[b] = True
                else:
                    failed[b] = True
            # ---- failed searches: restore, then restart or stop
            for b in np.nonzero(failed)[0]:
                x[b].copy_(t[b])
                g[b].copy_(r[b])
                f[b] = fold[b]
                if col[b] == 0:
                    status[b], message[b] = 2, "ABNORMAL_TERMINATION_IN_LNSRCH"
                    nit[b] += 1
                else:
                    col[b], head[b], theta[b] = 0, 0, 1.0
                    rho_h[:, b] = 0.0
                    need_dir[b] = True
            # ---- accepted points: the new iterate
            if np.any(done_ls):
                nit[done_ls] += 1
                self._accept(done_ls, x, g, f, r, d, stp, gd_h, gdold, fold, S, Y, rho_h, col, head, theta,
                             status, message, nit, nfev, need_dir)
            # ---- trial points: one batched evaluation
            if np.any(trial):
                stp_dev = torch.as_tensor(np.where(trial, stp, 0.0), device=dev)
                xn = torch.empty_like(x)
                vec.xpay(t, stp_dev, d, xn)
                selt = torch.as_tensor(trial, device=dev)[:, None]
                x = torch.where(selt, xn, x)
                fn, gn = self._eval(x, status)
                nfev[trial] += 1
                f = np.where(trial, fn, f)
                g = torch.where(selt, gn, g)
        return {"x": x, "fun": f, "jac": g, "nit": nit, "nfev": nfev, "status": status, "message": message}

    # helpers -------------------------------------------------------------
    def _orders(self, head):
        """Per window, ring slots newest first, padded with slots whose rho
        is zero (so every window runs the same m-step recursion)."""
        m = self.m
        return [[int((head[b] - 1 - k) % m) for k in range(m)] for b in range(self.B)]

    def _direction_batched(self, g, S, Y, rho, gam, order):
        """Two-loop recursion where window b visits its own slot order:
        the m history slots are gathered newest-first per window first."""
        B, m = self.B, self.m
        idx = torch.as_tensor(np.asarray(order, dtype=np.int64).T, device=self.device)   # [m][B]
        bidx = torch.arange(B, device=self.device)[None, :].expand(m, B)
        Sg = S[idx, bidx].contiguous()                 # [m][B][n], newest first
        Yg = Y[idx, bidx].contiguous()
        rg = rho[idx, bidx].contiguous()               # [m][B]
        return self._direction(g, Sg, Yg, rg, (-rg).contiguous(), gam, list(range(m)))

    def _accept(self, done, x, g, f, r, d, stp, gd_h, gdold, fold, S, Y, rho_h, col, head, theta, status,
                message, nit, nfev, need_dir):
        B, dev, vec = self.B, self.device, self.vec
        sbg = torch.amax(torch.abs(g), dim=1).cpu().numpy()
        y = g - r
        rr_dev = torch.empty(B, dtype=torch.float64, device=dev)
        vec.dot(y, y, rr_dev)
        rr = rr_dev.cpu().numpy()
        for b in np.nonzero(done)[0]:
            if self.callback is not None:
                self.callback(b, x[b])
            if nit[b] >= self.maxiter:
                status[b], message[b] = 1, "STOP: TOTAL NO. OF ITERATIONS REACHED LIMIT"
                continue
            if nfev[b] > self.maxfun:
                status[b], message[b] = 1, "STOP: TOTAL NO. OF F,G EVALUATIONS EXCEEDS LIMIT"
                continue
            if sbg[b] <= self.gtol[b]:
                status[b], message[b] = 0, "CONVERGENCE: NORM OF PROJECTED GRADIENT <= PGTOL"
                continue
            if fold[b] - f[b] <= self.ftol * max(abs(fold[b]), abs(f[b]), 1.0):
                status[b], message[b] = 0, "CONVERGENCE: RELATIVE REDUCTION OF F <= FACTR*EPSMCH"
                continue
            if stp[b] == 1.0:
                dr, ddum = gd_h[b] - gdold[b], -gdold[b]
                sb = d[b]
            else:
                dr, ddum = (gd_h[b] - gdold[b]) * stp[b], -gdold[b] * stp[b]
                sb = d[b] * stp[b]
            need_dir[b] = True
            if dr <= EPSMCH * ddum:
                continue
            k = int(head[b])
            S[k, b].copy_(sb)
            Y[k, b].copy_(y[b])
            rho_h[k, b] = 1.0 / dr
            head[b] = (k + 1) % self.m
            col[b] = min(col[b] + 1, self.m)
            theta[b] = rr[b] / dr


# ------------------------------------------------------------------ 4D-Var driver
class CrazyGradient(Exception):
    pass


def minimize_4dvar(cost_and_grad, x0, maxiter=15000, ftol=None, gtol=None, gradient_max_norm=1e6, max_retries=3,
                   m=10, callback=None):
    """The minimisation block of ``Inv_4Dvar`` (inv.py:280-400) for a batch of
    windows: ``cost_and_grad(x) -> (J [B], G)`` with x shaped like ``x0``
    ([B, ...]).

    ``gtol`` is relative to the largest gradient component at X = 0, as the
    reference sets it; ``ftol`` is scipy's relative reduction. A window whose
    cost or gradient turns non-finite, or whose gradient exceeds
    ``gradient_max_norm``, stops and restarts from its best state with a
    fresh memory (at most ``max_retries`` times), as the reference's
    ``CrazyGradient`` handling does; after the last retry its best state is
    the result. Returns the dict of :class:`BatchedLBFGS` plus ``retries``."""
    x0 = torch.as_tensor(x0, dtype=torch.float64, device="cuda")
    B = x0.shape[0]
    n = x0[0].numel()
    opts = {}
    if ftol is not None:
        opts["ftol"] = ftol
    if gtol is not None:
        _, g0 = cost_and_grad(torch.zeros_like(x0))
        opts["gtol"] = gtol * torch.amax(torch.abs(g0.to(torch.float64).reshape(B, n)), dim=1).cpu().numpy()
    best = {"f": np.full(B, np.inf), "x": x0.reshape(B, n).clone()}

    def fun(x):
        J, G = cost_and_grad(x.reshape(x0.shape))
        J = np.asarray(J.detach().cpu().numpy() if torch.is_tensor(J) else J, dtype=np.float64).reshape(B)
        G = G.to(torch.float64).reshape(B, n)
        gnorm = torch.amax(torch.abs(G), dim=1).cpu().numpy()
        ok = np.isfinite(J) & np.isfinite(gnorm) & (gnorm < gradient_max_norm)
        better = ok & (J < best["f"])
        if np.any(better):
            best["x"] = torch.where(torch.as_tensor(better, device=x.device)[:, None], x, best["x"])
            best["f"] = np.where(better, J, best["f"])
        return J, G, ~ok

    x = x0.reshape(B, n).clone()
    active = np.ones(B, dtype=bool)
    retries = np.zeros(B, dtype=np.int64)
    final = None
    while True:
        res = BatchedLBFGS(fun, B, n, m=m, maxiter=maxiter, callback=callback, **opts).minimize(x, active)
        if final is None:
            final = {k: (v.clone() if torch.is_tensor(v) else (list(v) if isinstance(v, list) else np.array(v)))
                     for k, v in res.items()}
        else:
            sel = torch.as_tensor(active, device=x.device)[:, None]
            for k in ("x", "jac"):
                final[k] = torch.where(sel, res[k], final[k])
            for k in ("fun", "nit", "nfev", "status"):
                final[k] = np.where(active, res[k], final[k])
            final["message"] = [res["message"][b] if active[b] else final["message"][b] for b in range(B)]
        crazy = active & (res["status"] == 3)
        if not np.any(crazy):
            break
        again = crazy & (retries < max_retries)
        gone = crazy & ~again
        if np.any(gone):
            sel = torch.as_tensor(gone, device=x.device)[:, None]
            final["x"] = torch.where(sel, best["x"], final["x"])
            final["fun"] = np.where(gone, best["f"], final["fun"])
            for b in np.nonzero(gone)[0]:
                final["message"][b] = "STOP: MAXIMUM RETRIES AFTER CRAZY GRADIENTS (best state returned)"
        if not np.any(again):
            break
        retries[again] += 1
        x = torch.where(torch.as_tensor(again, device=x.device)[:, None], best["x"], final["x"])
        active = again
    final["retries"] = retries
    final["x"] = final["x"].reshape(x0.shape)
    return final
