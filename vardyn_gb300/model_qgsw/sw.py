"""Drop-in multilayer shallow-water model class backed by the GB300 kernels.

``SW(param)`` keeps the constructor, attributes and methods of the
reference's mapping/models/model_qgsw/sw.py (SW, 68-1035) that its callers
use: ``step``, ``step_tgl``, ``step_adj`` (returning ``((adu0, adv0, adh0,
adH, adh_wind),)`` like the reference's jax.vjp), ``set_input_uvh``,
``get_physical_uvh``, ``compute_time_derivatives``, ``masks`` and the sponge
arrays ``sponge_u`` / ``sponge_v`` / ``sponge_h`` (assignable after
construction, as mod.py:2803-2806 does). Arrays may be NumPy (returned as
NumPy) or CUDA torch tensors (returned as tensors) of shape
``(n_ens, nl, x, y)``.

``step`` / ``step_adj`` take the reference's ``H`` (a perturbation added to
every layer's thickness) and ``h_wind`` (added to the model's mixed-layer
depth); ``step_adj`` returns their cotangents, summed to the shapes they were
given in.

The spectral barotropic filter (``barotropic_filter`` with
``barotropic_filter_spectral``, ``SW`` only: sw.py:305-320, 720-750) runs in
every right-hand side of the step, its tangent and its adjoint.

Not supported (they raise): the filter's exact form (its multigrid solve is
work in progress in the reference, sw.py:321-333, 736-743) and its spectral
form with land (the reference's Neumann solver does not construct then,
helmholtz.py:254). Open boundaries (``flag_obc``, sw.py:353-371) open the
outer face masks; the boundary arrays the reference allocates there are
never read, and are not kept.
"""
import numpy as np
import torch

from vardyn_gb300.sw import SWPlan


def _torch_dtype(dt):
    if dt is None:
        return torch.float64
    if isinstance(dt, torch.dtype):
        return dt
    return torch.float64 if "64" in str(np.dtype(dt) if not isinstance(dt, str) else dt) else torch.float32


class _Masks4:
    """The reference's Masks attribute shapes: (1, 1, x, y)."""

    def __init__(self, m):
        for name, val in vars(m).items():
            if isinstance(val, np.ndarray) and val.ndim == 2:
                setattr(self, name, val[None, None])
        self.psi_irrbound_xids = m.psi_irrbound_xids
        self.psi_irrbound_yids = m.psi_irrbound_yids


class SW:
    """SW(param) of sw.py:103-383."""

    _plan_cls = SWPlan

    def __init__(self, param):
        p = dict(param)
        self.param = p
        self.nx, self.ny, self.nl = int(p["nx"]), int(p["ny"]), int(p["nl"])
        self.dtype = _torch_dtype(p.get("dtype"))
        self.barotropic_filter = False
        if p.get("barotropic_filter", False) and type(self).__name__ == "SW":
            if not p.get("barotropic_filter_spectral", False):
                raise NotImplementedError("the barotropic filter's exact form is work in progress in the "
                                          "reference (sw.py:321-333)")
            if p.get("mask") is not None and np.any(np.asarray(p["mask"], dtype=np.float64) < 0.5):
                raise NotImplementedError("the spectral barotropic filter with land: the reference's Neumann "
                                          "solver does not construct (helmholtz.py:254)")
            self.barotropic_filter = True
        H = np.asarray(p["H"], dtype=np.float64)
        if H.ndim < 3:
            raise ValueError(f"H must be a nl x nx x ny array with unit axes for constant directions, got {H.shape}")
        self.H = H
        self.dt = float(p["dt"])
        if self.barotropic_filter:
            # tau, H_tot and lambd of sw.py:312-317, from the model's own H
            self.tau = 2 * self.dt
            self.g = float(np.asarray(p["g_prime"], dtype=np.float64).reshape(-1)[0])
            self.H_tot = H.sum(axis=-3, keepdims=True)
            self.lambd = 1.0 / (self.g * self.dt * self.tau * self.H_tot)
        self.n_ens = int(p.get("n_ens", 1))
        nx, ny = self.nx, self.ny
        self._sponge = {"u": None, "v": None, "h": None}
        self._plans = {}
        self.slip_coef = float(p.get("slip_coef", 1.0))
        self.g_prime = np.asarray(p["g_prime"], dtype=np.float64).reshape(-1, 1, 1)
        self.f = np.asarray(p["f"], dtype=np.float64)[None]
        self.f0 = float(self.f.mean())
        self._base = self._make_plan(None)
        self.masks = _Masks4(self._base.masks)
        self.dx = np.asarray(p["dx"], dtype=np.float64)
        self.dy = np.asarray(p["dy"], dtype=np.float64)
        self.taux, self.tauy = p["taux"], p["tauy"]
        self.forcing_momentum = p.get("forcing_momentum", "direct")
        self.sponge_coef = float(p.get("sponge_coef", 0.0) or 0.0)

    # ---------------- plans ----------------
    def _plan_kwargs(self):
        p = self.param
        nx, ny = self.nx, self.ny
        return dict(mask=p.get("mask"), slip_coef=p.get("slip_coef", 1.0),
                    bottom_drag_coef=p.get("bottom_drag_coef", 0.0), rho_water=p.get("rho_water", 1025.0),
                    h_min=p.get("h_min", 0.1), h_min_sharpness=p.get("h_min_sharpness", 10.0),
                    visc_coef=p.get("visc_coef", 0.0) or 0.0, diff_coef=p.get("diff_coef", 0.0) or 0.0,
                    sponge_coef=p.get("sponge_coef", 0.0) or 0.0, flag_linear=p.get("flag_linear", False),
                    forcing_momentum=p.get("forcing_momentum", "direct"), h_wind=p.get("h_wind", None),
                    taux=p["taux"], tauy=p["tauy"],
                    sponge_u=self._sponge["u"], sponge_v=self._sponge["v"], sponge_h=self._sponge["h"],
                    dtype=self.dtype, barotropic_filter=self.barotropic_filter,
                    flag_obc=bool(p.get("flag_obc", False)),
                    bf_lambd=self.lambd if self.barotropic_filter else None)

    def _make_plan(self, H, h_wind=None):
        p = self.param
        kw = self._plan_kwargs()
        if H is not None:
            # the wind depth stays the model's own (sw.py:622-630)
            kw["H_wind"] = self.H
        if h_wind is not None:
            base = kw["h_wind"]
            kw["h_wind"] = np.asarray(h_wind, dtype=np.float64) + (0.0 if base is None else np.asarray(base))
        Ht = self.H if H is None else self.H + np.asarray(H, dtype=np.float64)
        return self._plan_cls(self.nx, self.ny, self.nl, p["dx"], p["dy"], p["f"], Ht, p["g_prime"], p["dt"], **kw)

    def _plan(self, H=None, h_wind=None):
        if H is None and h_wind is None:
            return self._base
        key = tuple(None if a is None else (np.shape(a), np.asarray(a, dtype=np.float64).tobytes())
                    for a in (H, h_wind))
        pl = self._plans.get(key)
        if pl is None:
            if len(self._plans) > 4:
                self._plans.clear()
            pl = self._plans[key] = self._make_plan(H, h_wind)
        return pl

    @staticmethod
    def _host(a):
        return None if a is None else (a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a))

    @staticmethod
    def _sum_to(a, shape):
        """Sum a [nl, nx, ny] cotangent down to the broadcast shape of its input."""
        shape = tuple(shape)
        while a.dim() > len(shape):
            a = a.sum(0)
        for d in range(a.dim()):
            if shape[d] == 1 and a.shape[d] != 1:
                a = a.sum(d, keepdim=True)
        return a.reshape(shape)

    def _rebuild(self):
        self._plans.clear()
        self._base = self._make_plan(None)

    def _sponge_prop(name):
        def get(self):
            v = self._sponge[name]
            shape = {"u": (self.nx + 1, self.ny), "v": (self.nx, self.ny + 1), "h": (self.nx, self.ny)}[name]
            return np.zeros((1, 1) + shape) if v is None else np.asarray(v).reshape((1, 1) + shape)

        def set_(self, val):
            self._sponge[name] = None if val is None else np.asarray(
                val.cpu() if torch.is_tensor(val) else val, dtype=np.float64).reshape(np.shape(val)[-2:])
            self._rebuild()
        return property(get, set_)

    sponge_u = _sponge_prop("u")
    sponge_v = _sponge_prop("v")
    sponge_h = _sponge_prop("h")

    # ---------------- conversions ----------------
    def _swplan(self):
        """The shallow-water plan (the QG plan wraps one)."""
        return getattr(self._base, "sw", self._base)

    def _in(self, x):
        if x is None:
            return None
        if torch.is_tensor(x):
            return x.to(device="cuda", dtype=self.dtype)
        return torch.as_tensor(np.asarray(x), dtype=self.dtype, device="cuda")

    @staticmethod
    def _out(like, x):
        return x if torch.is_tensor(like) else x.cpu().numpy()

    def _tau(self, taux, tauy):
        return self._in(taux) if taux is not None else None, self._in(tauy) if tauy is not None else None


    # ---------------- API ----------------
    def set_input_uvh(self, u_phys, v_phys, h_phys):
        """sw.py:432-450: mask and multiply by the metric terms."""
        pl = self._swplan()
        x = [self._in(a) for a in (u_phys, v_phys, h_phys)]
        B = pl._batch(x[0])
        x = pl._uvh(*x, B)
        out = tuple(torch.empty_like(a) for a in x)
        pl.scale(B, False, x, out)
        return tuple(self._out(u_phys, a) for a in out)

    def get_physical_uvh(self, u, v, h, numpy=False):
        """sw.py:421-427."""
        pl = self._swplan()
        x = [self._in(a) for a in (u, v, h)]
        B = pl._batch(x[0])
        x = pl._uvh(*x, B)
        out = tuple(torch.empty_like(a) for a in x)
        pl.scale(B, True, x, out)
        return tuple(a.cpu().numpy() for a in out) if numpy else tuple(self._out(u, a) for a in out)

    def compute_time_derivatives(self, u, v, h, ref_vals=None, taux=None, tauy=None, h_wind=None):
        """sw.py:720-750 of model-space fields; ``ref_vals`` from a perturbed H
        are not supported (pass H to :meth:`step` instead)."""
        if ref_vals is not None:
            raise NotImplementedError("ref_vals: pass the H perturbation to step()")
        pl = self._plan(None, self._host(h_wind))
        r = pl.rhs(self._in(u), self._in(v), self._in(h), *self._tau(taux, tauy))
        return tuple(self._out(u, a) for a in r)

    def step(self, u0, v0, h0, H=None, nstep=1, u_b=None, v_b=None, h_b=None, Fu=None, Fv=None, Fh=None, taux=None,
             tauy=None, h_wind=None):
        """sw.py:752-904."""
        pl = self._plan(self._host(H), self._host(h_wind))
        if (u_b is None) != (v_b is None) or (u_b is None) != (h_b is None):
            # a missing boundary field defaults to the initial state (sw.py:787-791)
            u_b = u0 if u_b is None else u_b
            v_b = v0 if v_b is None else v_b
            h_b = h0 if h_b is None else h_b
        tx, ty = self._tau(taux, tauy)
        r = pl.step(self._in(u0), self._in(v0), self._in(h0), nstep=nstep, ub=self._in(u_b), vb=self._in(v_b),
                    hb=self._in(h_b), Fu=self._in(Fu), Fv=self._in(Fv), Fh=self._in(Fh), taux=tx, tauy=ty)
        return tuple(self._out(u0, a) for a in r)

    def step_tgl(self, u0, v0, h0, du0, dv0, dh0, H=None, dH=None, nstep=1, taux=None, tauy=None, h_wind=None,
                 dh_wind=None):
        """jax.jvp of step in (u0, v0, h0, H, h_wind) (sw.py:906-922)."""
        pl = self._plan(self._host(H), self._host(h_wind))
        tx, ty = self._tau(taux, tauy)
        r = pl.step_tgl(self._in(u0), self._in(v0), self._in(h0), self._in(du0), self._in(dv0), self._in(dh0),
                        nstep=nstep, taux=tx, tauy=ty, dH=self._host(dH), dh_wind=self._host(dh_wind))
        return tuple(self._out(du0, a) for a in r)

    def step_adj(self, u0, v0, h0, wuT, wvT, whT, H=None, nstep=1, taux=None, tauy=None, h_wind=None):
        """jax.vjp of step (sw.py:924-938): ((adu0, adv0, adh0, adH, adh_wind),),
        adH / adh_wind None when H / h_wind is None (no cotangent for an
        absent input), else summed to the shape they were given in."""
        Hh, hw = self._host(H), self._host(h_wind)
        pl = self._plan(Hh, hw)
        tx, ty = self._tau(taux, tauy)
        want = Hh is not None or hw is not None
        a = pl.step_adj(self._in(u0), self._in(v0), self._in(h0), self._in(wuT), self._in(wvT), self._in(whT),
                        nstep=nstep, taux=tx, tauy=ty, **({"want_ref": True} if want else {}))
        adH = None if Hh is None else self._out(H, self._sum_to(a["H"], np.shape(Hh)))
        adhw = None if hw is None else self._out(h_wind, self._sum_to(a["h_wind"], np.shape(hw)))
        return ((self._out(wuT, a["u0"]), self._out(wvT, a["v0"]), self._out(whT, a["h0"]), adH, adhw),)

    def adjoint_test_sw(self, nstep=1, seed=42):
        """<M dx, y> / <dx, M* y> in float64 sums (sw.py:940-1035), with
        NumPy random vectors of amplitude 1e-4 masked to the ocean."""
        rng = np.random.default_rng(seed)
        n, nl, nx, ny = self.n_ens, self.nl, self.nx, self.ny
        shapes = [(n, nl, nx + 1, ny), (n, nl, nx, ny + 1), (n, nl, nx, ny)]
        ms = [self.masks.u, self.masks.v, self.masks.h]
        r = lambda: [torch.as_tensor(rng.standard_normal(s) * 1e-4 * m, dtype=self.dtype, device="cuda")
                     for s, m in zip(shapes, ms)]
        x0, dx, w = r(), r(), r()
        d1 = self.step_tgl(*x0, *dx, nstep=nstep)
        a0 = self.step_adj(*x0, *w, nstep=nstep)[0][:3]
        ps1 = sum(float((a.double() * b.double()).sum()) for a, b in zip(d1, w))
        ps2 = sum(float((a.double() * b.double()).sum()) for a, b in zip(dx, a0))
        return ps1 / ps2
