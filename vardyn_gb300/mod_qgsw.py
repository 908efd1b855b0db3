"""Drop-in for the reference's multilayer SW / QG model wrapper
``Model_qgsw`` (mapping/src/mod.py:2412-3617) on the GPU.

Same constructor ``Model_qgsw(config, State)`` and the hot-path methods
``init``, ``set_bc``, ``step(State, nstep, t)``, ``step_tgl(dState, State,
nstep, t)`` and ``step_adj(adState, State, nstep, t)`` with the reference's
State conventions:

- one layer: ``State.var`` U (ny, nx+1), V (ny+1, nx), SSH (ny, nx);
- several layers: ``u_layers`` / ``v_layers`` / ``h_layers`` with the surface
  diagnostics SSH = sum of layers, U / V = layer 0 (mod.py:3011-3023), and
  the adjoint folding the surface adjoints into the layers (mod.py:3458-3482);
- forcing ``State.params`` U / V / SSH in units per day, into layer 0
  (mod.py:3180-3196); boundary fields of ``set_bc`` / ``_apply_bc`` (nearest
  time, mod.py:3041-3087) plus the optional ``bc`` control parameters; the MDT
  added before and removed after a chunk (mod.py:3162-3172, 3206-3215);
- sub-stepping by ``max_nstep`` chunks, with the boundary fields and the wind
  stress held per chunk exactly as the reference does.

Inputs that need NetCDF files or the reference's grid utilities (MDT file,
Rossby-radius file, wind file, GRID_FROM_FILE initial state, sponge widths
from ``dist_sponge_bc``) are not read here: pass ``mdt=(mdt, mdu, mdv)``,
``sponge=(sponge_u, sponge_v, sponge_h)`` (State convention) or
``wind=(taux_wind, tauy_wind, wind_dt)`` instead. ``H`` and ``h_wind`` as
control parameters are not supported (they raise).
"""
from datetime import timedelta

import numpy as np
import torch

from vardyn_gb300.model_qgsw.qg import QG
from vardyn_gb300.model_qgsw.sw import SW


def _np(a):
    return a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)


class Model_qgsw:
    """Model_qgsw(config, State) of mod.py:2414-2834."""

    def __init__(self, config, State, sponge=None, mdt=None, wind=None, dtype=None):
        MOD, EXP = config.MOD, config.EXP
        # base class M (mod.py:83-113)
        self.ny, self.nx = State.ny, State.nx
        self.name_var = MOD.name_var
        self.dtype = dtype if dtype is not None else (
            torch.float64 if getattr(MOD, "dtype", "float64") in ("float64", np.float64, torch.float64)
            else torch.float32)
        self.nl = MOD.nl
        name_class = str(MOD.name_class).lower()
        ny, nx = self.ny, self.nx
        # Coriolis (mod.py:2451-2461)
        if getattr(MOD, "f0", None) is not None and getattr(MOD, "constant_f", False):
            self.f = MOD.f0 * np.ones((ny, nx))
        else:
            self.f = np.array(State.f, dtype=np.float64)
            self.f[np.isnan(self.f)] = np.nanmean(self.f)
        self.g = 9.81
        for key in ("path_mdt", "filec_aux", "path_wind"):
            path = getattr(MOD, key, None)
            if path is not None:
                raise NotImplementedError(f"config.MOD.{key}: pass the arrays to Model_qgsw instead of a file")
        self.c = MOD.c0 * np.ones((ny, nx))
        # reduced gravity and layer thickness (mod.py:2572-2617)
        if MOD.nl == 1:
            gp = MOD.g_prime
            if gp is None:
                g_prime = np.array([[[9.81]]])
            else:
                g_prime = np.asarray(gp, dtype=np.float64)
                g_prime = g_prime.reshape((1,) * (3 - g_prime.ndim) + g_prime.shape)
            if MOD.H is None:
                H = np.expand_dims(self.c.T ** 2 / g_prime[0, 0, 0], axis=0)
                H0 = np.array([[[np.nanmean(self.c) ** 2 / g_prime[0, 0, 0]]]])
                H[np.isnan(H)] = 0.
                if name_class == "qg":
                    H = H0
            else:
                H = np.asarray(MOD.H, dtype=np.float64)
                H = H.reshape((1,) * (3 - H.ndim) + H.shape)
        else:
            g_prime = np.asarray(MOD.g_prime, dtype=np.float64)
            if g_prime.ndim == 1:
                g_prime = g_prime.reshape(-1, 1, 1)
            H = np.asarray(MOD.H, dtype=np.float64)
            if H.ndim == 1:
                H = H.reshape(-1, 1, 1)
            elif H.ndim == 2:
                H = H[None]
        self.H0 = H
        # time step (mod.py:2622-2649)
        self.dt = MOD.dtmodel
        if getattr(MOD, "cfl", None) is not None:
            spacing = min(np.nanmin(State.DX), np.nanmin(State.DY))
            if self.nl > 1:
                c_max = float(np.sqrt(np.asarray(MOD.g_prime)[0] * np.asarray(MOD.H).sum()))
            else:
                c_max = float(np.nanmax(self.c))
            dt = MOD.cfl * spacing / c_max
            self.dt = max(d for d in range(1, 3601) if 3600 % d == 0 and d <= dt)
        if self.dt > 0:
            self.nt = 1 + int((EXP.final_date - EXP.init_date).total_seconds() // self.dt)
            ts, t = [], EXP.init_date
            while t <= EXP.final_date:
                ts.append(t)
                t += timedelta(seconds=self.dt)
            self.timestamps = np.asarray(ts)
        else:
            self.nt = 1
            self.timestamps = np.array([EXP.init_date])
        self.T = np.arange(self.nt) * self.dt
        # State initialisation (mod.py:2652-2688)
        if getattr(config, "GRID", None) is not None and getattr(config.GRID, "super", None) == "GRID_FROM_FILE":
            raise NotImplementedError("GRID_FROM_FILE initial state: set State.var before stepping")
        for name in self.name_var:
            shape = {"U": (ny, nx + 1), "V": (ny + 1, nx), "SSH": (ny, nx)}.get(name)
            if shape is not None:
                State.var[self.name_var[name]] = np.zeros(shape)
        if self.nl > 1:
            State.var["u_layers"] = np.zeros((self.nl, ny, nx + 1))
            State.var["v_layers"] = np.zeros((self.nl, ny + 1, nx))
            State.var["h_layers"] = np.zeros((self.nl, ny, nx))
        self.bc = {k: {} for k in self.name_var}
        self.forcing = {k: {} for k in self.name_var}
        self.init_from_bc = getattr(MOD, "init_from_bc", None)
        self.bc_time = np.array([])
        # sponge (mod.py:2696-2768): weights passed in, State convention
        if sponge is None and getattr(MOD, "dist_sponge_bc", None):
            raise NotImplementedError("dist_sponge_bc: pass sponge=(sponge_u, sponge_v, sponge_h)")
        if sponge is None:
            sponge = (np.zeros((ny, nx + 1)), np.zeros((ny + 1, nx)), np.zeros((ny, nx)))
        self.sponge_u, self.sponge_v, self.sponge_h = (np.asarray(a, dtype=np.float64) for a in sponge)
        self.sponge_coef = getattr(MOD, "sponge_coef", 0.0)
        # model (mod.py:2771-2806)
        params = {
            "nx": nx, "ny": ny, "nl": MOD.nl, "dx": np.asarray(State.DX).T, "dy": np.asarray(State.DY).T,
            "H": H, "g_prime": g_prime, "f": np.pad(self.f.T, ((0, 1), (0, 1)), mode="edge"),
            "taux": 0., "tauy": 0., "bottom_drag_coef": MOD.bottom_drag_coef,
            "rho_water": getattr(MOD, "rho_water", 1025.0), "h_wind": getattr(MOD, "h_wind", None),
            "dtype": self.dtype, "mask": (1 - np.asarray(State.mask).astype(int).T),
            "slip_coef": MOD.slip_coef, "visc_coef": MOD.visc_coef, "diff_coef": MOD.diff_coef, "dt": self.dt,
            "barotropic_filter": False, "sponge_coef": self.sponge_coef,
            "forcing_momentum": getattr(MOD, "forcing_momentum", "direct"),
        }
        self.model = (QG if name_class == "qg" else SW)(params)
        self.model.sponge_u = self.sponge_u.T
        self.model.sponge_v = self.sponge_v.T
        self.model.sponge_h = self.sponge_h.T
        self.max_nstep = getattr(MOD, "max_nstep", 240)
        self.name_params = list(getattr(MOD, "name_params", None) or [])
        # bathymetry / layer-thickness and mixed-layer-depth controls start at
        # zero perturbation (mod.py:2829-2842; a file's H is passed as an array)
        if "H" in self.name_params and "H" not in State.params:
            State.params["H"] = np.zeros((ny, nx))
        if "h_wind" in self.name_params:
            State.params["h_wind"] = np.zeros((ny, nx))
        if "bc" in self.name_params:
            State.params["u_b"] = np.zeros((ny, nx + 1))
            State.params["v_b"] = np.zeros((ny + 1, nx))
            State.params["h_b"] = np.zeros((ny, nx))
        for name in self.name_var:
            State.params[self.name_var[name]] = np.zeros_like(_np(State.var[self.name_var[name]]))
        # wind stress arrays at wind_dt spacing, State convention (mod.py:2836-2969)
        self.taux_wind = self.tauy_wind = None
        self.wind_dt = 0
        if wind is not None:
            self.taux_wind, self.tauy_wind, self.wind_dt = np.asarray(wind[0]), np.asarray(wind[1]), float(wind[2])
        if mdt is not None:
            mdt, mdu, mdv = (np.asarray(a, dtype=np.float64) for a in mdt)
            self.mdt, self.mdu, self.mdv = mdt.T[None, None], mdu.T[None, None], mdv.T[None, None]
        else:
            self.mdt = self.mdu = self.mdv = None

    # ---------------- boundary conditions ----------------
    def init(self, State, t0=0):
        """mod.py:3025-3044."""
        if isinstance(self.init_from_bc, dict):
            if "SSH" in self.init_from_bc:
                for k in ("U", "V", "SSH"):
                    State.setvar(self.bc[k][t0], self.name_var[k])
            for name in self.init_from_bc:
                if self.init_from_bc[name] and t0 in self.bc[name]:
                    State.setvar(self.bc[name][t0], self.name_var[name])
        elif self.init_from_bc:
            for name in self.name_var:
                if t0 in self.bc[name]:
                    State.setvar(self.bc[name][t0], self.name_var[name])
        if self.nl > 1:
            self._sync_layers_from_surface(State)

    def set_bc(self, time_bc, var_bc):
        """mod.py:3060-3086."""
        for i, t in enumerate(time_bc):
            ssh = np.array(var_bc["SSH"][i], dtype=np.float64)
            ssh[np.isnan(ssh)] = 0.
            if "U" not in var_bc or "V" not in var_bc:
                u, v = np.zeros((self.ny, self.nx + 1)), np.zeros((self.ny + 1, self.nx))
            else:
                u, v = np.array(var_bc["U"][i], dtype=np.float64), np.array(var_bc["V"][i], dtype=np.float64)
                u[np.isnan(u)] = 0.
                v[np.isnan(v)] = 0.
            self.bc["U"][t], self.bc["V"][t], self.bc["SSH"][t] = u, v, ssh
        self.bc_time = np.asarray(time_bc)

    def _apply_bc(self, t0, t1):
        """mod.py:3088-3106: boundary fields of the nearest time."""
        zero = (np.zeros((self.ny, self.nx + 1)), np.zeros((self.ny + 1, self.nx)), np.zeros((self.ny, self.nx)))
        if "SSH" not in self.bc or len(self.bc["SSH"]) == 0:
            return zero
        if t0 not in self.bc_time:
            t0 = self.bc_time[np.argmin(np.abs(self.bc_time - t0))]
        return self.bc["U"][t0], self.bc["V"][t0], self.bc["SSH"][t0]

    def _get_wind_stress(self, t):
        """mod.py:2971-2983."""
        if self.taux_wind is None:
            return None, None
        it = int(round(t / self.wind_dt)) if self.wind_dt > 0 else 0
        it = int(np.clip(it, 0, len(self.taux_wind) - 1))
        return (1 - self.sponge_u) * self.taux_wind[it], (1 - self.sponge_v) * self.tauy_wind[it]

    def _sync_layers_from_surface(self, State):
        """mod.py:2985-2993."""
        ssh = _np(State.getvar(name_var=self.name_var["SSH"]))
        u = _np(State.getvar(name_var=self.name_var["U"]))
        v = _np(State.getvar(name_var=self.name_var["V"]))
        hl = np.zeros((self.nl, self.ny, self.nx)); hl[0] = ssh
        ul = np.zeros((self.nl, self.ny, self.nx + 1)); ul[0] = u
        vl = np.zeros((self.nl, self.ny + 1, self.nx)); vl[0] = v
        State.var["h_layers"], State.var["u_layers"], State.var["v_layers"] = hl, ul, vl

    def _diagnose_surface(self, State):
        State.setvar(_np(State.var["h_layers"]).sum(axis=0), name_var=self.name_var["SSH"])
        State.setvar(_np(State.var["u_layers"])[0], name_var=self.name_var["U"])
        State.setvar(_np(State.var["v_layers"])[0], name_var=self.name_var["V"])

    # ---------------- conversions ----------------
    def _t(self, a):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=self.dtype, device="cuda")

    def _state_in(self, S, adjoint_surface=False):
        """State -> model arrays (1, nl, x, y)."""
        if self.nl > 1:
            u = _np(S.var["u_layers"]).transpose(0, 2, 1)[None]
            v = _np(S.var["v_layers"]).transpose(0, 2, 1)[None]
            h = _np(S.var["h_layers"]).transpose(0, 2, 1)[None]
        else:
            u = _np(S.getvar(name_var=self.name_var["U"])).T[None, None]
            v = _np(S.getvar(name_var=self.name_var["V"])).T[None, None]
            h = _np(S.getvar(name_var=self.name_var["SSH"])).T[None, None]
        return self._t(u), self._t(v), self._t(h)

    def _layer0(self, a2d, scale=1.0, shape=None):
        """2-D State field -> (1, nl, x, y) with the field in layer 0."""
        a = _np(a2d).T * scale
        out = np.zeros((1, self.nl) + a.shape)
        out[0, 0] = a
        return self._t(out)

    def _forcing(self, S):
        return tuple(self._layer0(S.params[self.name_var[k]], 1.0 / (3600 * 24)) for k in ("U", "V", "SSH"))

    def _bc(self, S, t_chunk, n_chunk):
        ub, vb, hb = self._apply_bc(t_chunk, int(t_chunk + n_chunk * self.dt))
        if "bc" in self.name_params:
            ub = ub + _np(S.params["u_b"])
            vb = vb + _np(S.params["v_b"])
            hb = hb + _np(S.params["h_b"])
        return self._layer0(ub), self._layer0(vb), self._layer0(hb)

    def _wind(self, t_chunk):
        tx, ty = self._get_wind_stress(t_chunk)
        if tx is None:
            return None, None
        return self._t(np.asarray(tx)[:, 1:-1].T), self._t(np.asarray(ty)[1:-1, :].T)

    def _chunks(self, nstep, t):
        out, done = [], 0
        while done < nstep:
            n = min(nstep - done, self.max_nstep) if self.max_nstep > 0 else nstep - done
            out.append((t + done * self.dt, n))
            done += n
        return out

    def _ref_params(self, S):
        """The H (1, nx, ny) and h_wind (nx, ny) perturbations of State S
        (mod.py:3311-3320), or None."""
        H = np.asarray(_np(S.params["H"]), dtype=np.float64).T[None] if "H" in self.name_params else None
        hw = np.asarray(_np(S.params["h_wind"]), dtype=np.float64).T if "h_wind" in self.name_params else None
        return H, hw

    def _plan(self, S=None):
        if S is None:
            return self.model._base
        return self.model._plan(*self._ref_params(S))

    def _mdt(self, x, sign):
        if self.mdt is None:
            return x
        u, v, h = x
        add = [self._t(a) for a in (self.mdu, self.mdv, self.mdt)]
        u, v, h = u.clone(), v.clone(), h.clone()
        for f, a in zip((u, v, h), add):
            f[:, 0:1] += sign * a
        return u, v, h

    def _state_out(self, S, x):
        u, v, h = (a.cpu().numpy() for a in x)
        if self.nl > 1:
            S.var["h_layers"] = h[0].transpose(0, 2, 1)
            S.var["u_layers"] = u[0].transpose(0, 2, 1)
            S.var["v_layers"] = v[0].transpose(0, 2, 1)
            self._diagnose_surface(S)
        else:
            S.setvar(u[0, 0].T, name_var=self.name_var["U"])
            S.setvar(v[0, 0].T, name_var=self.name_var["V"])
            S.setvar(h[0, 0].T, name_var=self.name_var["SSH"])

    # ---------------- model ----------------
    def _fwd(self, x, S, t_chunk, n_chunk, F):
        pl = self._plan(S)
        ub, vb, hb = self._bc(S, t_chunk, n_chunk)
        tx, ty = self._wind(t_chunk)
        x = self._mdt(x, +1)
        x = pl.step(*x, nstep=n_chunk, ub=ub, vb=vb, hb=hb, Fu=F[0], Fv=F[1], Fh=F[2], taux=tx, tauy=ty)
        return self._mdt(x, -1)

    def step(self, State, nstep=1, t=0):
        """mod.py:3288-3346."""
        x = self._state_in(State)
        F = self._forcing(State)
        for t_chunk, n_chunk in self._chunks(nstep, t):
            x = self._fwd(x, State, t_chunk, n_chunk, F)
        self._state_out(State, x)

    def step_tgl(self, dState, State, nstep=1, t=0):
        """mod.py:3348-3453 (tangent of state, forcing, bc, H and h_wind
        parameters)."""
        pl = self._plan(State)
        dH, dhw = self._ref_params(dState)
        dref = {k: v for k, v in (("dH", dH), ("dh_wind", dhw)) if v is not None}
        x = self._state_in(State)
        dx = self._state_in(dState)
        F, dF = self._forcing(State), self._forcing(dState)
        for t_chunk, n_chunk in self._chunks(nstep, t):
            ub, vb, hb = self._bc(State, t_chunk, n_chunk)
            if "bc" in self.name_params:
                db = tuple(self._layer0(dState.params[k]) for k in ("u_b", "v_b", "h_b"))
            else:
                db = (None, None, None)
            tx, ty = self._wind(t_chunk)
            xm = self._mdt(x, +1)
            dx = pl.step_tgl(*xm, *dx, nstep=n_chunk, ub=ub, vb=vb, hb=hb, dub=db[0], dvb=db[1], dhb=db[2],
                             Fu=F[0], Fv=F[1], Fh=F[2], dFu=dF[0], dFv=dF[1], dFh=dF[2], taux=tx, tauy=ty,
                             **dref)
            x = self._fwd(x, State, t_chunk, n_chunk, F)
        du, dv, dh = (a.cpu().numpy() for a in dx)
        if self.nl > 1:
            dState.var["h_layers"] = dh[0].transpose(0, 2, 1)
            dState.var["u_layers"] = du[0].transpose(0, 2, 1)
            dState.var["v_layers"] = dv[0].transpose(0, 2, 1)
            dState.setvar(dState.var["h_layers"].sum(axis=0), name_var=self.name_var["SSH"])
            dState.setvar(dState.var["u_layers"][0], name_var=self.name_var["U"])
            dState.setvar(dState.var["v_layers"][0], name_var=self.name_var["V"])
        else:
            dState.setvar(du[0, 0].T, name_var=self.name_var["U"])
            dState.setvar(dv[0, 0].T, name_var=self.name_var["V"])
            dState.setvar(dh[0, 0].T, name_var=self.name_var["SSH"])

    def step_adj(self, adState, State, nstep=1, t=0):
        """mod.py:3455-3617: overwrites the state adjoint, accumulates the
        forcing (and bc, H, h_wind) parameter adjoints."""
        pl = self._plan(State)
        want_ref = "H" in self.name_params or "h_wind" in self.name_params
        adref = {k: np.array(_np(adState.params.get(k, np.zeros((self.ny, self.nx)))), dtype=np.float64)
                 for k in ("H", "h_wind") if k in self.name_params}
        ny, nx, nl = self.ny, self.nx, self.nl
        if nl > 1:
            ahs = _np(adState.getvar(name_var=self.name_var["SSH"]))
            aus = _np(adState.getvar(name_var=self.name_var["U"]))
            avs = _np(adState.getvar(name_var=self.name_var["V"]))
            ahl = np.array(_np(adState.var.get("h_layers", np.zeros((nl, ny, nx)))), dtype=np.float64)
            aul = np.array(_np(adState.var.get("u_layers", np.zeros((nl, ny, nx + 1)))), dtype=np.float64)
            avl = np.array(_np(adState.var.get("v_layers", np.zeros((nl, ny + 1, nx)))), dtype=np.float64)
            ahl = ahl + ahs[None]
            aul[0] += aus
            avl[0] += avs
            ad = tuple(self._t(a.transpose(0, 2, 1)[None]) for a in (aul, avl, ahl))
        else:
            ad = tuple(self._t(_np(adState.getvar(name_var=self.name_var[k])).T[None, None])
                       for k in ("U", "V", "SSH"))
        F = self._forcing(State)
        adF = [np.array(_np(adState.params[self.name_var[k]]), dtype=np.float64) for k in ("U", "V", "SSH")]
        bcp = "bc" in self.name_params
        adb = [np.array(_np(adState.params[k]), dtype=np.float64) for k in ("u_b", "v_b", "h_b")] if bcp else None
        chunks = self._chunks(nstep, t)
        states = [self._state_in(State)]
        for t_chunk, n_chunk in chunks[:-1]:
            states.append(self._fwd(states[-1], State, t_chunk, n_chunk, F))
        for i in range(len(chunks) - 1, -1, -1):
            t_chunk, n_chunk = chunks[i]
            ub, vb, hb = self._bc(State, t_chunk, n_chunk)
            tx, ty = self._wind(t_chunk)
            xm = self._mdt(states[i], +1)
            a = pl.step_adj(*xm, *ad, nstep=n_chunk, ub=ub, vb=vb, hb=hb, Fu=F[0], Fv=F[1], Fh=F[2], taux=tx,
                            tauy=ty, want_bc=True, want_forcing=True, **({"want_ref": True} if want_ref else {}))
            # H enters every layer as the same (1, nx, ny) perturbation
            if "H" in adref:
                adref["H"] += a["H"].sum(0).cpu().numpy().T
            if "h_wind" in adref:
                adref["h_wind"] += a["h_wind"].cpu().numpy().T
            ad = (a["u0"], a["v0"], a["h0"])
            for k, key in enumerate(("Fu", "Fv", "Fh")):
                adF[k] += a[key][0, 0].cpu().numpy().T / (3600 * 24)
            if bcp:
                for k, key in enumerate(("ub", "vb", "hb")):
                    adb[k] += a[key][0, 0].cpu().numpy().T
        au, av, ah = (x.cpu().numpy() for x in ad)
        if nl > 1:
            adState.var["h_layers"] = ah[0].transpose(0, 2, 1)
            adState.var["u_layers"] = au[0].transpose(0, 2, 1)
            adState.var["v_layers"] = av[0].transpose(0, 2, 1)
            adState.setvar(np.zeros((ny, nx)), self.name_var["SSH"])
            adState.setvar(np.zeros((ny, nx + 1)), self.name_var["U"])
            adState.setvar(np.zeros((ny + 1, nx)), self.name_var["V"])
        else:
            adState.setvar(au[0, 0].T, self.name_var["U"])
            adState.setvar(av[0, 0].T, self.name_var["V"])
            adState.setvar(ah[0, 0].T, self.name_var["SSH"])
        if bcp:
            adState.params["u_b"], adState.params["v_b"], adState.params["h_b"] = adb
        for k, key in enumerate(("U", "V", "SSH")):
            adState.params[self.name_var[key]] = adF[k]
        for k, val in adref.items():
            adState.params[k] = val
