"""4D-Var cost and gradient of QG 1.5-layer assimilation windows on the GPU.

Control: the initial SSH of each window. For ``B`` independent windows on the
same grid the engine computes, in one launch sequence per step,

    J_b(h0_b) = 1/2 * sum_k || inverr * (H_k M_{0->k}(h0_b) - y_k) ||^2 / sigma_R^2
    G_b = dJ_b/dh0_b

following Variational.cost_and_grad (mapping/src/tools_4Dvar.py:252-400):
forward sweep storing the model trajectory, misfits at observation steps
(obsop.py:610-628), Jo = misfit.R^-1.misfit (292), J = Jo/2 (326), then the
reverse sweep: model adjoint between observation steps and the observation
adjoint with the misfit as cotangent (391, obsop.py:668-678).

One difference from the reference's call structure, exact in real
arithmetic: the reference calls the model once per checkpoint interval and
every call re-derives PV from SSH (jqgm.py:536). Because the DST inversion
and h2pv are exact inverses on the points where PV evolves, the engine
integrates the (h, q) state continuously; the two agree to rounding (checked
against the oracle's chunked form in the tests).

Trajectory storage: ``full`` keeps every stage state of every step (the
"plain" form, memory 2*nstage fields per step); ``checkpoint=K`` keeps the
state every K steps and recomputes each K-step segment during the reverse
sweep (one extra forward, memory (nstep/K)*2 + 2*nstage*K fields).

``checkpoint=("revolve", slots, unit)`` keeps at most slots + 1 snapshots
and one unit's trajectory and follows a binomial schedule
(:func:`revolve_schedule`): the memory of a few fields for a bounded number
of recomputations, for windows or batches whose snapshots would not fit.

Float32 plans carry the prognostic PV as a compensated pair (q, q_lo): the
low part is one running field, saved with every snapshot so that a
recomputed segment repeats the forward sweep bit for bit.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .qg1l import QG1LPlan, SECONDS_PER_DAY


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def binomial_reach(slots, reps):
    """Units that a binomial schedule with ``slots`` free snapshot slots and
    at most ``reps`` forward repetitions of any unit can reverse:
    C(slots + reps, slots) (Griewank and Walther, Algorithm 799: revolve)."""
    return math.comb(slots + reps, slots)


def revolve_schedule(n_units, slots):
    """Binomial checkpointing schedule for reversing ``n_units`` time units
    with ``slots`` snapshot slots beyond the one holding the initial state.

    Returns a list of actions, executed in order:
      ("advance", a, b)  run units a .. b-1 forward from the current state
                         (no trajectory kept), leaving the state at unit b;
      ("save", b)        push the current state (at unit b) on the snapshot stack;
      ("restore", a)     make the snapshot on top of the stack (at unit a) the
                         current state (the snapshot stays);
      ("drop", a)        pop the snapshot at unit a;
      ("reverse", u)     run unit u forward keeping its trajectory, then its
                         adjoint (the current state is at unit u).
    The recursion splits [a, b) at m so that the right part, reversed with one
    slot fewer, holds at most binomial_reach(slots - 1, r) units and the left
    part, reversed after the right one frees its slot, at most
    binomial_reach(slots, r - 1), with r the smallest repetition count that
    reaches b - a; without free slots, every unit is recomputed from a."""
    acts = []

    def rev(a, b, free):
        n = b - a
        if n == 1:
            acts.append(("reverse", a))
            return
        if free == 0:
            for u in range(b - 1, a - 1, -1):
                if u > a:
                    acts.append(("advance", a, u))
                acts.append(("reverse", u))
                if u > a:
                    acts.append(("restore", a))
            return
        r = 1
        while binomial_reach(free, r) < n:
            r += 1
        right = max(1, min(n - 1, binomial_reach(free - 1, r)))
        m = b - right
        acts.append(("advance", a, m))
        acts.append(("save", m))
        rev(m, b, free - 1)
        acts.append(("drop", m))
        acts.append(("restore", a))
        rev(a, m, free)

    if n_units > 0:
        acts.append(("save", 0))
        rev(0, n_units, slots)
        acts.append(("drop", 0))
    return acts


class QGWindows4DVar:
    """Cost and gradient of ``B`` windows sharing one plan and one obs set."""

    def __init__(self, plan: QG1LPlan, hb, nstep, obs, sigma_R=1.0, checkpoint=None):
        self.plan = plan
        self.B = obs.B
        self.nstep = int(nstep)
        self.obs = obs
        self.sigma_R = float(sigma_R)
        self.hb = plan._as_batch(hb, "hb")
        if self.hb.shape[0] != self.B:
            raise ValueError("hb must have one field per window")
        B, ny, nx = self.B, plan.ny, plan.nx
        self.fs = ny * nx
        self.vd_dtype = _lib.VD_F64 if plan.dtype == torch.float64 else _lib.VD_F32
        dev, dt = plan.device, plan.dtype
        self.qb = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.qlo = plan.new_qlo(B)
        self.tmp = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.adh = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.adq = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.grad = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.J = torch.zeros(B, dtype=torch.float64, device=dev)
        self.obs_steps = sorted(int(s) for s in obs.steps if 0 <= s <= self.nstep)
        # h2pv(0, 0) == 0: with a zero background the solves skip the
        # subtraction of the background PV
        zero_bg = float(self.hb.abs().max()) == 0.0
        self.qb_arg = None if zero_bg else self.qb
        self.hb_arg = None if zero_bg else self.hb
        self.checkpoint = checkpoint
        S = plan.nstage
        self.revolve = isinstance(checkpoint, (tuple, list)) and len(checkpoint) == 3 and checkpoint[0] == "revolve"
        if self.revolve:
            # binomial schedule over units of `unit` steps with `slots`
            # snapshot slots (plus the initial state)
            _, slots, unit = checkpoint
            self.unit, self.slots = int(unit), int(slots)
            if self.unit < 1 or self.slots < 0:
                raise ValueError("revolve needs unit >= 1 and slots >= 0")
            self.nunit = math.ceil(self.nstep / self.unit)
            self.schedule = revolve_schedule(self.nunit, self.slots)
            self.traj = plan.new_traj(B, self.unit)
            self.traj_steps = self.unit
            self.stack = torch.zeros(self.slots + 1, 2 if self.qlo is None else 3, B, ny, nx, dtype=dt, device=dev)
            self.snap = None
        elif checkpoint is None:
            self.traj = plan.new_traj(B, self.nstep)
            self.traj_steps = self.nstep
            self.snap = None
        else:
            K = int(checkpoint)
            self.K = K
            self.nseg = math.ceil(self.nstep / K)
            # segment trajectory (K steps) + snapshots of (h, q) at segment starts
            self.traj = plan.new_traj(B, K)
            self.traj_steps = K
            self.snap = torch.zeros(self.nseg, 2 if self.qlo is None else 3, B, ny, nx, dtype=dt, device=dev)
        self.tv = self.traj.view(-1, 2, B, ny, nx)
        self.S = S
        self.graph = None

    # ------------------------------------------------------------------
    def memory_bytes(self):
        n = self.traj.numel() * self.traj.element_size()
        if self.snap is not None:
            n += self.snap.numel() * self.snap.element_size()
        if self.revolve:
            n += self.stack.numel() * self.stack.element_size()
        return n

    def recomputed_steps(self):
        """Forward steps the reverse sweep repeats (revolve: the schedule's
        advances plus the taping run of every unit; two-level: one more
        forward; full trajectory: none)."""
        if self.revolve:
            adv = sum(min(b * self.unit, self.nstep) - a * self.unit
                      for act, *ab in self.schedule if act == "advance" for a, b in [ab])
            return adv + self.nstep
        return 0 if self.snap is None else self.nstep

    def _copy(self, src, dst):
        _lib.call("vd_copy", self.vd_dtype, ctypes.c_longlong(src.numel()), _p(src), _p(dst), _stream())

    def _fill0(self, t):
        _lib.call("vd_fill", self.vd_dtype, ctypes.c_longlong(t.numel()), 0.0, _p(t), _stream())

    def _obs_forward(self, s, h_slot):
        if s not in self.obs.step_range:
            return
        if s == 0:
            self.obs.apply_misfit(s, h_slot)
        else:
            self.plan.finalize(self.B, h_slot, self.hb, self.tmp)
            self.obs.apply_misfit(s, self.tmp)

    # ------------------------------------------------------------------
    def _forward_full(self):
        p, B = self.plan, self.B
        prev = 0
        self._obs_forward(0, self.tv[0, 0])
        for s in self.obs_steps + [self.nstep]:
            if s <= prev:
                continue
            p.advance(B, self.traj, self.traj_steps, prev, s - prev, self.hb_arg, self.qb_arg, self.qlo)
            prev = s
            self._obs_forward(s, self.tv[s * self.S, 0])

    def _reverse_full(self):
        p, B = self.plan, self.B
        prev = self.nstep
        if self.nstep in self.obs.step_range:
            self.obs.apply_adjoint(self.nstep, self.adh)
        for s in sorted(self.obs_steps + [0], reverse=True):
            if s >= prev:
                continue
            p.advance_adj(B, self.traj, self.traj_steps, s, prev - s, self.adh, self.adq)
            prev = s
            if s in self.obs.step_range:
                self.obs.apply_adjoint(s, self.adh)

    def _forward_ckpt(self):
        """Forward keeping only segment-start snapshots."""
        p, B, K = self.plan, self.B, self.K
        self._obs_forward(0, self.tv[0, 0])
        for g in range(self.nseg):
            a = g * K
            n = min(K, self.nstep - a)
            self._copy(self.tv[0], self.snap[g, :2])
            if self.qlo is not None:
                self._copy(self.qlo, self.snap[g, 2])
            self._advance_segment(a, n, with_obs=True)
            self._copy(self.tv[n * self.S], self.tv[0])

    def _advance_segment(self, a, n, with_obs):
        p, B = self.plan, self.B
        local = [s - a for s in self.obs_steps if a < s <= a + n]
        prev = 0
        for ls in local + [n]:
            if ls <= prev:
                continue
            p.advance(B, self.traj, self.traj_steps, prev, ls - prev, self.hb_arg, self.qb_arg, self.qlo)
            prev = ls
            if with_obs:
                self._obs_forward(a + ls, self.tv[ls * self.S, 0])

    def _reverse_ckpt(self):
        p, B, K = self.plan, self.B, self.K
        if self.nstep in self.obs.step_range:
            self.obs.apply_adjoint(self.nstep, self.adh)
        for g in reversed(range(self.nseg)):
            a = g * K
            n = min(K, self.nstep - a)
            self._copy(self.snap[g, :2], self.tv[0])
            if self.qlo is not None:
                self._copy(self.snap[g, 2], self.qlo)
            self._advance_segment(a, n, with_obs=False)
            prev = n
            local = sorted([s - a for s in self.obs_steps if a <= s < a + n] + [0], reverse=True)
            for ls in local:
                if ls >= prev:
                    continue
                p.advance_adj(B, self.traj, self.traj_steps, ls, prev - ls, self.adh, self.adq)
                prev = ls
                if (a + ls) in self.obs.step_range:
                    self.obs.apply_adjoint(a + ls, self.adh)

    def _run_revolve(self):
        """Execute the binomial schedule: the first pass over a step computes
        its misfits (every step is first reached, in order, by the schedule's
        initial descent); later passes only recompute the trajectory."""
        p, B, L = self.plan, self.B, self.unit
        frontier = 0                  # steps whose misfits exist
        depth = 0

        def span(u):
            a = u * L
            return a, min(L, self.nstep - a)

        def copy_state(dst):
            self._copy(self.tv[0], dst[:2])
            if self.qlo is not None:
                self._copy(self.qlo, dst[2])

        def load_state(src):
            self._copy(src[:2], self.tv[0])
            if self.qlo is not None:
                self._copy(src[2], self.qlo)

        self._obs_forward(0, self.tv[0, 0])
        for act in self.schedule:
            kind = act[0]
            if kind == "advance":
                for u in range(act[1], act[2]):
                    a, n = span(u)
                    self._advance_segment(a, n, with_obs=a + n > frontier)
                    frontier = max(frontier, a + n)
                    self._copy(self.tv[n * self.S], self.tv[0])
            elif kind == "save":
                copy_state(self.stack[depth])
                depth += 1
            elif kind == "restore":
                load_state(self.stack[depth - 1])
            elif kind == "drop":
                depth -= 1
            else:                                     # reverse one unit
                u = act[1]
                a, n = span(u)
                self._advance_segment(a, n, with_obs=a + n > frontier)
                if a + n > frontier:
                    frontier = a + n
                    if a + n == self.nstep:
                        # the window's last misfits exist now: the cost and
                        # the final observation adjoint
                        self.obs.sumsq_per_window(self.J, 0.5 / self.sigma_R ** 2)
                        if self.nstep in self.obs.step_range:
                            self.obs.apply_adjoint(self.nstep, self.adh)
                prev = n
                local = sorted([s - a for s in self.obs_steps if a <= s < a + n] + [0], reverse=True)
                for ls in local:
                    if ls >= prev:
                        continue
                    p.advance_adj(B, self.traj, self.traj_steps, ls, prev - ls, self.adh, self.adq)
                    prev = ls
                    if (a + ls) in self.obs.step_range:
                        self.obs.apply_adjoint(a + ls, self.adh)

    # ------------------------------------------------------------------
    def _run(self, h0):
        """Enqueue one cost+gradient evaluation for the control ``h0`` [B, ny, nx]."""
        p, B = self.plan, self.B
        self._copy(h0, self.tv[0, 0])
        p.init_state(self.tv[0, 0], self.hb, self.tv[0, 1], self.qb, self.qlo)
        if self.revolve:
            self._fill0(self.adh)
            self._fill0(self.adq)
            self._run_revolve()
            p.init_state_adj(B, self.tv[0, 0], self.adq, self.adh)
            self._copy(self.adh, self.grad)
            return
        if self.snap is None:
            self._forward_full()
        else:
            self._forward_ckpt()
        self.obs.sumsq_per_window(self.J, 0.5 / self.sigma_R ** 2)
        self._fill0(self.adh)
        self._fill0(self.adq)
        if self.snap is None:
            self._reverse_full()
            h0_state = self.tv[0, 0]
        else:
            self._reverse_ckpt()
            self._copy(self.snap[0, :2], self.tv[0])
            h0_state = self.tv[0, 0]
        p.init_state_adj(B, h0_state, self.adq, self.adh)
        self._copy(self.adh, self.grad)

    def cost_and_grad(self, h0):
        """Returns (J [B] float64, grad [B, ny, nx]) as device tensors (views of
        internal buffers, overwritten by the next call)."""
        h0 = self.plan._as_batch(h0, "h0")
        if self.graph is not None:
            self._copy(h0, self.h0_static)
            self.graph.replay()
        else:
            self._run(h0)
        return self.J, self.grad

    def capture(self):
        """Capture one whole evaluation (forward + adjoint of the full window)
        into a CUDA graph; later cost_and_grad calls replay it."""
        B, ny, nx = self.B, self.plan.ny, self.plan.nx
        self.h0_static = torch.zeros(B, ny, nx, dtype=self.plan.dtype, device=self.plan.device)
        self._run(self.h0_static)          # warm-up: kernel attributes, allocator
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._run(self.h0_static)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = g
        return g


def checkpoints(nstep, nstep_check, obs_steps):
    """Model steps at which the cost function is evaluated
    (mapping/src/inv.py:144-163): step 0, every observation step, every
    nstep_check-th step, and the last step."""
    obs_steps = set(int(s) for s in obs_steps)
    cps, check = [0], 0
    for i in range(nstep):
        if i > 0 and (i in obs_steps or check == nstep_check):
            cps.append(i)
            if check == nstep_check:
                check = 0
        check += 1
    cps.append(nstep)
    return cps


class QGBasis4DVar:
    """Cost and gradient of ``B`` windows whose control is reduced-basis
    coefficients forcing the SSH (the reference's Inv_4Dvar with a basis,
    mapping/src/inv.py:142-215, tools_4Dvar.py:252-400).

    Forward, per checkpoint interval [c_i, c_{i+1}) of n_i steps
    (checkpoints of inv.py:144-163):
      misfit at c_i if observed;
      if c_i is a multiple of nstep_check: F = G(t_k) X with t_k the k-th
        basis time, k = c_i / nstep_check (operg, tools_4Dvar.py:299-304);
      h <- Qgm.step(h, hb, n_i) + n_i*dt/86400 * F (mod.py:867-913): PV is
        re-derived from SSH at every interval start (jqgm.py:536).
    Reverse: adF += n_i*dt/86400 * adh, model adjoint of the interval,
    adX += G(t_k)^T adF and adF = 0 at basis checkpoints
    (tools_4Dvar.py:355-392, mod.py:1058-1076).
    Background term (tools_4Dvar.py:262-273, 342-349, 395-398):
      prec=True   X = Q*X0 + Xb, Jb = X0.X0,      G = Q*adX + X0
      prec=False  X = X0 + Xb,   Jb = X0.X0/Q^2,  G = adX + X0/Q^2
    J = (Jo + Jb)/2 with Jo = sum misfit^2/sigma_R^2.

    Batched windows keep their own checkpoint lists (their own observation
    steps); the batch advances between the boundaries of the union of the
    lists, with a per-window forcing coefficient table (0 where a window does
    not end a model call), so that each window reproduces its single-window
    evaluation.

    Storage: the SSH at every interval start ([ninterval, B, ny, nx]) and the
    stage trajectory of one interval (recomputed per interval in reverse).
    """

    def __init__(self, plan: QG1LPlan, basis, h_init, hb, nstep, nstep_check, obs, Q=None, Xb=None,
                 sigma_R=1.0, prec=True):
        self.plan, self.basis, self.obs = plan, basis, obs
        self.B = obs.B
        self.nstep, self.nstep_check = int(nstep), int(nstep_check)
        self.sigma_R = float(sigma_R)
        self.prec = bool(prec)
        B, ny, nx = self.B, plan.ny, plan.nx
        dev, dt = plan.device, plan.dtype
        if basis.dtype != dt:
            raise TypeError("basis and model plans must share the dtype")
        self.vd_dtype = _lib.VD_F64 if dt == torch.float64 else _lib.VD_F32
        self.nb = basis.nbasis
        need = self.nstep // self.nstep_check + 1
        if basis.times.size < need:
            raise ValueError(f"the basis has {basis.times.size} times, the window needs {need}")
        self.hb = plan._as_batch(hb, "hb")
        self.h_init = plan._as_batch(h_init, "h_init").clone()
        if self.hb.shape[0] != B or self.h_init.shape[0] != B:
            raise ValueError("hb and h_init must have one field per window")
        zero_bg = float(self.hb.abs().max()) == 0.0
        self.qb = torch.zeros(B, ny, nx, dtype=dt, device=dev)
        self.hb_arg = None if zero_bg else self.hb
        self.qb_arg = None if zero_bg else self.qb
        q = basis.q() if Q is None else np.asarray(Q, dtype=np.float64)
        self.Q = torch.as_tensor(q, device=dev).to(dt)
        self.Qinv2 = torch.as_tensor(1.0 / q ** 2, device=dev).to(dt)
        xb = np.zeros(self.nb) if Xb is None else np.asarray(Xb, dtype=np.float64)
        self.Xb = torch.as_tensor(np.tile(xb, (B, 1)), device=dev).to(dt)
        self.obs_steps = sorted(int(s) for s in obs.steps if 0 <= s <= self.nstep)
        # Every window calls the model between its own checkpoints (its own
        # observation steps and the regular ones); the batch runs from one
        # boundary of the union of those lists to the next. A window ends a
        # model call only at its own checkpoints: there its SSH takes the
        # forcing n*dt/86400*F of that call; elsewhere its coefficient is 0 and
        # it continues integrating (PV re-derivation from SSH is exact there).
        self.win_cps = []
        for b in range(B):
            st = obs.obs_step[obs.obs_window == b]
            self.win_cps.append(checkpoints(self.nstep, self.nstep_check,
                                            [int(s) for s in np.unique(st) if 0 < s < self.nstep]))
        self.cps = sorted(set().union(*[set(c) for c in self.win_cps]))
        self.nint = len(self.cps) - 1
        coef = np.zeros((self.nint, B))
        for b, wc in enumerate(self.win_cps):
            wset = set(wc)
            last = 0
            for i in range(self.nint):
                end = self.cps[i + 1]
                if end in wset:
                    coef[i, b] = (end - last) * plan.dt / SECONDS_PER_DAY
                    last = end
        self.coef_host = coef
        self.coef = torch.as_tensor(coef, dtype=torch.float64, device=dev).contiguous()
        K = max(self.cps[i + 1] - self.cps[i] for i in range(self.nint))
        self.K = K
        self.traj = plan.new_traj(B, K)
        self.S = plan.nstage
        self.tv = self.traj.view(-1, 2, B, ny, nx)
        self.snap = torch.zeros(self.nint, B, ny, nx, dtype=dt, device=dev)
        z = lambda: torch.zeros(B, ny, nx, dtype=dt, device=dev)  # noqa: E731
        self.h, self.F, self.adh, self.adq, self.adF = z(), z(), z(), z(), z()
        # low part of the compensated PV state, re-derived with q at every
        # interval start (float32 plans)
        self.qlo = plan.new_qlo(B)
        self.X = torch.zeros(B, self.nb, dtype=dt, device=dev)
        self.adX = torch.zeros(B, self.nb, dtype=dt, device=dev)
        self.gb = torch.zeros(B, self.nb, dtype=dt, device=dev)
        self.grad = torch.zeros(B, self.nb, dtype=dt, device=dev)
        self.J = torch.zeros(B, dtype=torch.float64, device=dev)
        self.dot_scratch = torch.zeros(B, _lib.DOT_SCRATCH, dtype=torch.float64, device=dev)
        self.graph = None

    def memory_bytes(self):
        n = 0
        for t in (self.traj, self.snap):
            n += t.numel() * t.element_size()
        return n

    # ------------------------------------------------------------------
    def _fill0(self, t):
        _lib.call("vd_fill", self.vd_dtype, ctypes.c_longlong(t.numel()), 0.0, _p(t), _stream())

    def _copy(self, src, dst):
        _lib.call("vd_copy", self.vd_dtype, ctypes.c_longlong(src.numel()), _p(src), _p(dst), _stream())

    def _interval_forward(self, i):
        """Recompute the stage trajectory of interval i from its start SSH."""
        p, B = self.plan, self.B
        n = self.cps[i + 1] - self.cps[i]
        self._copy(self.snap[i], self.tv[0, 0])
        p.init_state(self.tv[0, 0], self.hb, self.tv[0, 1], self.qb, self.qlo)
        p.advance(B, self.traj, self.K, 0, n, self.hb_arg, self.qb_arg, self.qlo)
        return n

    def _run(self, X0):
        p, B, nb = self.plan, self.B, self.nb
        nbt = ctypes.c_longlong(B * nb)
        # background term
        if self.prec:
            _lib.call("vd_diag_axpy", self.vd_dtype, nbt, ctypes.c_longlong(nb), _p(self.Q), _p(X0),
                      _p(self.Xb), _p(self.X), _stream())
            self._copy(X0, self.gb)
        else:
            _lib.call("vd_axpby", self.vd_dtype, nbt, 1.0, _p(X0), 0.0, _p(self.X), _stream())
            _lib.call("vd_axpby", self.vd_dtype, nbt, 1.0, _p(self.Xb), 1.0, _p(self.X), _stream())
            _lib.call("vd_diag_axpy", self.vd_dtype, nbt, ctypes.c_longlong(nb), _p(self.Qinv2), _p(X0),
                      None, _p(self.gb), _stream())
        for b in range(B):
            _lib.call("vd_dot_f64", self.vd_dtype, ctypes.c_longlong(nb), _p(X0[b]), _p(self.gb[b]),
                      _p(self.dot_scratch[b]), _stream())
        # forward sweep
        self._copy(self.h_init, self.h)
        obs = self.obs
        for i in range(self.nint):
            c = self.cps[i]
            if c in obs.step_range:
                obs.apply_misfit(c, self.h)
            if c % self.nstep_check == 0:
                self.basis.project(c // self.nstep_check, self.X, out=self.F)
            self._copy(self.h, self.snap[i])
            self._copy(self.h, self.tv[0, 0])
            p.init_state(self.tv[0, 0], self.hb, self.tv[0, 1], self.qb, self.qlo)
            n = self.cps[i + 1] - c
            p.advance(B, self.traj, self.K, 0, n, self.hb_arg, self.qb_arg, self.qlo)
            _lib.call("vd_qg1l_force", p._h, B, _p(self.tv[n * self.S, 0]), _p(self.hb), _p(self.F),
                      _p(self.coef[i]), _p(self.h), _stream())
        if self.nstep in obs.step_range:
            obs.apply_misfit(self.nstep, self.h)
        obs.sumsq_per_window(self.J, 0.5 / self.sigma_R ** 2)
        for b in range(B):   # J[b] += Jb[b]/2, Jb[b] = dot_scratch[b, 0]
            _lib.call("vd_axpby", _lib.VD_F64, ctypes.c_longlong(1), 0.5, _p(self.dot_scratch[b]), 1.0,
                      _p(self.J[b:b + 1]), _stream())
        # reverse sweep
        self._fill0(self.adh)
        self._fill0(self.adF)
        self._fill0(self.adX)
        if self.nstep in obs.step_range:
            obs.apply_adjoint(self.nstep, self.adh)
        for i in reversed(range(self.nint)):
            c = self.cps[i]
            n = self._interval_forward(i)
            # adF += coef*adh; adh <- adjoint at the end of the interval
            _lib.call("vd_qg1l_force_adj", p._h, B, _p(self.adh), _p(self.adF), _p(self.coef[i]),
                      _p(self.adh), _stream())
            self._fill0(self.adq)
            p.advance_adj(B, self.traj, self.K, 0, n, self.adh, self.adq)
            p.init_state_adj(B, self.tv[0, 0], self.adq, self.adh)
            if c % self.nstep_check == 0:
                self.basis.project_T(c // self.nstep_check, self.adF, self.adX)
                self._fill0(self.adF)
            if c in obs.step_range:
                obs.apply_adjoint(c, self.adh)
        if self.prec:
            _lib.call("vd_diag_axpy", self.vd_dtype, nbt, ctypes.c_longlong(nb), _p(self.Q), _p(self.adX),
                      _p(self.gb), _p(self.grad), _stream())
        else:
            self._copy(self.gb, self.grad)
            _lib.call("vd_axpby", self.vd_dtype, nbt, 1.0, _p(self.adX), 1.0, _p(self.grad), _stream())

    def cost_and_grad(self, X0):
        """Returns (J [B] float64, grad [B, nbasis]) as device tensors (views of
        internal buffers, overwritten by the next call)."""
        if X0.dim() == 1:
            X0 = X0.unsqueeze(0)
        if X0.shape != (self.B, self.nb) or X0.dtype != self.plan.dtype:
            raise ValueError(f"control must be [{self.B}, {self.nb}] of the plan dtype")
        X0 = X0.contiguous()
        if self.graph is not None:
            self._copy(X0, self.X0_static)
            self.graph.replay()
        else:
            self._run(X0)
        return self.J, self.grad

    def capture(self):
        """Capture one whole evaluation into a CUDA graph."""
        self.X0_static = torch.zeros(self.B, self.nb, dtype=self.plan.dtype, device=self.plan.device)
        self._run(self.X0_static)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._run(self.X0_static)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = g
        return g


class MixedWindows4DVar:
    """Windows of different grid sizes evaluated together (one batched
    engine per size class, the layout of the reference's batch of
    independent assimilation windows, run_assimilation.py:27-349).

    Every engine runs on its own CUDA stream, forked from and joined back to
    the caller's stream, so the small grids fill the SMs next to the large
    ones; ``capture`` records the whole set (all streams) as one CUDA graph.
    ``cost_and_grad(xs)`` takes one control tensor per engine and returns
    [(J, grad)] in the same order."""

    def __init__(self, engines):
        self.engines = list(engines)
        self.streams = [torch.cuda.Stream() for _ in self.engines]
        self.graph = None
        self.x_static = None

    def _run(self, xs):
        cur = torch.cuda.current_stream()
        start = torch.cuda.Event()
        start.record(cur)
        done = []
        for eng, s, x in zip(self.engines, self.streams, xs):
            s.wait_event(start)
            with torch.cuda.stream(s):
                eng._run(x)
                e = torch.cuda.Event()
                e.record(s)
                done.append(e)
        for e in done:
            cur.wait_event(e)

    def cost_and_grad(self, xs):
        if len(xs) != len(self.engines):
            raise ValueError("one control per engine")
        xs = [eng.plan._as_batch(x, "h0") for eng, x in zip(self.engines, xs)]
        if self.graph is not None:
            for eng, x, xst in zip(self.engines, xs, self.x_static):
                eng._copy(x, xst)
            self.graph.replay()
        else:
            self._run(xs)
        return [(eng.J, eng.grad) for eng in self.engines]

    def tune(self, verbose=False):
        """Autotune each size class's inversion schedule for its batch
        (vardyn_gb300.autotune.tune); a captured graph is dropped, since it
        keeps the schedule it was captured with. Returns {(ny, nx):
        schedule}."""
        from . import autotune
        out = {}
        for eng in self.engines:
            sched, _ = autotune.tune(eng.plan, eng.B, verbose=verbose)
            out[(eng.plan.ny, eng.plan.nx)] = sched
        self.graph = None
        return out

    def capture(self):
        self.x_static = [torch.zeros(eng.B, eng.plan.ny, eng.plan.nx, dtype=eng.plan.dtype,
                                     device=eng.plan.device) for eng in self.engines]
        self._run(self.x_static)           # warm-up: workspaces, kernel attributes
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._run(self.x_static)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = g
        return g

    def memory_bytes(self):
        return sum(eng.memory_bytes() for eng in self.engines)
