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
"""
import ctypes
import math

import torch

from . import _lib
from .qg1l import QG1LPlan


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


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
        if checkpoint is None:
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
            self.snap = torch.zeros(self.nseg, 2, B, ny, nx, dtype=dt, device=dev)
        self.tv = self.traj.view(-1, 2, B, ny, nx)
        self.S = S
        self.graph = None

    # ------------------------------------------------------------------
    def memory_bytes(self):
        n = self.traj.numel() * self.traj.element_size()
        if self.snap is not None:
            n += self.snap.numel() * self.snap.element_size()
        return n

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
            p.advance(B, self.traj, self.traj_steps, prev, s - prev, self.hb_arg, self.qb_arg)
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
            self._copy(self.tv[0], self.snap[g])
            self._advance_segment(a, n, with_obs=True)
            self._copy(self.tv[n * self.S], self.tv[0])

    def _advance_segment(self, a, n, with_obs):
        p, B = self.plan, self.B
        local = [s - a for s in self.obs_steps if a < s <= a + n]
        prev = 0
        for ls in local + [n]:
            if ls <= prev:
                continue
            p.advance(B, self.traj, self.traj_steps, prev, ls - prev, self.hb_arg, self.qb_arg)
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
            self._copy(self.snap[g], self.tv[0])
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

    # ------------------------------------------------------------------
    def _run(self, h0):
        """Enqueue one cost+gradient evaluation for the control ``h0`` [B, ny, nx]."""
        p, B = self.plan, self.B
        self._copy(h0, self.tv[0, 0])
        p.init_state(self.tv[0, 0], self.hb, self.tv[0, 1], self.qb)
        h0_keep = self.tmp if self.snap is None else None
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
            self._copy(self.snap[0], self.tv[0])
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
