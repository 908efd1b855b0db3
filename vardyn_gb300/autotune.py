"""Autotuner of the QG 1.5-layer inversion schedule.

Batches of windows of uneven grid sizes (one plan per size, as the reference
runs one assimilation per window, ``run_assimilation.py:27-349``) do not all
run fastest with one fixed rule: whether the x-DST pass runs on the tensor
cores or on CUDA-core FMA, how many 32-column tiles a tensor-core CTA owns,
how many rows an FMA CTA owns and how many rows a tridiagonal thread owns
depend on the grid and on the number of windows. ``tune(plan, batch)`` times
the PV -> SSH inversion (forward x-DST, y tridiagonal solve, inverse x-DST:
the pass every model stage and adjoint stage runs) under each candidate
schedule on the plan's device, outside any graph capture, keeps the fastest
and sets it on the plan. Results are cached per (device, grid, dtype, engine
rule, batch) behind a lock, so plans of the same shape tune once per
process. Every candidate computes the same inversion (results agree to
rounding); the tuner only picks the fastest.
"""
import threading

import torch

_lock = threading.Lock()
_cache = {}


def candidates(plan):
    """Schedules worth timing for this plan: the built-in rule, FMA with each
    row tile, and (float32 plans with tensor-core images) tensor cores with
    each tile group; each with the three tridiagonal row counts and, in float32,
    the register-capped tridiagonal kernel."""
    out = [{}]
    f32 = plan.dtype == torch.float32
    rows = (16, 32, 64) if f32 else (16, 32)
    base = []
    for r in rows:
        base.append(dict(engine=1, fma_rows=r))
    if f32 and plan.dst_engine == "auto":
        for g in (1, 2, 4, 8):
            base.append(dict(engine=2, tc_group_fwd=g, tc_group_inv=g))
    tri = [dict(tridiag_rows=8), dict(tridiag_rows=16), dict(tridiag_rows=32)]
    if f32:
        tri.append(dict(tridiag_rows=16, tridiag_lean=1))
    for b in base:
        for t in tri:
            out.append(dict(b, **t))
    return out


def _inv_keys(plan):
    """The schedule fields the tuner sets (the inversion's); the others keep
    their values."""
    return tuple(k for k in plan.SCHEDULE_KEYS if k != "stencil_loads")


def _key(plan, batch):
    dev = plan.device
    return (torch.cuda.get_device_name(dev), plan.ny, plan.nx, str(plan.dtype), plan.dst_engine, int(batch))


def _time_inversion(plan, q, hb, qb, reps):
    plan.pv2h(q, hb, qb)                      # warm-up under this schedule
    st = torch.cuda.current_stream(plan.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        plan.pv2h(q, hb, qb)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(plan, batch, reps=10, verbose=False):
    """Pick and set the fastest inversion schedule of ``plan`` for ``batch``
    windows. Returns (schedule, {candidate index: ms})."""
    key = _key(plan, batch)
    with _lock:
        hit = _cache.get(key)
    if hit is not None:
        plan.set_schedule(**{k: 0 for k in _inv_keys(plan)})
        plan.set_schedule(**hit[0])
        return hit
    if torch.cuda.is_current_stream_capturing():
        raise RuntimeError("tune() times kernels: call it before graph capture")
    g = torch.Generator(device=plan.device).manual_seed(0)
    q = torch.randn(batch, plan.ny, plan.nx, generator=g, dtype=plan.dtype, device=plan.device) * 1e-5
    hb = torch.zeros_like(q)
    qb = torch.zeros_like(q)
    saved = plan.schedule()
    times = {}
    best, best_ms = None, float("inf")
    for i, cand in enumerate(candidates(plan)):
        try:
            plan.set_schedule(**{k: 0 for k in _inv_keys(plan)})
            plan.set_schedule(**cand)
        except RuntimeError:
            continue                           # a choice this plan cannot run
        ms = _time_inversion(plan, q, hb, qb, reps)
        times[i] = ms
        if verbose:
            print(f"  {plan.ny}x{plan.nx} b{batch} {cand or 'rule'}: {ms * 1e3:.1f} us")
        if ms < best_ms:
            best, best_ms = cand, ms
    plan.set_schedule(**{k: 0 for k in _inv_keys(plan)})
    if best is None:
        plan.set_schedule(**saved)
        return saved, times
    plan.set_schedule(**best)
    with _lock:
        _cache[key] = (dict(best), times)
    return dict(best), times


def clear_cache():
    with _lock:
        _cache.clear()
