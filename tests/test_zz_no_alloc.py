"""The non-allocating PV -> SSH inversion (vd_qg1l_pv2h_noalloc) against the
workspace version (vd_qg1l_pv2h), both called through the C ABI.

It serves callers that cannot allocate GPU memory themselves, e.g. code
running in a fixed CUDA-graph memory plan or a plugin whose device memory
belongs to the host application's allocator. Its spectral intermediate lives
in a fixed array inside the library, shared by every call, so every call in a
sequence must give the workspace version's answer: nothing left over from a
previous call (a larger batch, another grid) may leak into the next. Both
versions run the same kernels on the same inputs, so the results must be
bit-identical. This file is collected last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from vardyn_gb300 import _lib, build
    build.build()
    return _lib.load()


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _plan(ny, nx, dtype):
    from vardyn_gb300.qg1l import QG1LPlan
    return QG1LPlan(ny, nx, 5e3, 5e3, 900.0, 1e-4, 2.7, time_scheme="rk2", dtype=dtype)


def _inputs(B, ny, nx, dtype, seed, with_background=True):
    rng = np.random.default_rng(seed)
    mk = lambda s: torch.as_tensor(rng.standard_normal((B, ny, nx)) * s, dtype=dtype, device="cuda")
    q, hb, qb = mk(1e-6), mk(1e-2), mk(1e-7)
    return (q, hb, qb) if with_background else (q, None, None)


def _with_workspace(lib, plan, q, hb, qb):
    from vardyn_gb300 import _lib
    h = torch.empty_like(q)
    ws = plan.workspace(q.shape[0])
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("vd_qg1l_pv2h", plan.handle, q.shape[0], _p(q), _p(hb), _p(qb), _p(h), _p(ws),
              ws.numel(), st)
    return h


def _no_alloc(lib, plan, q, hb, qb):
    from vardyn_gb300 import _lib
    h = torch.empty_like(q)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("vd_qg1l_pv2h_noalloc", plan.handle, q.shape[0], _p(q), _p(hb), _p(qb), _p(h), st)
    return h


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_no_alloc_matches_workspace_version_over_a_call_sequence(lib, dtype):
    # larger batch, then a smaller one (the scratch keeps the larger call's
    # tail), then another grid shape, then no background fields
    big = _plan(256, 320, dtype)
    other = _plan(200, 136, dtype)
    sequence = [(big, 5, 1, True), (big, 2, 2, True), (other, 3, 3, True), (big, 1, 4, False),
                (other, 4, 5, False)]
    for call, (plan, B, seed, bg) in enumerate(sequence):
        q, hb, qb = _inputs(B, plan.ny, plan.nx, dtype, seed, bg)
        ref = _with_workspace(lib, plan, q, hb, qb)
        got = _no_alloc(lib, plan, q, hb, qb)
        torch.cuda.synchronize()
        err = float((got - ref).norm() / ref.norm())
        print(f"call {call}: {dtype} {plan.ny}x{plan.nx} B={B} background={bg} relative L2 difference {err:.2e}")
        assert torch.equal(got, ref)


def test_no_alloc_rejects_requests_above_its_scratch(lib):
    plan = _plan(512, 512, torch.float32)
    limit = lib.vd_qg1l_pv2h_noalloc_max_bytes()
    per_window = lib.vd_qg1l_spec_bytes(plan.handle, 1)
    too_many = limit // per_window + 1
    dummy = torch.zeros(1, dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the size check happens before any pointer is used
    status = lib.vd_qg1l_pv2h_noalloc(plan.handle, int(too_many), _p(dummy), _p(dummy), _p(dummy),
                                      _p(dummy), st)
    assert status == 5  # VD_ERR_SIZE
