"""The non-allocating PV -> SSH inversion (vd_qg1l_pv2h_noalloc) against the
workspace version (vd_qg1l_pv2h), both called through the C ABI.

It serves callers that cannot allocate GPU memory themselves, e.g. code
running in a fixed CUDA-graph memory plan or a plugin whose device memory
belongs to the host application's allocator. Its spectral intermediate lives
in a fixed array inside the library, shared by every call, so two calls in a
row must each give the workspace version's answer (nothing left over from the
previous call may leak into the next). This file is collected last."""
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


def _inputs(B, ny, nx, dtype, seed):
    rng = np.random.default_rng(seed)
    mk = lambda s: torch.as_tensor(rng.standard_normal((B, ny, nx)) * s, dtype=dtype, device="cuda")
    return mk(1e-6), mk(1e-2), mk(1e-7)


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


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-6), (torch.float64, 1e-12)])
def test_no_alloc_matches_workspace_version_twice(lib, dtype, tol):
    ny, nx, B = 256, 320, 3
    plan = _plan(ny, nx, dtype)
    for call, seed in enumerate((1, 2)):   # two calls in a row, different inputs
        q, hb, qb = _inputs(B, ny, nx, dtype, seed)
        ref = _with_workspace(lib, plan, q, hb, qb)
        got = _no_alloc(lib, plan, q, hb, qb)
        torch.cuda.synchronize()
        err = float((got - ref).norm() / ref.norm())
        print(f"call {call}: {dtype} relative L2 difference {err:.2e}")
        assert err <= tol


def test_no_alloc_rejects_requests_above_its_scratch(lib):
    from vardyn_gb300 import _lib
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
