"""Masked multigrid Helmholtz solver on the GPU (vd_mg_solve) against the
float64 restatement of the reference's MG_Helmholtz and a direct solve."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl
import torch

from oracle.helmholtz_mg import MGOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def case(n0, n1, seed):
    rng = np.random.default_rng(seed)
    mask = np.ones((n0, n1))
    mask[n0 // 3:n0 // 2, n1 // 4:n1 // 2] = 0
    mask[:5, :7] = 0
    cu = 1.0 + 0.3 * rng.random((n0 + 1, n1))
    cv = 1.0 + 0.3 * rng.random((n0, n1 + 1))
    return rng, mask, cu, cv


@pytest.mark.parametrize("niter_bottom", [-1, 20])
def test_mg_fp64_matches_oracle(niter_bottom):
    from vardyn_gb300.helmholtz_mg import MG_Helmholtz
    rng, mask, cu, cv = case(96, 64, 3)
    lam = np.array([1e-3, 4e-3])
    g = MG_Helmholtz(1.0, 1.3, 96, 64, cu, cv, lambd=lam, mask=mask, niter_bottom=niter_bottom, max_ite=8)
    o = MGOracle(1.0, 1.3, 96, 64, cu, cv, lam, mask=mask, niter_bottom=niter_bottom, max_ite=8)
    assert g.n_levels == o.n_levels
    rhs = rng.standard_normal((2, 96, 64)) * mask
    f = g.solve(rhs)
    fo = o.solve(rhs)
    assert rel(f, fo) < 1e-11


@pytest.mark.parametrize("niter_bottom", [-1, 20])
@pytest.mark.parametrize("n0,n1", [(48, 32), (16, 24), (8, 8)])
def test_mg_small_grids_fp64_match_oracle(n0, n1, niter_bottom):
    """Grids whose every level runs in the one-block coarse kernel (from level
    0, on the caller's buffers), and a single-level grid."""
    from vardyn_gb300.helmholtz_mg import MG_Helmholtz
    rng = np.random.default_rng(n0 * n1)
    mask = np.ones((n0, n1))
    mask[n0 // 3:n0 // 2, n1 // 4:n1 // 2] = 0
    cu = 1.0 + 0.3 * rng.random((n0 + 1, n1))
    cv = 1.0 + 0.3 * rng.random((n0, n1 + 1))
    lam = np.array([1e-3, 4e-3, 0.5])
    g = MG_Helmholtz(1.0, 1.3, n0, n1, cu, cv, lambd=lam, mask=mask, niter_bottom=niter_bottom, max_ite=5)
    o = MGOracle(1.0, 1.3, n0, n1, cu, cv, lam, mask=mask, niter_bottom=niter_bottom, max_ite=5)
    assert g.n_levels == o.n_levels
    rhs = rng.standard_normal((3, n0, n1)) * mask
    assert rel(g.solve(rhs), o.solve(rhs)) < 1e-11


def test_mg_converges_to_direct_solve_and_fp32():
    from vardyn_gb300.helmholtz_mg import MG_Helmholtz
    rng, mask, cu, cv = case(128, 96, 4)
    lam = np.array([2e-4])
    g = MG_Helmholtz(2.0, 1.5, 128, 96, cu, cv, lambd=lam, mask=mask, niter_bottom=-1, max_ite=20)
    o = MGOracle(2.0, 1.5, 128, 96, cu, cv, lam, mask=mask, niter_bottom=-1, max_ite=20)
    rhs = rng.standard_normal((1, 128, 96)) * mask
    f = g.solve(rhs)
    A, i_s, j_s = o.operator_matrix(0)
    x = spl.spsolve(A.tocsc(), rhs[0, i_s, j_s])
    assert rel(f[0, i_s, j_s], x) < 1e-8
    assert np.all(f[0][mask == 0] == 0)
    r = g.residual(f, rhs)
    assert np.linalg.norm(r) < 1e-8 * np.linalg.norm(rhs)
    g32 = MG_Helmholtz(2.0, 1.5, 128, 96, cu, cv, lambd=lam, mask=mask, niter_bottom=-1, max_ite=20,
                       dtype=torch.float32)
    f32 = g32.solve(torch.as_tensor(rhs, device="cuda", dtype=torch.float32))
    assert rel(f32[0].double().cpu().numpy()[i_s, j_s], x) < 1e-5
