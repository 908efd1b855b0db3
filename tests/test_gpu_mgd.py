"""Masked Dirichlet multigrid of the multilayer QG PV inversion (vd_mgd_*):

- against a direct sparse solve (scipy.sparse.linalg.spsolve) of the same
  5-point Dirichlet Helmholtz operator on a domain with ~20 % land, float64
  and float32, including the in-place solve of a padded field's interior;
- inside the QG projector (QGPlan(inversion="multigrid")) against the
  reference's own projector outputs on the domain with an island, which the
  reference inverts with the DST and capacitance matrices (qg.py:222-298,
  helmholtz.py:146-184: the same discrete problem);
- the projector's transpose and a model step against the spectral inversion."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

from oracle.helmholtz_masked import dirichlet_operator

from test_gpu_qg_ml import NL, NX, NY, T, _dot, _state, g, params, plan, rel  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def land_mask(n0, n1, seed, frac=0.2):
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n0)[:, None] ** 2 + np.fft.fftfreq(n1)[None, :] ** 2
    f = np.real(np.fft.ifft2(np.exp(-k / 0.003) * (rng.standard_normal((n0, n1)) + 1j * rng.standard_normal((n0, n1)))))
    return (f < np.quantile(f, 1 - frac)).astype(np.float64)       # 1 = ocean


@pytest.mark.parametrize("dtype,tol,bar", [(torch.float64, 1e-11, 1e-9), (torch.float32, 1e-6, 2e-5)])
def test_matches_direct_sparse_solve_with_land(dtype, tol, bar):
    from vardyn_gb300.helmholtz_mg import MaskedDirichletMG
    n0, n1, d0, d1 = 127, 95, 5e3, 4e3
    lams = np.array([0.0, 3.1e-9, 7.7e-9])
    mask = land_mask(n0, n1, 5)
    mg = MaskedDirichletMG(n0, n1, d0, d1, lams, mask=mask, dtype=dtype, tol=tol, max_cycles=60)
    assert mg.levels >= 4
    rng = np.random.default_rng(6)
    B = 2
    b = rng.standard_normal((len(lams), B, n0, n1)) * 1e-9
    u = mg.solve(torch.as_tensor(b, dtype=dtype, device="cuda")).double().cpu().numpy()
    rel_res = mg.rel.cpu().numpy()
    for m, lam in enumerate(lams):
        A, oc = dirichlet_operator(n0, n1, d0, d1, lam, mask)
        for k in range(B):
            x = spla.spsolve(A.tocsc(), b[m, k][oc[:, 0], oc[:, 1]])
            got = u[m, k][oc[:, 0], oc[:, 1]]
            err = np.linalg.norm(got - x) / np.linalg.norm(x)
            print(f"\n{dtype} mode {m} window {k}: relative error vs spsolve {err:.2e}, "
                  f"relative residual {rel_res[m * B + k]:.1e}")
            assert err <= bar
            assert np.abs(u[m, k][mask == 0]).max() == 0.0
    assert (rel_res <= tol).all()


def test_strided_solve_in_a_padded_field():
    from vardyn_gb300.helmholtz_mg import MaskedDirichletMG
    n0, n1 = 63, 47
    mask = land_mask(n0, n1, 7)
    mg = MaskedDirichletMG(n0, n1, 5e3, 5e3, [1e-9, 2e-9], mask=mask, tol=1e-12)
    rng = np.random.default_rng(8)
    pad = torch.as_tensor(rng.standard_normal((2, 3, n0 + 2, n1 + 2)) * 1e-9, device="cuda")
    out = torch.full_like(pad, 7.0)
    X, Y = n0 + 2, n1 + 2
    mg.solve_strided(3, pad[:, :, 1:, 1:], Y, X * Y, out[:, :, 1:, 1:], Y, X * Y)
    ref = mg.solve(pad[:, :, 1:-1, 1:-1].contiguous())
    assert torch.allclose(out[:, :, 1:-1, 1:-1], ref, rtol=1e-12, atol=0)
    # the padding of the output is left as it was
    assert float(out[:, :, 0, :].min()) == 7.0 and float(out[:, :, :, -1].max()) == 7.0


def test_qg_projector_with_multigrid_matches_reference_capacitance(g):
    q = plan(g, True, inversion="multigrid", mg_tol=1e-13, mg_max_cycles=80)
    assert q.masked and not q.cmm and q.mg is not None
    assert rel(q.homsol, g["qgi_homsol"][0]) < 1e-9
    P = q.project(T(g["qgi_u"]), T(g["qgi_v"]), T(g["qgi_h"]))
    for a, k in zip(P, ["Pu", "Pv", "Ph"]):
        e = rel(a, g["qgi_" + k])
        print(f"\nmultigrid projector vs the reference's capacitance inversion, {k}: {e:.1e}")
        assert e < 1e-9, k


def test_qg_projector_transpose_and_step_with_multigrid(g):
    qm = plan(g, True, inversion="multigrid", mg_tol=1e-13, mg_max_cycles=80)
    qs = plan(g, True)
    rng = np.random.default_rng(3)
    m = qm.masks
    shapes = [(2, NL, NX + 1, NY), (2, NL, NX, NY + 1), (2, NL, NX, NY)]
    x = [T(rng.standard_normal(s) * mk) for s, mk in zip(shapes, (m.u, m.v, m.h))]
    y = [T(rng.standard_normal(s)) for s in shapes]
    lhs, rhs = _dot(qm.project(*x), y), _dot(x, qm.project_adj(*y))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
    st = _state(np.random.default_rng(21), qm)
    a = qm.step(*st, nstep=2)
    b = qs.step(*st, nstep=2)
    for u, v in zip(a, b):
        assert rel(u, v.cpu().numpy()) < 1e-9
