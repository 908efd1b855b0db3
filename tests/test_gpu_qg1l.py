"""QG 1.5-layer CUDA path (through the C ABI) against the oracle and the
reference's golden vectors.

Tolerances: float64 mode reproduces the reference to <= 1e-11 relative L2
(72 steps at 128^2); float32 errors are measured against the float64 golden
run and bounded as stated in each test."""
import numpy as np
import pytest
import torch

from oracle.qg1l import QgmOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def Qgm(**kw):
    from vardyn_gb300.model_qg1l.jqgm import Qgm as _Q
    return _Q(**kw)


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    m = ~(np.isnan(a) | np.isnan(b))
    assert np.array_equal(np.isnan(a), np.isnan(b))
    return np.linalg.norm(a[m] - b[m]) / max(np.linalg.norm(b[m]), 1e-300)


def small_kw(g, scheme):
    return dict(dx=g["small_dx"], dy=g["small_dy"], dt=1200.0, SSH=g["small_ssh"], c=2.7, g=9.81,
                f=g["small_f"], time_scheme=scheme, Kdiffus=50.0, bathymetry_PV_term=g["small_bathy"])


def test_pieces_fp64_match_reference(golden):
    g = golden
    m = Qgm(dtype="float64", **small_kw(g, "Euler"))
    ssh, hb = g["small_ssh"], g["small_hb"]
    u, v = m.h2uv(ssh)
    assert rel(u, g["small_h2uv_u"]) < 1e-13 and rel(v, g["small_h2uv_v"]) < 1e-13
    q = m.h2pv(ssh, hb)
    assert rel(q, g["small_h2pv"]) < 1e-13
    qb = m.h2pv(hb, hb)
    assert rel(m.pv2h(q, hb, qb), g["small_pv2h"]) < 1e-12
    u0, v0 = m.h2uv(np.nan_to_num(ssh))
    assert rel(m.rhs(u0, v0, q), g["small_rhs"]) < 1e-12


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3"])
def test_step_fp64_matches_reference_small(golden, scheme):
    m = Qgm(dtype="float64", **small_kw(golden, scheme))
    out = m.step(golden["small_ssh"], golden["small_hb"], nstep=3)
    assert rel(out, golden[f"small_step_{scheme}"]) < 1e-11


def c1_model(scheme, dtype):
    n = 128
    dx = np.full((n, n), 1.0e4)
    return Qgm(dx=dx, dy=dx, dt=1200.0, c=2.7, g=9.81, f=1e-4, time_scheme=scheme, dtype=dtype)


@pytest.mark.parametrize("scheme", ["rk2", "rk3"])
def test_c1_fp64_matches_reference(golden, scheme):
    out = c1_model(scheme, "float64").step(golden["c1_h0"], np.zeros((128, 128)), nstep=72)
    assert rel(out, golden[f"c1_step72_{scheme}"]) < 1e-11


def test_c1_rk4_extension_fp64_matches_oracle(golden):
    n = 128
    dx = np.full((n, n), 1.0e4)
    ref = QgmOracle(dx=dx, dy=dx, dt=1200.0, c=2.7, f=1e-4, time_scheme="rk4")
    exp = ref.step(golden["c1_h0"], np.zeros((n, n)), 72)
    out = c1_model("rk4", "float64").step(golden["c1_h0"], np.zeros((n, n)), nstep=72)
    assert rel(out, exp) < 1e-11


@pytest.mark.parametrize("scheme", ["rk2", "rk3"])
def test_c1_fp32_error_vs_fp64_reference(golden, scheme):
    """FP32 bulk arithmetic: SSH relative L2 error after 72 steps <= 1e-5."""
    out = c1_model(scheme, "float32").step(golden["c1_h0"].astype(np.float32),
                                          np.zeros((128, 128), np.float32), nstep=72)
    err = rel(out, golden[f"c1_step72_{scheme}"])
    print(f"C1 {scheme} fp32 SSH rel-L2 vs fp64 reference: {err:.3e}")
    assert err < 1e-5


def _rand_case(scheme, ny=22, nx=27, seed=0, land=True):
    rng = np.random.default_rng(seed)
    dx = np.full((ny, nx), 1.0e4)
    f = 1e-4 + 1.6e-11 * (np.arange(ny)[:, None] * 1e4 + np.zeros((1, nx)))
    ssh = 0.1 * rng.standard_normal((ny, nx))
    if land:
        ssh[8:10, 12:14] = np.nan
    kw = dict(dx=dx, dy=dx, dt=900.0, SSH=ssh, c=2.7, f=f, time_scheme=scheme, Kdiffus=30.0,
              bathymetry_PV_term=0.03 * rng.standard_normal((ny, nx)))
    return kw, np.nan_to_num(ssh), 0.01 * rng.standard_normal((ny, nx)), rng


# nx = 27: dense transform (26 = 2 x 13); nx = 31: FFT transform (L = 60)
@pytest.mark.parametrize("nx", [27, 31])
@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3", "rk4"])
def test_tangent_fp64_matches_oracle(scheme, nx):
    kw, h0, hb, rng = _rand_case(scheme, nx=nx)
    ref = QgmOracle(**kw)
    m = Qgm(dtype="float64", **kw)
    dh = 0.01 * rng.standard_normal(h0.shape)
    exp = ref.step_tgl(dh, h0, hb, 4)
    exp[ref.ind0] = 0.0
    assert rel(m.step_tgl(dh, h0, hb, 4), exp) < 1e-10


@pytest.mark.parametrize("nx", [27, 31])
@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3", "rk4"])
def test_adjoint_fp64_matches_oracle(scheme, nx):
    kw, h0, hb, rng = _rand_case(scheme, seed=4, nx=nx)
    ref = QgmOracle(**kw)
    m = Qgm(dtype="float64", **kw)
    ad = rng.standard_normal(h0.shape)
    assert rel(m.step_adj(ad, h0, hb, 4), ref.step_adj(ad, h0, hb, 4)) < 1e-10


@pytest.mark.parametrize("dtype,tol,nx", [("float64", 1e-12, 48), ("float64", 1e-12, 49), ("float32", 2e-4, 48)])
def test_dot_product_on_gpu(dtype, tol, nx):
    """<M dx, y> = <dx, M^T y> (mod.py:5367-5446 form), inner products in FP64."""
    kw, h0, hb, rng = _rand_case("rk2", ny=40, nx=nx, seed=7)
    m = Qgm(dtype=dtype, **kw)
    dx_ = rng.standard_normal(h0.shape)
    y = rng.standard_normal(h0.shape)
    y[m.ind0] = 0
    tl = np.nan_to_num(np.asarray(m.step_tgl(dx_, h0, hb, 6), dtype=np.float64))
    ad = np.asarray(m.step_adj(y, h0, hb, 6), dtype=np.float64)
    lhs = np.sum(tl * y)
    rhs = np.sum(dx_ * ad)
    assert abs(lhs - rhs) / abs(lhs) < tol


def test_batched_equals_single():
    import torch as T
    kw, h0, hb, rng = _rand_case("rk3", ny=34, nx=41, seed=2, land=False)
    m = Qgm(dtype="float64", **kw)
    hs = np.stack([h0 + 0.01 * rng.standard_normal(h0.shape) for _ in range(3)])
    hbs = np.stack([hb] * 3)
    batched = m.plan.step(T.as_tensor(hs, device="cuda"), T.as_tensor(hbs, device="cuda"), 5).cpu().numpy()
    for b in range(3):
        assert rel(batched[b], m.step(hs[b], hb, 5)) < 1e-14


@pytest.mark.parametrize("ny,nx", [(37, 45), (64, 130), (130, 64), (200, 262), (37, 61), (50, 16), (24, 769),
                                   (33, 9)])
def test_odd_and_ragged_grids_fp64(ny, nx):
    """Odd transform lengths (middle element of the even/odd split), ragged
    CTA tiles, more than one column tile; nx - 1 = 60, 15, 768 and 8 take the
    FFT form of the float64 transform (radices 4/2/3/5), the others the dense
    one."""
    rng = np.random.default_rng(ny * nx)
    dx = np.full((ny, nx), 5.0e3)
    kw = dict(dx=dx, dy=dx, dt=600.0, c=2.7, f=1e-4, time_scheme="rk2")
    ref = QgmOracle(**kw)
    m = Qgm(dtype="float64", **kw)
    h0 = 0.1 * rng.standard_normal((ny, nx))
    hb = 0.01 * rng.standard_normal((ny, nx))
    q = ref.h2pv(h0, hb)
    qb = ref.h2pv(hb, hb)
    assert rel(m.pv2h(q, hb, qb), ref.pv2h(q, hb, qb)) < 1e-12
    assert rel(m.step(h0, hb, 3), ref.step(h0, hb, 3)) < 1e-11


def test_helmholtz_512_fp32_error():
    """One inversion at 512^2: FP32 error of the DST-x / tridiagonal-y solve
    against the float64 DST2-lambda-DST2 of the reference form."""
    n = 512
    rng = np.random.default_rng(11)
    dx = np.full((n, n), 5.0e3)
    ref = QgmOracle(dx=dx, dy=dx, dt=900.0, c=2.7, f=1e-4, time_scheme="rk2")
    from vardyn_gb300.synthetic import kminus3_ssh
    h = kminus3_ssh(n, n, 5e3, 5e3, rng)
    hb = np.zeros((n, n))
    q = ref.h2pv(h, hb)
    exp = ref.pv2h(q, hb, hb * 0)
    m32 = Qgm(dtype="float32", dx=dx, dy=dx, dt=900.0, c=2.7, f=1e-4, time_scheme="rk2")
    got = m32.pv2h(q.astype(np.float32), hb.astype(np.float32), np.zeros((n, n), np.float32))
    err = rel(got, exp)
    print(f"512^2 fp32 Helmholtz rel-L2 (tensor-core 3xTF32 DST): {err:.3e}")
    assert err < 5e-6
    from vardyn_gb300.qg1l import QG1LPlan
    pf = QG1LPlan(n, n, 5e3, 5e3, 900.0, 1e-4, 2.7, dtype=torch.float32, dst_engine="fma")
    args = [torch.as_tensor(a, dtype=torch.float32, device="cuda")[None] for a in (q, hb, hb * 0)]
    err_f = rel(pf.pv2h(*args)[0].cpu().numpy(), exp)
    print(f"512^2 fp32 Helmholtz rel-L2 (CUDA-core FMA DST): {err_f:.3e}")
    assert err_f < 2e-6
    m64 = Qgm(dtype="float64", dx=dx, dy=dx, dt=900.0, c=2.7, f=1e-4, time_scheme="rk2")
    assert rel(m64.pv2h(q, hb, hb * 0), exp) < 1e-12


def sf_kw(g, scheme):
    return dict(dx=g["small_dx"], dy=g["small_dy"], dt=1200.0, SSH=g["small_ssh"], c=2.7, g=9.81,
                f=g["small_f"], time_scheme=scheme, Kdiffus=50.0, bathymetry_PV_term=g["small_bathy"])


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3"])
def test_streamfunction_form_fp64_matches_reference(golden, scheme):
    """Drop-in Qgm_sf (streamfunction form, jqgm.py:571-1031) against the
    reference's own outputs: steps, phi2pv and pv2phi."""
    from vardyn_gb300.model_qg1l.jqgm import Qgm_sf
    m = Qgm_sf(dtype="float64", **sf_kw(golden, scheme))
    out = m.step(golden["small_ssh"], golden["small_hb"], nstep=3)
    assert rel(out, golden[f"sf_step_{scheme}"]) < 1e-11
    if scheme == "Euler":
        f, ssh, hb = golden["small_f"], golden["small_ssh"], golden["small_hb"]
        phi, phib = 9.81 / f * np.nan_to_num(ssh), 9.81 / f * hb
        q = m.phi2pv(phi, phib)
        assert rel(q, golden["sf_phi2pv"]) < 1e-13
        assert rel(m.pv2phi(q, phib, m.phi2pv(phib, phib)), golden["sf_pv2phi"]) < 1e-12


def test_streamfunction_form_tangent_and_adjoint_fp64(golden):
    from oracle.qg1l import QgmSfOracle
    from vardyn_gb300.model_qg1l.jqgm import Qgm_sf
    m = Qgm_sf(dtype="float64", **sf_kw(golden, "rk2"))
    o = QgmSfOracle(**sf_kw(golden, "rk2"))
    rng = np.random.default_rng(5)
    h0 = np.nan_to_num(golden["small_ssh"])
    hb = golden["small_hb"]
    dh = rng.standard_normal(h0.shape) * 1e-2
    ad = rng.standard_normal(h0.shape)
    tl = m.step_tgl(dh, h0, hb, nstep=3)
    assert rel(np.nan_to_num(tl), np.nan_to_num(o.step_tgl(dh, h0, hb, 3))) < 1e-10
    adj = m.step_adj(ad, h0, hb, nstep=3)
    assert rel(adj, o.step_adj(ad, h0, hb, 3)) < 1e-10
