"""Gaussian space-time basis on the GPU (vd_basis_project / _T) against the
float64 oracle restatement of Basis_gauss3d / Basis_multi."""
import types

import numpy as np
import pytest
import torch

from oracle.basis import Gauss3dOracle, MultiOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


COMPS = [dict(sigma_D=100, sigma_T=5, facns=2, facnlt=2, sigma_Q=0.1),
         dict(sigma_D=60, sigma_T=10, facns=1.5, facnlt=3, sigma_Q=0.2, time_spinup=3.0),
         dict(sigma_D=80, sigma_T=4, facns=1, facnlt=1, sigma_Q=0.3, flux=True, normalize_fact=False)]


def make(geo, dtype, land=True, ny=70, nx=90):
    from vardyn_gb300.basis import BasisPlan, Gauss3dParams
    if geo:
        xc, yc = -70 + np.arange(nx) * 0.05, 30 + np.arange(ny) * 0.05
    else:
        xc, yc = np.arange(nx) * 5.0, 3.0 + np.arange(ny) * 5.0
    mask = None
    if land:
        mask = np.zeros((ny, nx), bool)
        mask[20:31, 40:47] = True
        mask[-4:, :5] = True
    time = np.arange(0, 12.01, 0.25)
    params = [Gauss3dParams(**c) for c in COMPS]
    plan = BasisPlan(xc, yc, time, params, land=mask, geographic=geo, dtype=dtype)
    lon, lat = np.meshgrid(xc, yc)
    orc = MultiOracle([Gauss3dOracle(lon, lat, mask=mask, geo=geo, **c) for c in COMPS])
    orc.set_basis(time)
    return plan, orc, time, mask


@pytest.mark.parametrize("geo", [False, True])
def test_project_fp64_matches_oracle(geo):
    plan, orc, time, mask = make(geo, torch.float64)
    rng = np.random.default_rng(5)
    B = 3
    X = rng.standard_normal((B, plan.nbasis))
    Xd = torch.as_tensor(X, device="cuda")
    for k in (0, 1, 7, 20, len(time) - 1):
        phi = plan.project(k, Xd).cpu().numpy()
        for b in range(B):
            ref = orc.operg(time[k], X[b])
            assert rel(phi[b], ref) < 1e-13, (k, b)
            assert np.all(phi[b][mask] == 0)


@pytest.mark.parametrize("geo", [False, True])
def test_project_T_fp64_matches_oracle_and_accumulates(geo):
    plan, orc, time, mask = make(geo, torch.float64)
    rng = np.random.default_rng(6)
    B = 2
    A = rng.standard_normal((B, plan.ny, plan.nx))
    X0 = rng.standard_normal((B, plan.nbasis))
    adX = torch.as_tensor(X0.copy(), device="cuda")
    Ad = torch.as_tensor(A, device="cuda")
    ks = (0, 9, 33)
    for k in ks:
        plan.project_T(k, Ad, adX)
    got = adX.cpu().numpy()
    for b in range(B):
        ref = X0[b] + sum(orc.operg_transpose(time[k], A[b]) for k in ks)
        assert rel(got[b] - X0[b], ref - X0[b]) < 1e-13
    # the adjoint input is read only
    assert torch.equal(Ad.cpu(), torch.as_tensor(A))


def test_dot_product_identity_fp64():
    plan, orc, time, mask = make(False, torch.float64)
    rng = np.random.default_rng(7)
    X = torch.as_tensor(rng.standard_normal((1, plan.nbasis)), device="cuda")
    A = torch.as_tensor(rng.standard_normal((1, plan.ny, plan.nx)), device="cuda")
    for k in (2, 30):
        phi = plan.project(k, X)
        adX = torch.zeros_like(X)
        plan.project_T(k, A, adX)
        lhs = float((phi * A).sum())
        rhs = float((X * adX).sum())
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_project_fp32_and_accumulate():
    plan, orc, time, mask = make(False, torch.float32)
    rng = np.random.default_rng(8)
    X = rng.standard_normal((2, plan.nbasis))
    Xd = torch.as_tensor(X, device="cuda", dtype=torch.float32)
    base = torch.as_tensor(rng.standard_normal((2, plan.ny, plan.nx)), device="cuda", dtype=torch.float32)
    out = base.clone()
    plan.project(12, Xd, out=out, accumulate=True)
    for b in range(2):
        ref = orc.operg(time[12], X[b])
        assert rel(out[b].double().cpu().numpy() - base[b].double().cpu().numpy(), ref) < 2e-6
    A = rng.standard_normal((2, plan.ny, plan.nx))
    adX = torch.zeros(2, plan.nbasis, device="cuda", dtype=torch.float32)
    plan.project_T(12, torch.as_tensor(A, device="cuda", dtype=torch.float32), adX)
    for b in range(2):
        assert rel(adX[b].double().cpu().numpy(), orc.operg_transpose(time[12], A[b])) < 2e-6


def test_reference_facing_classes():
    """Basis_gauss3d / Basis_multi with the reference's (config, State)
    construction and State-dict semantics."""
    from vardyn_gb300.basis import Basis_gauss3d, Basis_multi
    ny, nx = 50, 60
    lon1, lat1 = -40 + np.arange(nx) * 0.05, 35 + np.arange(ny) * 0.05
    lon, lat = np.meshgrid(lon1, lat1)
    mask = np.zeros((ny, nx), bool)
    mask[5:9, 10:20] = True
    State = types.SimpleNamespace(lon=lon, lat=lat, mask=mask, ny=ny, nx=nx)

    def cfg(c):
        return types.SimpleNamespace(name_mod_var="ssh", flag_variable_Q=False, compute_velocities=False,
                                     c_grid_var=None, normalize_fact=c.get("normalize_fact", True),
                                     flux=c.get("flux", False), time_spinup=c.get("time_spinup"),
                                     sigma_D=c["sigma_D"], sigma_T=c["sigma_T"], facns=c["facns"],
                                     facnlt=c["facnlt"], sigma_Q=c["sigma_Q"])
    time = np.arange(0, 6.01, 0.5)
    rng = np.random.default_rng(9)
    # single component
    b1 = Basis_gauss3d(types.SimpleNamespace(BASIS=cfg(COMPS[0])), State, dtype=torch.float64)
    Xb, Q = b1.set_basis(time, return_q=True)
    o1 = Gauss3dOracle(lon, lat, mask=mask, geo=True, **COMPS[0])
    Xb_o, Q_o = o1.set_basis(time)
    assert np.array_equal(Q, Q_o) and np.array_equal(Xb, Xb_o)
    X = rng.standard_normal(b1.nbasis)
    params = {"ssh": np.zeros((ny, nx))}
    b1.operg(2.5, X, State=params)
    assert rel(params["ssh"], o1.operg(2.5, X)) < 1e-13
    ad = {"ssh": rng.standard_normal((ny, nx))}
    ad0 = ad["ssh"].copy()
    adX = b1.operg_transpose(2.5, ad)
    assert rel(adX, o1.operg_transpose(2.5, ad0)) < 1e-13
    assert np.all(ad["ssh"] == 0)
    # multi
    bm = Basis_multi(types.SimpleNamespace(BASIS={"a": cfg(COMPS[0]), "b": cfg(COMPS[1])}), State,
                     dtype=torch.float64)
    Xb, Q = bm.set_basis(time, return_q=True)
    om = MultiOracle([Gauss3dOracle(lon, lat, mask=mask, geo=True, **c) for c in COMPS[:2]])
    _, Qm = om.set_basis(time)
    assert np.array_equal(Q, Qm)
    X = rng.standard_normal(bm.nbasis)
    params = {"ssh": np.ones((ny, nx))}
    bm.operg(4.0, X, State=params)
    assert rel(params["ssh"], om.operg(4.0, X)) < 1e-13
    cat = bm.operg(4.0, X)
    parts = [c.operg(4.0, X[s]).ravel() for c, s in zip(om.comps, om.slices)]
    assert rel(cat, np.concatenate(parts)) < 1e-13
    ad = {"ssh": rng.standard_normal((ny, nx))}
    ad0 = ad["ssh"].copy()
    adX = bm.operg_transpose(4.0, ad)
    assert rel(adX, om.operg_transpose(4.0, ad0)) < 1e-13
    assert np.all(ad["ssh"] == 0)


BM_KW = dict(lmin=60, lmax=300, npsp=3.5, facpsp=1.5, lmeso=150, tmeso=10, time_ref=3.3, facns=1.2, facnlt=2.0)


@pytest.mark.parametrize("geo", [False, True])
def test_bm_project_and_transpose_fp64_match_oracle(geo):
    from oracle.basis import BMOracle
    from vardyn_gb300.basis import BMParams, BMPlan
    if geo:
        xc, yc = -60 + np.arange(110) * 0.05, 25 + np.arange(95) * 0.05
    else:
        xc, yc = np.arange(100) * 5.0, 2.0 + np.arange(90) * 5.0
    mask = np.zeros((yc.size, xc.size), bool)
    mask[:20, :30] = True
    time = np.arange(0, 10.01, 0.25)
    plan = BMPlan(xc, yc, time, BMParams(**BM_KW), land=mask, geographic=geo, dtype=torch.float64)
    lon, lat = np.meshgrid(xc, yc)
    o = BMOracle(lon, lat, mask=mask, geo=geo, **BM_KW)
    o.set_basis(time)
    rng = np.random.default_rng(11)
    B = 2
    X = rng.standard_normal((B, plan.nbasis))
    Xd = torch.as_tensor(X, device="cuda")
    for k in (0, 13, 40):
        phi = plan.project(k, Xd).cpu().numpy()
        for b in range(B):
            assert rel(phi[b], o.operg(time[k], X[b])) < 1e-12
    A = rng.standard_normal((B, yc.size, xc.size))
    adX = torch.zeros(B, plan.nbasis, dtype=torch.float64, device="cuda")
    for k in (5, 22):
        plan.project_T(k, torch.as_tensor(A, device="cuda"), adX)
    got = adX.cpu().numpy()
    for b in range(B):
        ref = o.operg_transpose(time[5], A[b]) + o.operg_transpose(time[22], A[b])
        assert rel(got[b], ref) < 1e-12


def test_bm_fp32_and_dot_product():
    from vardyn_gb300.basis import BMParams, BMPlan
    xc, yc = np.arange(120) * 4.0, np.arange(100) * 4.0
    time = np.arange(0, 8.01, 0.5)
    p64 = BMPlan(xc, yc, time, BMParams(**BM_KW), dtype=torch.float64)
    p32 = BMPlan(xc, yc, time, BMParams(**BM_KW), dtype=torch.float32)
    rng = np.random.default_rng(12)
    X = torch.as_tensor(rng.standard_normal((1, p64.nbasis)), device="cuda")
    A = torch.as_tensor(rng.standard_normal((1, yc.size, xc.size)), device="cuda")
    phi = p64.project(7, X)
    adX = torch.zeros_like(X)
    p64.project_T(7, A, adX)
    lhs, rhs = float((phi * A).sum()), float((X * adX).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    phi32 = p32.project(7, X.float())
    assert rel(phi32.double().cpu().numpy(), phi.cpu().numpy()) < 3e-6


def test_bm_reference_facing_class():
    """Basis_bm(config, State): the time reference comes from
    config.EXP.init_date (basis.py:527); State-dict semantics as operg /
    operg_transpose of the reference."""
    import datetime
    from oracle.basis import BMOracle
    from vardyn_gb300.basis import Basis_bm
    ny, nx = 60, 70
    lon, lat = np.meshgrid(-40 + np.arange(nx) * 0.05, 35 + np.arange(ny) * 0.05)
    mask = np.zeros((ny, nx), bool)
    mask[5:12, 10:25] = True
    State = types.SimpleNamespace(lon=lon, lat=lat, mask=mask, ny=ny, nx=nx)
    kw = dict(BM_KW)
    kw.pop("time_ref")
    init = datetime.datetime(2012, 10, 3, 6)
    tref = (init - datetime.datetime(1950, 1, 1)).total_seconds() / 86400
    cfgB = types.SimpleNamespace(name_mod_var="ssh", compute_velocities=False, file_depth=None, norm_time=True,
                                 flux=False, tdecmin=2.0, tdecmax=20.0, factdec=1.0, sloptdec=-1.28, Qmax=1e-3,
                                 slopQ=-2.0, **kw)
    config = types.SimpleNamespace(BASIS=cfgB, EXP=types.SimpleNamespace(init_date=init))
    b = Basis_bm(config, State, dtype=torch.float64)
    time = np.arange(0, 6.01, 0.5)
    Xb, Q = b.set_basis(time, return_q=True)
    o = BMOracle(lon, lat, mask=mask, geo=True, time_ref=tref, **kw)
    _, Qo = o.set_basis(time)
    assert np.array_equal(Q, Qo)
    rng = np.random.default_rng(13)
    X = rng.standard_normal(b.nbasis)
    params = {"ssh": np.zeros((ny, nx))}
    b.operg(3.0, X, State=params)
    assert rel(params["ssh"], o.operg(3.0, X)) < 1e-12
    ad = {"ssh": rng.standard_normal((ny, nx))}
    ad0 = ad["ssh"].copy()
    adX = b.operg_transpose(3.0, ad)
    assert rel(adX, o.operg_transpose(3.0, ad0)) < 1e-12
    assert np.all(ad["ssh"] == 0)


def test_wavelet_projection_matches_oracle():
    """Wavelet basis G and G^T (wave-packet kernels on the wavelet tables)
    against the oracle's sparse form, float64, with land."""
    from oracle.basis import WaveletOracle
    from vardyn_gb300.basis import WaveletParams, WaveletPlan
    x = np.arange(64) * 8.0
    y = np.arange(48) * 8.0
    prm = dict(npsp=3.5, facpsp=1.5, facnst=1., lmin=60., lmax=250., tmin=3., tmax=15., sigma_Q=0.02)
    land = np.zeros((48, 64), bool)
    land[20:30, 25:40] = True
    time = np.arange(0, 20, 0.5)
    pl = WaveletPlan(x, y, time, WaveletParams(**prm), land=land, dtype=torch.float64)
    X2, Y2 = np.meshgrid(x, y)
    o = WaveletOracle(X2, Y2, mask=land, **prm)
    o.set_basis(time)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((2, pl.nbasis))
    ad = rng.standard_normal((2, 48, 64))
    for k in (0, 9, 25, time.size - 1):
        phi = pl.project(k, torch.as_tensor(X, device="cuda")).cpu().numpy()
        adX = torch.zeros((2, pl.nbasis), dtype=torch.float64, device="cuda")
        pl.project_T(k, torch.as_tensor(ad, device="cuda"), adX)
        for b in range(2):
            ref = o.operg(time[k], X[b])
            assert np.abs(phi[b] - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
            refT = o.operg_transpose(time[k], ad[b])
            assert np.abs(adX[b].cpu().numpy() - refT).max() <= 1e-12 * max(1.0, np.abs(refT).max())
