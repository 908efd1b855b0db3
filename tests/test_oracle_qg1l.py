"""The float64 QG 1.5-layer oracle against the reference's golden vectors,
and its tangent/adjoint against finite differences and dot-product tests."""
import numpy as np
import pytest

from oracle.qg1l import (QgmOracle, build_mask, dst1_via_irfft, dst2,
                         model_step, model_step_adj, model_step_tgl)


def small_model(g, scheme):
    return QgmOracle(dx=g["small_dx"], dy=g["small_dy"], dt=1200.0, SSH=g["small_ssh"],
                     c=2.7, g=9.81, f=g["small_f"], time_scheme=scheme, Kdiffus=50.0,
                     bathymetry_PV_term=g["small_bathy"])


def rel(a, b):
    m = ~(np.isnan(a) | np.isnan(b))
    assert np.array_equal(np.isnan(a), np.isnan(b))
    return np.linalg.norm(a[m] - b[m]) / max(np.linalg.norm(b[m]), 1e-300)


def test_dst_matches_reference(golden):
    x = golden["dst_in"]
    assert np.max(np.abs(dst2(x) - golden["dst_out"])) < 1e-13
    assert np.max(np.abs(dst1_via_irfft(x) - dst2.__globals__["dst1"](x))) < 1e-13


def test_mask_matches_reference(golden):
    ssh = golden["small_ssh"]
    assert np.array_equal(build_mask(*ssh.shape, ssh), golden["small_mask"])
    m = build_mask(16, 20)
    assert (m[0] == 1).all() and (m[:, -1] == 1).all()
    assert (m[-3, 1:-1] == 2).all() and (m[2, 2:-3] == 3).all()


def test_pieces_match_reference(golden):
    g = golden
    m = small_model(g, "Euler")
    ssh, hb = g["small_ssh"], g["small_hb"]
    u, v = m.h2uv(ssh)
    assert rel(u, g["small_h2uv_u"]) < 1e-14 and rel(v, g["small_h2uv_v"]) < 1e-14
    q = m.h2pv(ssh, hb)
    assert rel(q, g["small_h2pv"]) < 1e-14
    qb = m.h2pv(hb, hb)
    assert rel(m.pv2h(q, hb, qb), g["small_pv2h"]) < 1e-13
    u0, v0 = m.h2uv(np.nan_to_num(ssh))
    assert rel(m.rhs(u0, v0, q), g["small_rhs"]) < 1e-13


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3"])
def test_step_matches_reference_small(golden, scheme):
    m = small_model(golden, scheme)
    out = m.step(golden["small_ssh"], golden["small_hb"], nstep=3)
    assert rel(out, golden[f"small_step_{scheme}"]) < 1e-12


@pytest.mark.parametrize("scheme", ["rk2", "rk3"])
def test_step_matches_reference_c1(golden, scheme):
    n = 128
    dx = np.full((n, n), 1.0e4)
    m = QgmOracle(dx=dx, dy=dx, dt=1200.0, c=2.7, g=9.81, f=1e-4, time_scheme=scheme)
    out = m.step(golden["c1_h0"], np.zeros((n, n)), nstep=72)
    assert rel(out, golden[f"c1_step72_{scheme}"]) < 1e-12


def _rand_case(scheme, seed=0, land=True):
    rng = np.random.default_rng(seed)
    ny, nx = 20, 26
    dx = np.full((ny, nx), 1.0e4)
    f = 1e-4 + 1.6e-11 * (np.arange(ny)[:, None] * 1e4 + np.zeros((1, nx)))
    ssh = 0.1 * rng.standard_normal((ny, nx))
    if land:
        ssh[8:10, 12:14] = np.nan
    m = QgmOracle(dx=dx, dy=dx, dt=900.0, SSH=ssh, c=2.7, f=f, time_scheme=scheme,
                  Kdiffus=30.0, bathymetry_PV_term=0.03 * rng.standard_normal((ny, nx)))
    h0 = np.nan_to_num(ssh)
    hb = 0.01 * rng.standard_normal((ny, nx))
    return m, h0, hb, rng


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3", "rk4"])
def test_tangent_matches_finite_differences(scheme):
    m, h0, hb, rng = _rand_case(scheme)
    dh = 0.01 * rng.standard_normal(h0.shape)
    tl = m.step_tgl(dh, h0, hb, nstep=4)
    eps = 1e-4
    fd = (m.step(h0 + eps * dh, hb, 4) - m.step(h0 - eps * dh, hb, 4)) / (2 * eps)
    fd[m.ind0] = 0.0    # land is overwritten with NaN: zero tangent there
    assert rel(tl, fd) < 1e-6


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3", "rk4"])
def test_adjoint_dot_product(scheme):
    m, h0, hb, rng = _rand_case(scheme, seed=3)
    dh = rng.standard_normal(h0.shape)
    ad = rng.standard_normal(h0.shape)
    tl = np.nan_to_num(m.step_tgl(dh, h0, hb, nstep=4))
    adj = m.step_adj(ad, h0, hb, nstep=4)
    lhs = np.sum(tl * ad)
    rhs = np.sum(dh * adj)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_model_wrapper_adjoint():
    m, h0, hb, rng = _rand_case("rk2", seed=5, land=False)
    dh, dF = rng.standard_normal(h0.shape), rng.standard_normal(h0.shape)
    ah, aF = rng.standard_normal(h0.shape), rng.standard_normal(h0.shape)
    tl = model_step_tgl(m, dh, dF, h0, hb, 3)
    adh, adF = model_step_adj(m, ah, aF.copy(), h0, hb, 3)
    lhs = np.sum(tl * ah)
    rhs = np.sum(dh * adh) + np.sum(dF * (adF - aF))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
    F = 0.01 * rng.standard_normal(h0.shape)
    out = model_step(m, h0, F, hb, 3)
    assert np.allclose(out, m.step(h0, hb, 3) + 3 * 900.0 / 86400 * F)


def _sf_kw(g, scheme):
    return dict(dx=g["small_dx"], dy=g["small_dy"], dt=1200.0, SSH=g["small_ssh"], c=2.7, g=9.81,
                f=g["small_f"], time_scheme=scheme, Kdiffus=50.0, bathymetry_PV_term=g["small_bathy"])


@pytest.mark.parametrize("scheme", ["Euler", "rk2", "rk3"])
def test_streamfunction_form_matches_reference(golden, scheme):
    """QgmSfOracle reproduces the reference's Qgm_sf (jqgm.py:571-1031) run on
    a beta plane with land, diffusion, bathymetry and hb != 0."""
    from oracle.qg1l import QgmSfOracle
    m = QgmSfOracle(**_sf_kw(golden, scheme))
    assert np.array_equal(m.mask, golden["sf_mask"])
    out = m.step(golden["small_ssh"], golden["small_hb"], 3)
    ref = golden[f"sf_step_{scheme}"]
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    assert np.nanmax(np.abs(out - ref)) <= 1e-12 * np.nanmax(np.abs(ref))
    if scheme == "Euler":
        f, ssh, hb = golden["small_f"], golden["small_ssh"], golden["small_hb"]
        phi, phib = 9.81 / f * np.nan_to_num(ssh), 9.81 / f * hb
        q = m.phi2pv(phi, phib)
        assert np.abs(q - golden["sf_phi2pv"]).max() <= 1e-12 * np.abs(golden["sf_phi2pv"]).max()
        back = m.pv2phi(q, phib, m.phi2pv(phib, phib))
        assert np.abs(back - golden["sf_pv2phi"]).max() <= 1e-12 * np.abs(golden["sf_pv2phi"]).max()


def test_streamfunction_form_adjoint_dot_product(golden):
    from oracle.qg1l import QgmSfOracle
    m = QgmSfOracle(**_sf_kw(golden, "rk2"))
    rng = np.random.default_rng(4)
    h0 = np.nan_to_num(golden["small_ssh"])
    dh = rng.standard_normal(h0.shape) * 1e-2
    ad = rng.standard_normal(h0.shape)
    tl = np.nan_to_num(m.step_tgl(dh, h0, golden["small_hb"], 3))
    adj = m.step_adj(ad, h0, golden["small_hb"], 3)
    lhs, rhs = np.sum(tl * ad), np.sum(dh * adj)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
