"""The library's Gaussian basis projection and transpose on the GPU against
golden vectors produced by the reference's own basis.py
(tests/golden/gen_golden_basis.py): three components on a lon/lat grid with
land; the multi-component plan sums the components' fields."""
import os

import numpy as np
import pytest
import torch

from test_oracle_basis_golden import COMPS

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "basis_golden.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


def test_projection_and_transpose_match_reference():
    from vardyn_gb300.basis import BasisPlan, Gauss3dParams
    g = dict(np.load(GOLD))
    plan = BasisPlan(g["lon"], g["lat"], g["time"], [Gauss3dParams(**c) for c in COMPS], land=g["mask"],
                     geographic=True, dtype=torch.float64)
    X = torch.as_tensor(np.concatenate([g[f"c{c}_X"] for c in range(len(COMPS))]), device="cuda")[None]
    for k in g["times_k"]:
        want = sum(g[f"c{c}_t{k}_phi"] for c in range(len(COMPS)))
        phi = plan.project(int(k), X)[0].cpu().numpy()
        assert np.abs(phi - want).max() <= 1e-12 * np.abs(want).max()
        adX = torch.zeros_like(X)
        plan.project_T(int(k), torch.as_tensor(g[f"t{k}_ad"], device="cuda")[None].contiguous(), adX)
        want_ad = np.concatenate([g[f"c{c}_t{k}_adX"] for c in range(len(COMPS))])
        assert np.abs(adX[0].cpu().numpy() - want_ad).max() <= 1e-12 * np.abs(want_ad).max()


def test_wave_packet_projection_and_transpose_match_reference():
    from test_oracle_bm_golden import BM
    from vardyn_gb300.basis import BMParams, BMPlan
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bm_golden.npz")))
    plan = BMPlan(g["lon"], g["lat"], g["time"], BMParams(time_ref=float(g["time_ref"]), **BM), land=g["mask"],
                  geographic=True, dtype=torch.float64)
    X = torch.as_tensor(g["X"], device="cuda")[None].contiguous()
    for k in g["times_k"]:
        phi = plan.project(int(k), X)[0].cpu().numpy()
        want = g[f"t{k}_phi"]
        assert np.abs(phi - want).max() <= 1e-12 * np.abs(want).max()
        adX = torch.zeros_like(X)
        plan.project_T(int(k), torch.as_tensor(g[f"t{k}_ad"], device="cuda")[None].contiguous(), adX)
        want_ad = g[f"t{k}_adX"]
        assert np.abs(adX[0].cpu().numpy() - want_ad).max() <= 1e-12 * np.abs(want_ad).max()


def test_wavelet_projection_and_transpose_match_reference():
    from test_oracle_wavelet_golden import WAV
    from vardyn_gb300.basis import WaveletParams, WaveletPlan
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "wavelet_golden.npz")))
    plan = WaveletPlan(g["lon"], g["lat"], g["time"], WaveletParams(**WAV), land=g["mask"], geographic=True,
                       dtype=torch.float64)
    X = torch.as_tensor(g["X"], device="cuda")[None].contiguous()
    for k in g["times_k"]:
        phi = plan.project(int(k), X)[0].cpu().numpy()
        want = g[f"t{k}_phi"]
        assert np.abs(phi - want).max() <= 1e-12 * np.abs(want).max()
        adX = torch.zeros_like(X)
        plan.project_T(int(k), torch.as_tensor(g[f"t{k}_ad"], device="cuda")[None].contiguous(), adX)
        want_ad = g[f"t{k}_adX"]
        assert np.abs(adX[0].cpu().numpy() - want_ad).max() <= 1e-12 * np.abs(want_ad).max()


def _bmaux_plan(dtype):
    from test_oracle_bmaux_golden import PRM, aux_sorted
    from vardyn_gb300.basis import BMauxParams, BMauxPlan
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bmaux_golden.npz")))
    plan = BMauxPlan(g["lon"], g["lat"], g["time"], BMauxParams(aux_sorted(g), time_ref=float(g["time_ref"]), **PRM),
                     land=g["mask"], geographic=True, dtype=dtype)
    return g, plan


def test_aux_wave_packet_projection_and_transpose_match_reference():
    """Basis_bmaux: G and G^T on the GPU (per-centre time reduction, then the
    wave-packet passes) against the projection formed from the reference's
    own Gx and Gt. The time centres start at -time_ref mod tdec, which turns
    tdec's last-bit rounding into ~1e-12-day offsets: the bar is 1e-11."""
    g, plan = _bmaux_plan(torch.float64)
    X = torch.as_tensor(g["X"], device="cuda")[None].contiguous()
    for k in g["times_k"]:
        phi = plan.project(int(k), X)[0].cpu().numpy()
        want = g[f"t{k}_phi"]
        e1 = np.abs(phi - want).max() / np.abs(want).max()
        adX = torch.zeros_like(X)
        plan.project_T(int(k), torch.as_tensor(g[f"t{k}_ad"], device="cuda")[None].contiguous(), adX)
        want_ad = g[f"t{k}_adX"]
        e2 = np.abs(adX[0].cpu().numpy() - want_ad).max() / np.abs(want_ad).max()
        print(f"\nbmaux t{k}: G {e1:.1e}, G^T {e2:.1e}")
        assert e1 <= 1e-11 and e2 <= 1e-11


def test_aux_wave_packets_float32_batched_and_drop_in():
    """float32 against the reference's vectors, three windows in one call
    equal to single calls, and the drop-in class with its State semantics."""
    from types import SimpleNamespace as NS
    import datetime
    from test_oracle_bmaux_golden import PRM
    from vardyn_gb300.basis import Basis_bmaux
    g, plan = _bmaux_plan(torch.float32)
    rng = np.random.default_rng(5)
    Xs = np.stack([g["X"], rng.standard_normal(g["X"].size), rng.standard_normal(g["X"].size)])
    X = torch.as_tensor(Xs, dtype=torch.float32, device="cuda").contiguous()
    k = int(g["times_k"][2])
    phi = plan.project(k, X).cpu().numpy()
    want = g[f"t{k}_phi"]
    assert np.linalg.norm(phi[0] - want) <= 2e-6 * np.linalg.norm(want)
    for b in range(3):
        one = plan.project(k, X[b:b + 1].contiguous())[0].cpu().numpy()
        assert np.abs(one - phi[b]).max() <= 1e-6 * np.abs(phi[b]).max()
    # drop-in: config / State as the reference's
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    ny, nx = lon.shape
    ds = dict(f=g["aux_f"], lat=g["aux_lat"], lon=g["aux_lon"], Tdec=g["aux_tdec"], Std=g["aux_std"])
    state = NS(ny=ny, nx=nx, lon=lon, lat=lat, mask=g["mask"], lon_unit="-180_180", params={})
    t0 = datetime.datetime(1950, 1, 1) + datetime.timedelta(days=float(g["time_ref"]))
    cfg = NS(EXP=NS(init_date=t0), BASIS=NS(name_mod_var="ssh", file_aux=ds, file_depth=None, file_facQaux=None,
                                            compute_velocities=False, path_background=None, **PRM))
    B = Basis_bmaux(cfg, state, dtype=torch.float64)
    _, Q = B.set_basis(g["time"], return_q=True)
    assert np.allclose(Q, g["q"], rtol=1e-13, atol=0)
    t = g["time"][k]
    out = B.operg(t, g["X"])
    assert np.abs(out - want).max() <= 1e-11 * np.abs(want).max()
    adX = B.operg_transpose(t, {"ssh": g[f"t{k}_ad"].copy()})
    assert np.abs(adX - g[f"t{k}_adX"]).max() <= 1e-11 * np.abs(g[f"t{k}_adX"]).max()
