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
