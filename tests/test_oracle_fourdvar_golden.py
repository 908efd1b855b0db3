"""The 4D-Var cost and gradient assembly against golden values produced by the
reference's own Variational.cost_and_grad (mapping/src/tools_4Dvar.py:252-400)
with Model_qg1l_jax.step / step_adj (mapping/src/mod.py:867-1076), the jax
along-track operator and a Gaussian reduced basis, on a lon/lat grid
(tests/golden/gen_golden_fourdvar.py). The oracle's restatement
(oracle/fourdvar.py) must reproduce them: one case with the preconditioned
background term, one with the plain term and a non-zero background."""
import os

import numpy as np
import pytest

from oracle import obsop as ob
from oracle.basis import Gauss3dOracle
from oracle.fourdvar import checkpoints, cost_and_grad_basis
from oracle.qg1l import QgmOracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "fourdvar_golden.npz")
PARAMS = ("sigma_D", "sigma_T", "facns", "facnlt", "sigma_Q")


def golden():
    return dict(np.load(GOLD))


def geometry(g):
    lon, lat = np.meshgrid(g["lon"], g["lat"])
    DX = np.radians(g["lon"][1] - g["lon"][0]) * 6371e3 * np.cos(np.radians(lat))
    DY = np.full(lon.shape, np.radians(g["lat"][1] - g["lat"][0]) * 6371e3)
    return lon, lat, DX, DY


class GeoObs:
    """Observations of one window with the jax operator's neighbours on the
    lon/lat grid (3-D Cartesian distances, obsop.py:417-460)."""

    def __init__(self, g, tag):
        lon, lat, DX, DY = geometry(g)
        self.ny, self.nx = lon.shape
        grid_pts = ob.geo2cart(np.column_stack((lon.ravel(), lat.ravel())))
        dmax = ob.dmax_from_metrics(DX, DY, 4)
        self.steps = g[f"{tag}_obs_steps"]
        self.per_step = {}
        for s in self.steps:
            pts = ob.geo2cart(np.column_stack((g[f"{tag}_obs{s}_lon"], g[f"{tag}_obs{s}_lat"])))
            data, rows, cols = ob.sparse_op_points(grid_pts, pts, 4, dmax)
            self.per_step[int(s)] = (data, rows, cols, g[f"{tag}_obs{s}_SSH"], g[f"{tag}_obs{s}_SSH_err"])

    def misfit(self, s, h):
        data, rows, cols, y, e = self.per_step[s]
        return ob.misfit(np.asarray(h).ravel(), data, rows, cols, y, e)

    def adj(self, s, mis, h):
        data, rows, cols, y, e = self.per_step[s]
        return ob.misfit_adj(mis, data, rows, cols, e, self.ny * self.nx, x_flat=np.asarray(h).ravel(),
                             yobs=y).reshape(self.ny, self.nx)

    def operator_rows(self):
        """Per-observation (idx, w) arrays [n, 4] in input order, steps in
        order (the layout of the library's AlongTrackObs ``operator``)."""
        idx, w, step = [], [], []
        for s in self.steps:
            data, rows, cols, y, e = self.per_step[int(s)]
            n = y.size
            i4, w4 = np.full((n, 4), -1, dtype=np.int64), np.zeros((n, 4))
            fill = np.zeros(n, dtype=np.int64)
            for d, r, c in zip(data, rows, cols):
                i4[r, fill[r]], w4[r, fill[r]] = c, d
                fill[r] += 1
            idx.append(i4)
            w.append(w4)
            step.append(np.full(n, s))
        return np.concatenate(idx), np.concatenate(w), np.concatenate(step)


def basis_params(g, tag):
    return {k: float(g[f"{tag}_basis_{k}"]) for k in PARAMS}


@pytest.mark.parametrize("tag", ["p", "n"])
def test_checkpoints_restatement_matches_reference(tag):
    g = golden()
    steps = [int(s) for s in g[f"{tag}_obs_steps"] if 0 < s < int(g["nstep"])]
    assert checkpoints(int(g["nstep"]), int(g["nstep_check"]), steps) == [int(c) for c in g[f"{tag}_checkpoints"]]


@pytest.mark.parametrize("tag", ["p", "n"])
def test_oracle_cost_and_gradient_match_reference(tag):
    g = golden()
    lon, lat, DX, DY = geometry(g)
    qgm = QgmOracle(dx=DX, dy=DY, dt=float(g["dt"]), c=2.7, g=9.81, f=1e-4, time_scheme="rk2")
    basis = Gauss3dOracle(lon, lat, geo=True, normalize_fact=True, flux=False, **basis_params(g, tag))
    _, Q = basis.set_basis(g[f"{tag}_time_basis"])
    assert np.allclose(Q, g[f"{tag}_Q"], rtol=1e-14, atol=0)
    J, G = cost_and_grad_basis(qgm, basis, g[f"{tag}_time_basis"], g[f"{tag}_X0"], g[f"{tag}_Xb"], g[f"{tag}_Q"],
                               g[f"{tag}_h_init"], np.zeros(lon.shape), int(g["nstep"]), int(g["nstep_check"]),
                               GeoObs(g, tag), prec=bool(g[f"{tag}_prec"]))
    Jr, Gr = float(g[f"{tag}_J"]), g[f"{tag}_G"]
    assert abs(J - Jr) / abs(Jr) < 1e-12
    assert np.linalg.norm(G - Gr) / np.linalg.norm(Gr) < 1e-11
