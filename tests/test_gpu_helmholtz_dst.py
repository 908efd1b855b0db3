"""Spectral Helmholtz solvers on the GPU (QG plan pv2h per mode, edge
padding and capacitance kernels of vd_helm.cu) against the reference's own
outputs and the float64 oracle."""
import os

import numpy as np
import pytest
import torch

from oracle import helmholtz_dst as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "qg1l_golden.npz")
NX, NY, DX, DY, F0 = 40, 30, 2.0e3, 2.5e3, 1.0e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    from vardyn_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLD))


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return np.abs(a - b).max() / np.abs(b).max()


def solver(g, dtype=torch.float64):
    from vardyn_gb300.helmholtz_dst import HelmholtzDST
    return HelmholtzDST(NX, NY, DX, DY, F0 ** 2 * g["helm_lam"], dtype=dtype)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-5)])
def test_solve_matches_reference(g, dtype, tol):
    s = solver(g, dtype)
    out = s.solve(torch.tensor(g["helm_rhs"], dtype=dtype, device="cuda"))
    assert out.shape == g["helm_dst_sol"].shape
    assert rel(out, g["helm_dst_sol"]) < tol


def test_capacitance_matches_reference(g):
    cap = solver(g).capacitance_matrices(g["helm_bx"], g["helm_by"])
    assert rel(cap, g["helm_cap"]) < 1e-10


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 1e-4)])
def test_cmm_matches_reference(g, dtype, tol):
    s = solver(g, dtype)
    cap = s.capacitance_matrices(g["helm_bx"], g["helm_by"])
    out = s.solve_cmm(torch.tensor(g["helm_rhs"], dtype=dtype, device="cuda"), cap, g["helm_bx"], g["helm_by"],
                      g["helm_mask"])
    assert rel(out, g["helm_cmm_sol"]) < tol
    assert torch.all(out[..., torch.tensor(g["helm_mask"], device="cuda") == 0] == 0)


def test_functional_dropins(g):
    from vardyn_gb300 import helmholtz_dst as H
    helm = O.compute_laplace_dstI(NX, NY, DX, DY)[None, None] - F0 ** 2 * g["helm_lam"].reshape(1, 2, 1, 1)
    rhs = torch.tensor(g["helm_rhs"], device="cuda")
    assert rel(H.solve_helmholtz_dstI(rhs, helm), g["helm_dst_sol"]) < 1e-12
    th = torch.tensor(helm, device="cuda")
    cap = H.compute_capacitance_matrices(th, g["helm_bx"], g["helm_by"])
    assert rel(cap, g["helm_cap"]) < 1e-10
    out = H.solve_helmholtz_dstI_cmm(rhs, th, cap, g["helm_bx"], g["helm_by"], torch.tensor(g["helm_mask"]))
    assert rel(out, g["helm_cmm_sol"]) < 1e-11


def test_batched_modes_against_oracle():
    """Leading batch axes, three modes, a non-square grid."""
    from vardyn_gb300.helmholtz_dst import HelmholtzDST
    rng = np.random.default_rng(5)
    nx, ny, dx, dy = 200, 130, 3.0e3, 2.0e3
    shift = np.array([0.0, 2e-8, 9e-8])
    rhs = rng.standard_normal((2, 3, 3, nx - 1, ny - 1))
    helm = O.compute_laplace_dstI(nx, ny, dx, dy)[None] - shift.reshape(3, 1, 1)
    s = HelmholtzDST(nx, ny, dx, dy, shift)
    out = s.solve(torch.tensor(rhs, device="cuda"))
    assert out.shape == (2, 3, 3, nx + 1, ny + 1)
    assert rel(out, O.solve_helmholtz_dstI(rhs, helm)) < 1e-11
    mask = np.ones((nx + 1, ny + 1))
    mask[0], mask[-1], mask[:, 0], mask[:, -1] = 0, 0, 0, 0
    mask[60:75, 40:52] = 0
    mask[120:140, 90:95] = 0
    isl = np.argwhere(mask[1:-1, 1:-1] == 0)
    bx, by = isl[:, 0], isl[:, 1]
    cap = s.capacitance_matrices(bx, by)
    ocap = O.compute_capacitance_matrices(helm[None], bx, by)
    assert rel(cap, ocap) < 1e-9
    out = s.solve_cmm(torch.tensor(rhs, device="cuda"), cap, bx, by, mask)
    ref = O.solve_helmholtz_dstI_cmm(rhs, helm, ocap, bx, by, mask)
    assert rel(out, ref) < 1e-10


@pytest.mark.parametrize("nx,ny", [(20, 8), (12, 15), (9, 48), (17, 100), (7, 768), (30, 131), (9, 1500),
                                   (9, 2048)])
def test_transform_lengths_fp64(nx, ny):
    """float64 solves through the FFT form of the transform (2 ny = 16, 30,
    96, 200, 1536, 3000: radices 4, 2, 3, 5; 4096: one row pair fills 131 KB
    of shared memory) and the dense form (2 x 131 = 262)."""
    from vardyn_gb300.helmholtz_dst import HelmholtzDST
    rng = np.random.default_rng(nx * ny)
    shift = np.array([0.0, 0.3, 2.0])
    s = HelmholtzDST(nx, ny, 1.1, 0.9, shift)
    rhs = rng.standard_normal((2, 3, nx - 1, ny - 1))
    helm = O.compute_laplace_dstI(nx, ny, 1.1, 0.9)[None] - shift.reshape(3, 1, 1)
    out = s.solve(torch.as_tensor(rhs, device="cuda")).cpu().numpy()
    for b in range(2):
        assert rel(out[b], O.solve_helmholtz_dstI(rhs[b], helm)) < 1e-12


def test_cmm_without_boundary_points_is_masked_solve(g):
    s = solver(g)
    rhs = torch.tensor(g["helm_rhs"], device="cuda")
    empty = np.zeros(0, dtype=np.int64)
    cap = s.capacitance_matrices(empty, empty)
    mask = np.ones((NX + 1, NY + 1))
    mask[3:9, 4:6] = 0
    out = s.solve_cmm(rhs, cap, empty, empty, mask)
    assert rel(out, g["helm_dst_sol"] * mask) < 1e-12


def test_single_mode_and_2d_rhs():
    from vardyn_gb300.helmholtz_dst import HelmholtzDST
    rng = np.random.default_rng(8)
    nx, ny = 33, 65
    rhs = rng.standard_normal((nx - 1, ny - 1))
    s = HelmholtzDST(nx, ny, 1.0, 1.3, [0.25])
    out = s.solve(torch.tensor(rhs, device="cuda"))
    assert out.shape == (nx + 1, ny + 1)
    assert rel(out, O.solve_helmholtz_dstI(rhs, O.compute_laplace_dstI(nx, ny, 1.0, 1.3) - 0.25)) < 1e-12
