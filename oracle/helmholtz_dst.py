"""Oracle (test infrastructure only): restatement of the spectral Helmholtz
solvers of mapping/models/model_qgsw/helmholtz.py in float64 NumPy/SciPy.

  compute_laplace_dstI            helmholtz.py:129-135
  solve_helmholtz_dstI            138-143 (2-D DST-I, division, edge padding)
  compute_capacitance_matrices    146-169
  solve_helmholtz_dstI_cmm        172-184

Pinned: against outputs of the reference's own helmholtz.py (golden
fixture, generated by tests/golden/gen_golden.py).
"""
import numpy as np
import scipy.fft


def dstI2D(x):
    return scipy.fft.dstn(np.asarray(x, dtype=np.float64), type=1, norm="ortho", axes=(-2, -1))


def compute_laplace_dstI(nx, ny, dx, dy):
    x, y = np.meshgrid(np.arange(1, nx, dtype=np.float64), np.arange(1, ny, dtype=np.float64), indexing="ij")
    return 2 * (np.cos(np.pi / nx * x) - 1) / dx ** 2 + 2 * (np.cos(np.pi / ny * y) - 1) / dy ** 2


def solve_helmholtz_dstI(rhs, helm):
    sol = dstI2D(dstI2D(rhs) / helm)
    pad = [(0, 0)] * (sol.ndim - 2) + [(1, 1), (1, 1)]
    return np.pad(sol, pad, mode="edge")


def compute_capacitance_matrices(helm, bx, by):
    nl, M = helm.shape[-3], len(bx)
    G = np.zeros((nl, M, M))
    for m in range(M):
        rhs = np.zeros(helm.shape[-3:])
        rhs[..., bx[m], by[m]] = 1
        sol = dstI2D(dstI2D(rhs) / helm)
        G[:, :, m] = sol.reshape((nl,) + sol.shape[-2:])[:, bx, by]
    return np.stack([np.linalg.inv(G[l]) for l in range(nl)])


def solve_helmholtz_dstI_cmm(rhs, helm, cap, bx, by, mask):
    sol1 = dstI2D(dstI2D(rhs) / helm)
    alphas = np.einsum("...ij,...j->...i", cap, -sol1[..., bx, by])
    rhs2 = np.zeros_like(rhs)
    rhs2[..., bx, by] = alphas
    return solve_helmholtz_dstI(rhs + rhs2, helm) * mask
