"""Direct solve of the masked Dirichlet Helmholtz problems of the multilayer
QG PV inversion (mapping/models/model_qgsw/qg.py:222-298): per vertical mode,
the 5-point operator (u_E + u_W - 2u)/d0^2 + (u_N + u_S - 2u)/d1^2 - lambda u
on the ocean nodes of the interior psi grid, u = 0 at land nodes and beyond
the walls. This is the discrete problem the reference's DST + capacitance
method solves (helmholtz.py:146-184: its irregular boundary points are every
land point next to the ocean), assembled as a sparse matrix and solved with
scipy.sparse.linalg.spsolve. Test infrastructure and the CPU baseline of the
inversion only."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def dirichlet_operator(n0, n1, d0, d1, lam, mask):
    """(A, ocean_nodes): the CSR operator on the ocean nodes (mask > 0), in
    the order of ``np.argwhere``."""
    mask = np.asarray(mask)
    idx = -np.ones((n0, n1), dtype=np.int64)
    oc = np.argwhere(mask > 0)
    idx[oc[:, 0], oc[:, 1]] = np.arange(len(oc))
    a0, a1 = 1.0 / d0 ** 2, 1.0 / d1 ** 2
    rows = [np.arange(len(oc))]
    cols = [np.arange(len(oc))]
    vals = [np.full(len(oc), -2 * a0 - 2 * a1 - lam)]
    for di, dj, c in ((1, 0, a0), (-1, 0, a0), (0, 1, a1), (0, -1, a1)):
        ii, jj = oc[:, 0] + di, oc[:, 1] + dj
        ok = (ii >= 0) & (ii < n0) & (jj >= 0) & (jj < n1)
        nb = np.full(len(oc), -1, dtype=np.int64)
        nb[ok] = idx[ii[ok], jj[ok]]
        sel = nb >= 0
        rows.append(np.arange(len(oc))[sel])
        cols.append(nb[sel])
        vals.append(np.full(int(sel.sum()), c))
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(len(oc), len(oc)))
    return A, oc


def solve(n0, n1, d0, d1, lam, mask, b):
    """u [n0][n1] with A u = b on the ocean nodes, 0 elsewhere."""
    A, oc = dirichlet_operator(n0, n1, d0, d1, lam, mask)
    u = np.zeros((n0, n1))
    u[oc[:, 0], oc[:, 1]] = spla.spsolve(A.tocsc(), np.asarray(b)[oc[:, 0], oc[:, 1]])
    return u
