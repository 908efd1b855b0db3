"""Generate golden vectors for the masked multigrid Helmholtz solver from the
reference's own ``mapping/models/model_qgsw/helmholtz_multigrid.py``
(``MG_Helmholtz``, 156-419) and its ``tools.avg_pool2d``: ``solve`` (full
multigrid then V-cycles) on masked grids with variable face coefficients,
for the exact bottom solve (niter_bottom = -1), bottom smoothing
(niter_bottom = 20) and a single-level grid.

jax is the NumPy stand-in of ``_jax_standin.py`` (jit is the identity,
fori_loop the plain loop).

Usage (only where the reference checkout exists):
    python tests/golden/gen_golden_mg.py <VarDyn checkout>
Writes ``tests/golden/mg_golden.npz``.
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import _jax_standin  # noqa: E402

CASES = {"a": (48, 32, -1, [1e-3, 4e-3], 5), "b": (48, 32, 20, [1e-3, 4e-3], 5), "c": (8, 8, -1, [0.5], 3)}


def load_mg(ref_root):
    _jax_standin.install(enable_x64=True)
    d = os.path.join(ref_root, "mapping", "models", "model_qgsw")
    mods = {}
    for name, fn in (("tools", "tools.py"), ("helmholtz_multigrid_reference", "helmholtz_multigrid.py")):
        spec = importlib.util.spec_from_file_location(name, os.path.join(d, fn))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods["helmholtz_multigrid_reference"]


def main():
    ref_root = _jax_standin.reference_root()
    mg = load_mg(ref_root)
    out = {}
    for tag, (nx, ny, nb, lam, ite) in CASES.items():
        rng = np.random.default_rng(nx * ny + nb + 7)
        mask = np.ones((nx, ny))
        mask[nx // 3:nx // 2, ny // 4:ny // 2] = 0
        mask[:3, :5] = 0
        cu = 1.0 + 0.3 * rng.random((nx + 1, ny))
        cv = 1.0 + 0.3 * rng.random((nx, ny + 1))
        lam = np.asarray(lam, dtype=np.float64)
        rhs = rng.standard_normal((lam.size, nx, ny)) * mask
        solver = mg.MG_Helmholtz(1.0, 1.3, nx, ny, cu, cv, lambd=lam.reshape(-1, 1, 1), mask=mask,
                                 niter_bottom=nb, max_ite=ite, dtype=np.float64)
        f = np.asarray(solver.solve(rhs))
        out.update({f"{tag}_mask": mask, f"{tag}_cu": cu, f"{tag}_cv": cv, f"{tag}_lam": lam, f"{tag}_rhs": rhs,
                    f"{tag}_f": f, f"{tag}_meta": np.array([nx, ny, nb, ite, solver.n_levels])})
    np.savez_compressed(os.path.join(HERE, "mg_golden.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
