"""CPU oracle for the VarDyn 4D-Var inner loop (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
import it. It is a float64 NumPy/SciPy restatement of the reference's algorithms,
with every function citing the reference file:line it follows.

Parity pins: restatements checked against golden vectors produced by the
reference's own source files, loaded unmodified and executed with a NumPy
stand-in for ``jax`` (``tests/golden/gen_golden*.py``):
- the QG 1.5-layer family (``qg1l``, ``qg1l_tiles``, ``qg1l_trac``);
- the spectral and multigrid Helmholtz solvers (``helmholtz_dst``,
  ``helmholtz_mg``);
- the shallow-water model and the QG projector (``sw``, ``qg_ml``);
- both observation operators (``obsop``);
- the Gaussian, wave-packet and wavelet bases (``basis``).

The tangent/adjoint restatements are pinned by finite differences of the
pinned forwards and by dot-product tests. The 4D-Var cost/gradient assembly
(``fourdvar``) is pinned by properties only: producing the reference's needs
jax's vjp.
"""
