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
- the Gaussian, wave-packet and wavelet bases (``basis``);
- the 4D-Var cost/gradient assembly (``fourdvar``): golden J and G from the
  reference's own Variational.cost_and_grad with Model_qg1l_jax, the jax
  observation operator and Basis_gauss3d, its two jax.vjp uses taking the
  pinned adjoint restatements (``gen_golden_fourdvar.py``).

``helmholtz_masked`` (direct sparse solve of the masked Dirichlet problem the
multigrid inversion solves) equals the reference's capacitance-matrix
solutions on the ocean nodes. The tangent/adjoint restatements are pinned by
finite differences of the pinned forwards and by dot-product tests.
"""
