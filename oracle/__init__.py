"""CPU oracle for the VarDyn 4D-Var inner loop (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
import it. It is a float64 NumPy/SciPy restatement of the reference's algorithms,
with every function citing the reference file:line it follows.

Parity pin: the QG 1.5-layer forward restatement (``oracle.qg1l``) is pinned
against golden vectors produced by the reference's own ``jqgm.py`` source
executed with a NumPy stand-in for ``jax`` (``tests/golden/gen_golden.py``).
The tangent/adjoint restatements are pinned by finite differences of that
pinned forward and by dot-product tests. The observation operator and the
4D-Var cost/gradient are restatements pinned by properties only (the reference
ships no golden values and jax is not importable): parity there is unpinned.
"""
