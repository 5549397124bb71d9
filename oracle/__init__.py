"""CPU oracle for the cell-assembly path (test infrastructure only).

This package is a plain numpy restatement of scikit-fem 12.0.1's cell
assembly: tensor meshes, DOF numbering, quadrature, reference bases,
affine / isoparametric mappings, ``BilinearForm._assemble`` /
``LinearForm._assemble`` and the COO -> CSR step with ``eliminate_zeros``.
Each function cites the reference file:line it follows.

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg import it.  The product path
(``skfem_gb300``) never imports this package and has no CPU fallback.

Parity pinning: ``tests/golden/make_golden.py`` runs the real reference on
small cases and stores (indptr, indices, data, b, quadrature) as ``.npz``
fixtures; ``tests/test_oracle_golden.py`` checks this restatement against
them.
"""

from .skfem_oracle import *  # noqa: F401,F403
