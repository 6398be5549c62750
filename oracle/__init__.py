"""CPU oracle for the scikit-topt density-method hot path (TEST INFRASTRUCTURE).

This package is a NumPy/SciPy restatement of the reference algorithm
(kevin-tofu/scikit-topt 0.3.9).  It exists only to check the GPU product:
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it, and nothing in
``sktopt_gb300`` does.  Each function cites the reference file:line it
follows (paths are relative to the reference project root).

Parity status
-------------
* The reference cannot be imported here: scikit-fem, PyAMG and numba are
  not installed and there is no network.  The third-party arithmetic the
  reference delegates to is restated from its published behaviour:

  - scikit-fem 11.x (pyproject.toml:18): ``MeshHex.init_tensor`` node and
    element numbering, ``ElementHex1`` / ``ElementTetP1`` bases with exact
    Gauss quadrature, ``asm`` COO->CSR with duplicates summed and sorted
    columns, ``enforce`` (rows and columns of the Dirichlet DOFs zeroed,
    unit diagonal, RHS set to the prescribed value), ``condense``/``solve``.
  - SciPy 1.18 (present here): ``spsolve``, ``splu``, ``cg``, ``cKDTree``.

* The reference's own tests pin no numerical results (they check
  ``isfinite`` and stepwise self-consistency only).  The oracle is pinned
  against the known answers of ``scikit-topt/tests/test_scheduler.py`` and
  against analytic properties (rigid-body null space of element matrices,
  exact volumes, symmetric positive definiteness, filter row sums, finite
  differences).  Everything at the scikit-fem boundary is therefore
  **parity unpinned**: it follows the restatement, not a run of the
  reference.
"""
