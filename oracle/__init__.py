"""CPU oracle for the scikit-topt density-method hot path (TEST INFRASTRUCTURE).

This package is a NumPy/SciPy restatement of the reference algorithm
(kevin-tofu/scikit-topt 0.3.9).  It exists only to check the GPU product:
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it, and nothing in
``sktopt_gb300`` does.  Each function cites the reference file:line it
follows (paths are relative to the reference project root).

Parity status
-------------
* Pinned to the reference's own code: everything the reference computes
  with NumPy/SciPy itself.  ``tests/golden/make_ref_fixtures.py`` imports the
  unmodified reference sources (inert stand-ins replace the missing
  scikit-fem, PyAMG, numba, matplotlib and meshio) and writes fixtures from
  its projection, derivatives, interpolation and volumes, orientation fixes,
  element sets, schedules, Gaussian filter, OC bisection, log update, both
  ``rho_update`` hooks and whole runs of its driver loop
  (``DensityMethod._optimize_impl``) with this oracle's FEM plugin;
  ``tests/test_cpu_ref_pinned.py`` checks this package against them.
* Parity unpinned: the arithmetic the reference delegates to scikit-fem
  11.x (pyproject.toml:18), restated here from its published behaviour --
  ``MeshHex.init_tensor`` node and element numbering, ``ElementHex1`` /
  ``ElementTetP1`` bases with exact Gauss quadrature, ``asm`` COO->CSR with
  duplicates summed and sorted columns, ``enforce`` (rows and columns of the
  Dirichlet DOFs zeroed, unit diagonal, RHS set to the prescribed value),
  ``condense``/``solve``, facet integrals, the nodal Helmholtz system.  Those
  parts are pinned by analytic properties (rigid-body null space of element
  matrices, exact volumes, symmetric positive definiteness, filter row
  sums, finite differences) and by fixtures of this restatement
  (``tests/golden/make_golden.py``).
* Third-party, absent from the reference tree: PyAMG (pyproject.toml:23,
  ``pyamg >=5.2.1,<6.0.0``), whose ``smoothed_aggregation_solver`` the
  reference's ``cg_pyamg`` option builds (solver_elastic.py:94-103).
  ``amg.py`` (with the serial kernels in ``csrc/amg.c``) restates its
  published algorithm with the 5.x defaults.  Its parity is on the solve:
  the preconditioned CG reaches the reference's stopping rule and agrees
  with the direct solve; the hierarchy follows PyAMG's structure but is
  not compared with PyAMG's (not installable here).
* SciPy 1.18 (present here) supplies ``spsolve``, ``splu``, ``cg`` and
  ``cKDTree`` as in the reference.
"""
