"""CPU oracle for the MFLOPS3D-MD hot path -- TEST INFRASTRUCTURE ONLY.

This package is a plain FP64 NumPy/SciPy restatement of the reference
algorithms (pums974/MFLOPS3D-MD, Fortran 90).  It exists to check the CUDA
product path; nothing in the product imports it.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and
its ``--impl reference`` arm) may use it.

Parity status
-------------
The reference cannot be compiled in this environment (Fortran 90 + LAPACK +
MPI + PETSc, no Fortran compiler) and ships no stored golden vectors.  The
oracle is therefore *pinned* only to the reference's own analytic
known-answer recipes:

* ``src/main/test_solver_3d.f90:218-258`` (x^9 + y^9 + x*y, sigma = 2,
  Dirichlet, relative L2 error ``err`` at ``:310-361``);
* ``src/main/test_derivatives.f90:69-98,135-206`` (sin/cos field, scheme
  order by grid doubling);
* the Neumann extrapolation and null-mode recipes of ``test_solver_3d``.

Bit-level parity with the Fortran binary is unpinned (no binary can be run
here); the product is held to the oracle within the tolerances stated in
each test.

Modules
-------
``mesh``         1D grids (reference arcsin grid and the tanh grid).
``derivatives``  compact first/second derivatives (``class_derivatives``).
``solver``       matrix-diagonalisation Poisson/Helmholtz (``class_solver_3d``).
``md``           influence-matrix multidomain coupling (``class_md`` + ``class_field``).
``filter``       least-squares B-spline filter (``class_filter`` + FITPACK routines).
``les``          Smagorinsky / WALE / sigma eddy viscosity (``class_navier_3D``).
"""
