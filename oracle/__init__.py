"""CPU oracle for the MPET assemble + solve path (TEST INFRASTRUCTURE ONLY).

This package restates, in numpy/scipy FP64, what the reference's
``MPETSolver`` computes through DOLFIN/FFC and PETSc:

* ``fem``  - P2 vector / P1 Lagrange dofmap on simplices, exact local
  tensors of the forms at src/mpet/mpet/mpetsolver.py:196-254, and the
  DOLFIN sparsity rule (dense cell block over all mixed DOFs).
* ``mpet`` - the time-step order of ``MPETSolver.step`` (mpetsolver.py:317-379)
  and ``solve_direct`` (mpetsolver.py:382-462), DirichletBC row replacement
  and the symmetric elimination of bc_symmetric.py:11-22, with SuperLU
  (``scipy.sparse.linalg.splu``) in place of MUMPS.
* ``krylov`` - preconditioned MINRES and a smoothed-aggregation AMG used as
  the CPU baseline of the iterative GPU path.

Parity pinning: FEniCS/DOLFIN/PETSc cannot be imported on this machine, so
there are no golden vectors produced by the reference itself.  The oracle is
pinned against the reference's own tests instead: the convergence-rate
thresholds of src/mpet/test/test_convergence_mpetsolver.py:234-239 (2D,
theta = 1 and theta = 0.5) and the sparsity counts of the Kuhn cube.  Bitwise
agreement with DOLFIN's DOF numbering is unpinned.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference arms may import this package; the product path never does.
"""
