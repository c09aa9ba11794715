"""CPU oracle for the petgem forward-modelling hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
package: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may use it, and only as the reference results that outputs
are compared with (or as the timed CPU baseline), never as the
implementation being measured.

The oracle is a plain numpy/scipy restatement of the reference algorithms,
function by function, each citing the petgem file:line it follows:

* ``oracle.basis``     -- hierarchical H(curl) basis on the tetrahedron
                          (petgem/hvfem.py:319-1052) and the quadrature
                          used to integrate it (hvfem.py:1055-1610).
* ``oracle.topology``  -- edges / faces / faces-edges / DOF numbering /
                          PEC boundary DOFs (petgem/mesh.py, petgem/vectors.py,
                          hvfem.py:15-98).
* ``oracle.fem``       -- Jacobian, orientation, elemental mass/stiffness,
                          COO assembly, PEC, point-dipole RHS, receiver
                          interpolation (hvfem.py, solver.py, postprocessing.py).
* ``oracle.solve``     -- scipy stand-ins for the PETSc KSP solve
                          (solver.py:584-594).
* ``oracle.adjoint``   -- receiver-misfit gradient (adjoint) and central
                          finite differences of the oracle forward model.

Parity pinning: the oracle is checked against golden vectors produced by
running the reference's own functions (``tests/golden/make_golden.py``) and
against the topology asserts of the reference's ``tests/test_mesh.py:31-36``.
"""
