"""CPU oracle for the tt-fort sweep hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library and its
Python mirror in ``tt-fort_gb300/ttgpu``) imports, links or executes this
package.  It is used by ``tests/`` as the checker, by
``__graft_entry__.smoke()`` as the checker, and by ``bench.py`` as the timed
CPU baseline (the ``cpu_baseline`` leg and ``--impl reference``).

Every function restates the reference Fortran algorithm it names (file:line
inside oseledets/tt-fort) with numpy/scipy (LAPACK/BLAS) doing the dense
arithmetic.  All arrays are flat and column-major, exactly like the
reference's ``real(8) x(*)`` arguments; shapes are recovered with
``reshape(..., order='F')``.

Parity pins (what the oracle itself is checked against, in ``tests/``):
  * exact-diagonalisation eigenvalues of the d=20 Heisenberg chain stored in
    the reference fixture ``Heisen_20.sdv`` (``tests/golden/heisen20_ed.json``);
  * the closed-form answer of the reference fixture ``test_eye_ksl.dat``
    (operator i*I, one KSL step must return exp(i*tau)*y0);
  * dense scipy references (``eigh``, ``expm``, ``solve``) at small d.
"""
