"""CPU oracle for the lineax solve path — TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, what the reference lineax solvers compute,
so that the GPU engine can be checked against it.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import it, and only to check results or as the timed CPU baseline — the
GPU product path never calls into it.

* ``dense``  — LU / Cholesky / QR / triangular solves.  The reference reaches
  LAPACK getrf/getrs, potrf/potrs, geqrf/ormqr and trsm through
  ``jax.scipy.linalg`` (lineax/_solver/lu.py:53,64; cholesky.py:60,74;
  qr.py:62-90; triangular.py:81).  On JAX's CPU backend those LAPACK kernels
  are bound to the ones SciPy ships (scipy.linalg.cython_lapack), so SciPy's
  LAPACK is used here directly.
* ``krylov`` — statement-for-statement NumPy restatements of lineax's CG
  (lineax/_solver/cg.py:114-227) and GMRES (lineax/_solver/gmres.py:106-413),
  in FP64.
* ``getf2.c`` — the unblocked right-looking LU recurrence in plain C with
  explicit fma(); the GPU plain-FP64 LU is designed to reproduce it bit for
  bit, so it pins the factor and the pivots exactly.

Parity pin: JAX/lineax cannot be imported in this environment (neither here
nor on the GPU host), so the oracle is pinned against the known-answer tests
of the reference's own test-suite (extracted into tests/golden/ by
tests/golden/make_golden.py) and against SciPy's LAPACK, which is the routine
JAX's CPU backend calls.
"""
