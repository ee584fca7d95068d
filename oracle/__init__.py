"""CPU oracle for the HSS direct-solver hot path -- TEST INFRASTRUCTURE ONLY.

This package is a plain NumPy/SciPy FP64 restatement of the MATLAB reference
(EduardoCorona84/HSSC_DirectSolver).  Each function names the reference
file:line it follows.  It exists to check the CUDA library, never to be the
thing that is measured or shipped: only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import
it.  The product package (``hssc_directsolver_gb300``) never imports it and
fails loudly when its CUDA library is missing.

Parity status: the reference is MATLAB and cannot run here (no MATLAB/Octave),
and its own tests hold no golden vectors -- they print relative errors against
dense solves.  The oracle is pinned to those test criteria (apply / inverse
apply errors against dense products and dense solves, at the reference test
parameters) and to the reference's documented sample error magnitudes; the
MATLAB builtins it replaces (qr, inv, mldivide, svd, rand) are restated with
deterministic, documented algorithms.  See tests/test_oracle_*.py.
"""
