"""CPU oracle for the lapy_gb300 FEM path — TEST INFRASTRUCTURE ONLY.

A NumPy/SciPy restatement of the reference (Deep-MI/LaPy) functions on the
path: cotangent stiffness / mass assembly (lapy/solver.py), the shift-invert
eigensolve, Poisson and heat solves (SciPy eigsh / splu with the reference's
arguments), and the heat-method geodesic pieces (lapy/diffgeo.py).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package, and only as the reference the results are compared
with or as the timed CPU baseline.  The product (``lapy_gb300``) never calls it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the reference itself on
the same inputs and stores its outputs under ``tests/golden/``; the CPU tests
check this oracle against them and against the golden values of the
reference's own test suite (lapy/utils/tests/expected_outcomes.json).
"""

from .lapy_oracle import *  # noqa: F401,F403
