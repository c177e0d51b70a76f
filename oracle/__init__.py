"""CPU oracle for the resident light-stack hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in NumPy, the reference's
CPU algorithms for calibration, star detection, triangle registration,
warping, rejection and integration (each function cites the reference
file:line it follows).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it, and
only as the checker or as the timed CPU baseline.  The product path
(``glass_gb300``) never imports, calls or falls back to anything here.

Pinning: ``tests/test_oracle_golden.py`` checks every function here against
golden vectors produced by the reference's own code (``tests/golden/``,
generated by ``tests/golden/make_golden.py`` from the reference sources) and
against the hand-computed known answers in the reference's tests.
"""
