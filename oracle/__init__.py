"""CPU oracle for NEUWON's ``Model.advance()`` hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain FP64 numpy (``reference_step``) and in C
(``cpu_step.c``), the reference's algorithm for one staggered time step.  It is
test infrastructure, never the product: only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference arm may import, link or run anything in
this directory.  The product path (``neuwon_gb300``) never calls it and fails
loudly when its CUDA library is missing.

Parity is pinned: ``tests/golden/make_golden.py`` runs the reference itself
(imported with import-only stubs for its absent third-party dependencies) and
commits its outputs as fixtures; ``tests/test_oracle_golden.py`` checks this
oracle against those fixtures and against the reference test suite's own
golden HH trace (``neuwon/rxd/tests/test_model.py:77-113``).
"""
