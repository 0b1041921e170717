"""TEST INFRASTRUCTURE ONLY: FP64 CPU oracle for odtbrain_gb300.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  The GPU product never calls it.
"""
