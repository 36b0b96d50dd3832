"""ORACLE — CPU test infrastructure for the S-PGO LM step.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package, and only as the checker or the timed CPU baseline.
The product path (the ``s-pgo_gb300`` package and its CUDA library) never
imports, links or runs anything here.
"""
