"""Oracle for the projection hot path: TEST INFRASTRUCTURE ONLY.

``oracle.restate`` wraps the plain-C restatement of the reference algorithms
(``oracle/restate.c``); ``oracle/ref`` holds the harness that compiles the
reference's own headers (where the reference sources exist) to produce the
golden fixtures under ``tests/golden``. Only the tests, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg may import this package; the product
library (``carpio_gb300``) never does.
"""
