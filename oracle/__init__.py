"""CPU oracle for the even-odd Wilson-clover solve -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package; the product (``chroma_gb300``) never does.
"""
from .oracle import Oracle, OracleOp, load  # noqa: F401
