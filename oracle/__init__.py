"""CPU oracles for the STRIDE (DPR4 v3) and PLDT v5 decoders -- test
infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker.  The product path
(``meshpress_gb300``) never imports it.
"""
from .oracle import (OracleError, bitcodec_read, decode, decode_mt,  # noqa: F401
                     decode_v5, parse_header, parse_header_v5, build, library_path, side_table,
                     tables_v5)
