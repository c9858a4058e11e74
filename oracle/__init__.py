"""ORACLE — test infrastructure only.

CPU restatements of the reference's algorithms, used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker.  The product package never imports this package.
"""
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent


def build_c() -> None:
    """Compile the oracle's C restatements (none yet besides Python ones)."""
    return None
