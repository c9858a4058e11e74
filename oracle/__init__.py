"""ORACLE — test infrastructure only.

CPU restatements of the reference's algorithms (and, for the Monte Carlo that
the reference cannot run, of the builder's algorithm), used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker.  The product package never imports this package.
"""
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
MC_LIB = BUILD_DIR / "libpvd_mc_oracle.so"


def build_c(force: bool = False) -> Path:
    """Compile the C restatements (gcc, strict IEEE: no FP contraction, no fast-math)."""
    src = ORACLE_DIR / "mc_oracle.c"
    if not force and MC_LIB.exists() and MC_LIB.stat().st_mtime >= src.stat().st_mtime:
        return MC_LIB
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = MC_LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", str(src),
           "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    tmp.replace(MC_LIB)
    return MC_LIB
