"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``mt_oracle.cpp`` into ``oracle/liboracle.so`` with OpenMP and with
floating-point contraction disabled (``-ffp-contract=off``), so that every
floating-point operation is rounded once, in the reference source's order, and
the result bits do not depend on the host compiler or CPU (x86_64 and
aarch64 alike).
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
SOURCE = ORACLE_DIR / "mt_oracle.cpp"
LIBRARY = ORACLE_DIR / "liboracle.so"
DEPS = [SOURCE, ORACLE_DIR.parent / "meshtryoshka_gb300" / "csrc" / "mc_tables.h"]


def build(force: bool = False) -> Path:
    if not force and LIBRARY.exists():
        t = LIBRARY.stat().st_mtime
        if all(d.stat().st_mtime <= t for d in DEPS):
            return LIBRARY
    cxx = os.environ.get("CXX", "g++")
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [
        cxx,
        "-O2",
        "-std=c++20",
        "-fopenmp",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-fPIC",
        "-shared",
        str(SOURCE),
        "-o",
        str(tmp),
    ]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout + proc.stderr)
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force=True))
