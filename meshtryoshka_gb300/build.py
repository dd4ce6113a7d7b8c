"""Builds ``libmtgb.so``, the sm_103a CUDA library behind the C ABI in
``include/meshtryoshka_gb300.h``.

Every ``csrc/*.cu`` translation unit is compiled by ``nvcc`` in parallel for
``sm_103a`` only, then linked into one shared library in the package
directory (in-tree, never installed). The library links the shared CUDA
runtime so it shares one runtime instance with PyTorch.

Run ``python -m meshtryoshka_gb300.build`` (or call :func:`build`) to
(re)build; the build is skipped when the library is newer than every source.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
CSRC = PACKAGE_DIR / "csrc"
INCLUDE = PACKAGE_DIR.parent / "include"
BUILD_DIR = PACKAGE_DIR / "_build"
LIBRARY = PACKAGE_DIR / "libmtgb.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
    "-diag-suppress=177",
]

# Translation units whose floating-point results must equal the reference
# kernels' source evaluated operation by operation: no multiply-add
# contraction anywhere in them. The compositing kernels keep contraction for
# speed and spell every result-defining operation with explicit
# __fmul_rn / __fadd_rn intrinsics instead.
UNCONTRACTED = {"extraction", "raster_front", "explicit", "subdivision"}


def find_nvcc() -> str:
    for candidate in (
        os.environ.get("NVCC"),
        shutil.which("nvcc"),
        "/usr/local/cuda/bin/nvcc",
    ):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found: the meshtryoshka_gb300 CUDA library cannot be built")


def cuda_lib_dir(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent / "lib64"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def headers() -> list[Path]:
    # This file is a dependency too: a change of flags rebuilds everything.
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(
            "command failed: " + " ".join(cmd) + "\n" + proc.stdout + proc.stderr
        )


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the CUDA library; returns its path."""
    nvcc = find_nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = sources()
    hdrs = headers()
    jobs = []
    objects = []
    for src in srcs:
        obj = BUILD_DIR / (src.stem + ".o")
        objects.append(obj)
        if force or _stale(obj, [src, *hdrs]):
            fmad = ["-fmad=false"] if src.stem in UNCONTRACTED else []
            jobs.append(
                [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *fmad, f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)]
            )
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(pool.map(_run, jobs))
    if force or jobs or _stale(LIBRARY, objects):
        libdir = cuda_lib_dir(nvcc)
        tmp = LIBRARY.with_suffix(".so.tmp")
        _run(
            [
                nvcc,
                *ARCH_FLAGS,
                "-shared",
                "-cudart",
                "shared",
                "-o",
                str(tmp),
                *map(str, objects),
                f"-L{libdir}",
                "-Xlinker",
                f"-rpath={libdir}",
            ]
        )
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
