"""The reference's two CUB extensions, built as they are, for timing beside
this library's scan and sorts on the same GPU.

The reference wraps ``cub::DeviceScan::ExclusiveSum``
(triangle_extraction/compute_exclusive_cumsum.cu:8-39) and
``cub::DeviceRadixSort::SortPairs`` over all 64 key bits
(triangle_rasterization/sort_keys.cu:215-270) as torch C++ extensions; they
are the only parts of its render path that run on this GPU (the rest is
Slang, whose compiler is not available). This is test and measurement
infrastructure, never part of the product path.

* ``stage()`` copies the two source files from a reference checkout into
  ``oracle/_ref/cub/`` (git-ignored, never committed), so that a machine
  without the checkout can build them; a no-op without a checkout.
* ``load()`` builds the staged sources with ``torch.utils.cpp_extension``
  for sm_103a (build files under ``oracle/_ref/cub/build``) and returns the
  two extension modules, or None when nothing is staged.
"""

from __future__ import annotations

import os
import shutil
from pathlib import Path

from . import build_ref

STAGE = Path(__file__).resolve().parent / "_ref" / "cub"
SOURCES = {
    "compute_exclusive_cumsum": ("triangle_extraction", "compute_exclusive_cumsum.cu"),
    "sort_keys": ("triangle_rasterization", "sort_keys.cu"),
}


def stage() -> bool:
    root = build_ref.reference_root()
    if not all((root / pkg / name).exists() for pkg, name in SOURCES.values()):
        return False
    STAGE.mkdir(parents=True, exist_ok=True)
    for pkg, name in SOURCES.values():
        src, dst = root / pkg / name, STAGE / name
        if not dst.exists() or dst.read_bytes() != src.read_bytes():
            shutil.copyfile(src, dst)
    return True


def staged() -> bool:
    return all((STAGE / name).exists() for _, name in SOURCES.values())


def _load_one(module: str, name: str, verbose: bool):
    from torch.utils import cpp_extension

    directory = STAGE / "build" / module
    directory.mkdir(parents=True, exist_ok=True)
    return cpp_extension.load(
        name=f"reference_{module}", sources=[str(STAGE / name)], build_directory=str(directory),
        extra_cuda_cflags=["-O3", "-gencode", "arch=compute_103a,code=sm_103a"], verbose=verbose)


def load(verbose: bool = False):
    """(scan module, sort module) built for sm_103a (the two builds in
    parallel), or None when the sources are not staged."""
    if not staged():
        return None
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        futures = [pool.submit(_load_one, module, name, verbose) for module, (_, name) in SOURCES.items()]
        return tuple(f.result() for f in futures)


def build_in_background():
    """Starts load() in a thread (the builds take a minute or two) and returns
    a function that waits for it; the returned function gives None when the
    sources are not staged or the build failed."""
    import threading

    if not staged() or os.environ.get("MESHTRYOSHKA_SKIP_REFERENCE_CUB"):
        return lambda: None
    result: dict = {}

    def run():
        try:
            result["modules"] = load()
        except Exception as exc:  # reported by the caller, never fatal
            result["error"] = f"{type(exc).__name__}: {exc}"

    thread = threading.Thread(target=run, daemon=True)
    thread.start()

    def wait():
        thread.join()
        return result.get("modules")

    return wait
