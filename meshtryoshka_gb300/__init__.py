"""GB300-native (sm_103a) implementation of Meshtryoshka's per-step render path.

Subpackages mirror the reference's Python surface:

* :mod:`meshtryoshka_gb300.triangle_extraction` — sparse-voxel extraction and
  per-step marching cubes over several level sets;
* :mod:`meshtryoshka_gb300.triangle_rasterization` — tile-based multi-shell
  triangle rasterization with NeuS-style compositing, fused and explicit modes.

Both call hand-written CUDA kernels through the C ABI declared in
``include/meshtryoshka_gb300.h`` (``libmtgb.so``, built in-tree by
:mod:`meshtryoshka_gb300.build`).
"""

import importlib
import sys

__version__ = "0.1.0"


def install_aliases() -> None:
    """Make ``import triangle_extraction`` / ``import triangle_rasterization``
    resolve to this package's implementations (drop-in for the trainer)."""
    for name in ("triangle_extraction", "triangle_rasterization"):
        sys.modules[name] = importlib.import_module(f"{__name__}.{name}")
