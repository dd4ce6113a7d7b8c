"""Recipe: compile the reference's own kernel sources for the CPU.

TEST INFRASTRUCTURE ONLY. The reference's render-path kernels are Slang
(slangtorch JIT); neither slangtorch nor slangc exists here. Most of these
kernels use a C-like subset of Slang, so this recipe rewrites each source
file textually (attributes dropped, ``let``/``var`` to ``auto``, ``$for`` to
``for``, float literals suffixed, struct definitions hoisted), writes the
result under ``oracle/_ref/`` (git-ignored, never committed), and compiles it
with ``oracle/ref_shim/slang.h`` (host stand-ins for Slang types and
intrinsics) and ``oracle/ref_shim/driver.cpp`` (grid emulation and a C ABI)
into ``oracle/_ref/libref.so``.

Backward kernels: the two hand-written ones (fused intersect-and-composite
and explicit composite) are kept; the ``bwd_diff(helper)`` calls in them use
adjoints of the small helpers written by hand in ``oracle/ref_shim/autodiff_*.h``.
The backward kernels that are pure automatic differentiation (SH evaluation,
triangle vertex creation) are dropped.

The reference's module-level helpers in ``common.slang`` (64-bit indexing,
DiffTensorView load/store) are replaced by equivalents in the shim; every
kernel body is the reference's own code.

Usage: ``python oracle/build_ref.py [reference root]`` (default: the
``MESHTRYOSHKA_REFERENCE`` environment variable, else a ``reference``
checkout beside this repository). Returns without building when the
reference tree is absent.
"""

from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
OUT_DIR = ORACLE_DIR / "_ref"
SHIM_DIR = ORACLE_DIR / "ref_shim"
LIBRARY = OUT_DIR / "libref.so"
# A checkout of the reference next to this repository, when there is one.
DEFAULT_ROOT = ORACLE_DIR.parent.parent / "reference"

# (package, file) -> functions to drop (backward passes need Slang autodiff).
SOURCES = {
    ("triangle_extraction", "constants.slang"): [],
    ("triangle_extraction", "compute_vertex_occupancy.slang"): [],
    ("triangle_extraction", "count_occupancy.slang"): [],
    ("triangle_extraction", "create_voxels.slang"): [],
    ("triangle_extraction", "dilate_occupancy.slang"): [],
    ("triangle_extraction", "count_triangle_vertices.slang"): [],
    ("triangle_extraction", "create_triangle_vertices.slang"): ["create_triangle_vertices_backward"],
    ("triangle_extraction", "count_triangle_faces.slang"): [],
    ("triangle_extraction", "create_triangle_faces.slang"): [],
    ("triangle_extraction", "compute_sdf_regularizers.slang"): [],
    ("triangle_extraction", "write_occupancy.slang"): [],
    ("triangle_extraction", "upscale_occupancy.slang"): [],
    ("triangle_extraction", "upscale_parameters.slang"): [],
    ("triangle_extraction", "get_occupancy_mesh.slang"): [],
    ("triangle_rasterization", "keys.slang"): [],
    ("triangle_rasterization", "project_vertices.slang"): [],
    ("triangle_rasterization", "bound_triangles.slang"): [],
    ("triangle_rasterization", "generate_keys.slang"): [],
    ("triangle_rasterization", "delineate_tiles.slang"): [],
    ("triangle_rasterization", "evaluate_spherical_harmonics.slang"): ["evaluate_spherical_harmonics_backward"],
    ("triangle_rasterization", "intersect_and_composite.slang"): [],
    ("triangle_rasterization", "intersect.slang"): [],
    ("triangle_rasterization", "interpolate.slang"): [],
    ("triangle_rasterization", "composite.slang"): [],
}

# Hand-written backward kernels that call bwd_diff(helper)(...): the
# adjoints of those helpers come from a shim header, included right before
# the kernel.
AUTODIFF = {
    "intersect_and_composite.slang": ("intersect_and_composite_backward", "autodiff_intersect_and_composite.h"),
    "composite.slang": ("composite_backward", "autodiff_composite.h"),
}

# Files whose local/struct arrays are copied as values (aggregate returns):
# their array declarations become std::array.
ARRAY_VALUE_FILES = {"create_triangle_vertices.slang", "evaluate_spherical_harmonics.slang",
                     "upscale_parameters.slang"}

# Files that apply Slang's floating-point `%` (fmod) as `x % 1`.
FLOAT_MOD = re.compile(r"\b(\w+)\s*%\s*1\s*;")
FLOAT_MOD_FILES = {"upscale_parameters.slang"}

ATTRIBUTE = re.compile(r"^\s*\[(AutoPyBindCUDA|CUDAKernel|Differentiable|NoDiffThis|require\(cuda\)|"
                       r"BackwardDerivative\([^)]*\))\]\s*$", re.M)
FLOAT_LITERAL = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])")
SLANG_FOR = re.compile(r"\$for\s*\(\s*(\w+)\s+in\s+Range\(\s*([^,]+?)\s*,\s*([^)]+?)\s*\)\s*\)")
IMPORT = re.compile(r'^\s*import\s+"\./(\w+)\.slang"\s*;\s*$', re.M)
ARRAY_DECL = re.compile(r"\b(float3|float|int|uint|uint8_t)\s+(\w+)\s*((?:\[[^\]\n]+\])+)")


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def matching_brace(src: str, open_idx: int) -> int:
    depth = 0
    for i in range(open_idx, len(src)):
        if src[i] == "{":
            depth += 1
        elif src[i] == "}":
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced braces")


def drop_function(src: str, name: str) -> str:
    m = re.search(r"\bvoid\s+" + name + r"\s*\(", src)
    if not m:
        raise ValueError(f"function {name} not found")
    body = src.index("{", m.end())
    end = matching_brace(src, body)
    return src[: m.start()] + src[end + 1 :]


def hoist_structs(src: str) -> str:
    """Move struct definitions to the top (Slang allows use before definition)
    and terminate them with ';'."""
    structs = []
    out = src
    while True:
        m = re.search(r"\bstruct\s+(\w+)\s*(?::\s*\w+\s*)?\{", out)
        if not m:
            break
        end = matching_brace(out, m.end() - 1)
        body = out[m.end() - 1 : end + 1]
        structs.append(f"struct {m.group(1)} {body};")
        rest = out[end + 1 :]
        rest = re.sub(r"^\s*;", "", rest)
        out = out[: m.start()] + "@@STRUCT@@" + rest
    return "\n".join(structs) + "\n" + out.replace("@@STRUCT@@", "")


def to_std_array(match: re.Match) -> str:
    base, name, dims = match.group(1), match.group(2), match.group(3)
    sizes = re.findall(r"\[([^\]]+)\]", dims)
    t = base
    for s in reversed(sizes):
        t = f"std::array<{t}, {s}>"
    return f"{t} {name}"


def translate(src: str, fname: str, drops: list[str]) -> tuple[str, list[str]]:
    src = strip_comments(src)
    imports = IMPORT.findall(src)
    src = IMPORT.sub("", src)
    src = ATTRIBUTE.sub("", src)
    for name in drops:
        src = drop_function(src, name)
    src = SLANG_FOR.sub(lambda m: f"for (int {m.group(1)} = {m.group(2)}; {m.group(1)} < {m.group(3)}; ++{m.group(1)})",
                        src)
    src = re.sub(r"\blet\b", "const auto", src)
    src = re.sub(r"\bvar\b", "auto", src)
    src = re.sub(r"\bno_diff\s+", "", src)
    src = re.sub(r"\bgroupshared\b", "static", src)
    src = re.sub(r"\bMemoryOrder\.(\w+)", r"MemoryOrder::\1", src)
    src = re.sub(r"\b__atomic_or\(", "slang_atomic_or(", src)
    if fname in FLOAT_MOD_FILES:
        src = FLOAT_MOD.sub(r"std::fmod(\1, 1.0f);", src)
    src = re.sub(r"typealias\s+(\w+)\s*=\s*(\w+)\[(\w+)\]\s*;", r"using \1 = std::array<\2, \3>;", src)
    src = FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", src)
    if fname in ARRAY_VALUE_FILES:
        src = ARRAY_DECL.sub(to_std_array, src)
    src = re.sub(r",(\s*)\)", r"\1)", src)  # trailing commas in parameter / argument lists
    src = re.sub(r"\bbwd_diff\((\w+)\)\s*\(", r"bwd_diff_\1(", src)
    src = re.sub(r"\b(\w+)\.Differential\(", r"\1Diff(", src)
    src = hoist_structs(src)
    if fname in AUTODIFF:
        kernel, header = AUTODIFF[fname]
        m = re.search(r"\bvoid\s+" + kernel + r"\s*\(", src)
        src = src[: m.start()] + f'#include "{header}"\n' + src[m.start():]
    return src, imports


def generate(root: Path) -> list[Path]:
    OUT_DIR.mkdir(exist_ok=True)
    written = []
    for (pkg, fname), drops in SOURCES.items():
        path = root / pkg / fname
        text, imports = translate(path.read_text(), fname, drops)
        stem = fname.removesuffix(".slang")
        header = [f"// Rewritten from {pkg}/{fname} of the reference by oracle/build_ref.py; not committed."]
        for imp in imports:
            if imp != "common":
                header.append(f'#include "{pkg}__{imp}.inc"')
        target = OUT_DIR / f"{pkg}__{stem}.inc"
        target.write_text("\n".join(header) + "\n" + text)
        written.append(target)
    return written


def reference_root() -> Path:
    return Path(os.environ.get("MESHTRYOSHKA_REFERENCE", DEFAULT_ROOT))


def build(root: Path | str | None = None, force: bool = False) -> Path | None:
    root = Path(root) if root else reference_root()
    if not (root / "triangle_extraction").is_dir():
        return None
    driver = SHIM_DIR / "driver.cpp"
    deps = [driver, *sorted(SHIM_DIR.glob("*.h")), Path(__file__)]
    if not force and LIBRARY.exists() and all(d.stat().st_mtime <= LIBRARY.stat().st_mtime for d in deps):
        return LIBRARY
    generate(root)
    cxx = os.environ.get("CXX", "g++")
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [cxx, "-std=c++23", "-O1", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-pthread",
           f"-I{OUT_DIR}", f"-I{SHIM_DIR}", str(driver), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("reference kernel build failed:\n" + proc.stderr[-6000:])
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
