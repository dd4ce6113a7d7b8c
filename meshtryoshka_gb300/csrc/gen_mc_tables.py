"""Regenerate ``mc_tables.h`` from the reference's marching-cubes tables.

The triangulation table has to be identical to the one the reference uses
(``triangle_extraction/constants.slang:1-158``): face topology is compared
bit-for-bit, and the table fixes which edges form each triangle and in which
order. The table is stored here in a different, GPU-friendly encoding:

* ``MT_MC_CASE_COUNT[c]``  number of edge ids emitted for cube code ``c``
  (``FIRST[c + 1] - FIRST[c]``, always a multiple of 3, at most 15);
* ``MT_MC_CASE_EDGES[c]``  the edge ids packed as 4-bit nibbles, edge ``j``
  of the case in bits ``[4j, 4j + 4)`` (one 64-bit load per case);
* ``MT_MC_EDGE_OWNER[e]``  which upper neighbour owns edge ``e`` (-1 = the
  voxel itself, 0..5 = slot in the ``neighbors`` table);
* ``MT_MC_EDGE_AXIS[e]``   the axis (vertex type) of edge ``e``.

It also records FNV-1a checksums of the reference's flat ``FIRST`` / ``IDS``
arrays so a test can show the encoding round-trips to the same table.

Usage: ``python gen_mc_tables.py <path to reference constants.slang>``.
"""

import re
import sys
from pathlib import Path


def parse(src: str, name: str) -> list[int]:
    m = re.search(name + r"\[[^\]]*\](?:\[[^\]]*\])?\s*=\s*\{(.*?)\};", src, re.S)
    if m is None:
        raise ValueError(f"table {name} not found")
    return [int(x) for x in re.findall(r"-?\d+", m.group(1))]


def fnv1a(values: list[int]) -> int:
    h = 0xCBF29CE484222325
    for v in values:
        for byte in int(v & 0xFFFFFFFF).to_bytes(4, "little"):
            h ^= byte
            h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def main(path: str) -> None:
    src = Path(path).read_text()
    first = parse(src, "FIRST_MARCHING_CUBES_ID")
    ids = parse(src, "MARCHING_CUBES_IDS")
    loc = parse(src, "MC_EDGE_LOCATIONS")
    assert len(first) == 257 and len(ids) == first[-1]
    # The reference declares MC_EDGE_LOCATIONS[12][4] but initialises two
    # entries per row; only (owner, axis) are read.
    assert len(loc) == 24
    counts, packed = [], []
    for c in range(256):
        edges = ids[first[c] : first[c + 1]]
        assert len(edges) % 3 == 0 and len(edges) <= 15
        word = 0
        for j, e in enumerate(edges):
            assert 0 <= e < 12
            word |= e << (4 * j)
        counts.append(len(edges))
        packed.append(word)
    owners = [loc[2 * e] for e in range(12)]
    axes = [loc[2 * e + 1] for e in range(12)]

    out = []
    out.append("// Generated by gen_mc_tables.py; do not edit by hand.")
    out.append("// Marching-cubes triangulation in the reference's edge convention")
    out.append("// (triangle_extraction/constants.slang:1-158), re-encoded per case.")
    out.append("#pragma once")
    out.append("#include <stdint.h>")
    out.append("")
    out.append(f"#define MT_MC_FIRST_FNV1A 0x{fnv1a(first):016x}ull")
    out.append(f"#define MT_MC_IDS_FNV1A 0x{fnv1a(ids):016x}ull")
    out.append(f"#define MT_MC_TOTAL_IDS {first[-1]}")
    out.append("")
    # Brace-free value lists, so the same data can initialise host arrays and
    # __constant__ device arrays.
    out.append("#define MT_MC_CASE_COUNT_VALUES \\")
    for r in range(0, 256, 16):
        out.append("  " + ", ".join(f"{x:2d}" for x in counts[r : r + 16]) + ", \\")
    out.append("")
    out.append("")
    out.append("#define MT_MC_CASE_EDGES_VALUES \\")
    for r in range(0, 256, 4):
        out.append("  " + ", ".join(f"0x{x:015x}ull" for x in packed[r : r + 4]) + ", \\")
    out.append("")
    out.append("")
    out.append("#define MT_MC_EDGE_OWNER_VALUES " + ", ".join(str(x) for x in owners))
    out.append("#define MT_MC_EDGE_AXIS_VALUES " + ", ".join(str(x) for x in axes))
    out.append("")
    target = Path(__file__).parent / "mc_tables.h"
    target.write_text("\n".join(out))
    print(f"wrote {target}")


if __name__ == "__main__":
    main(sys.argv[1])
