"""CPU checks of the oracle (no GPU): the MC tables against the reference's,
and the oracle's restatement of the reference loops against the
first-principles definitions in ``semantics.py``."""

from __future__ import annotations

import os
import re

import numpy as np
import pytest

from oracle import oracle
from tests import semantics

from oracle import build_ref

REFERENCE_CONSTANTS = str(build_ref.reference_root() / "triangle_extraction" / "constants.slang")

# FNV-1a checksums of the reference's FIRST_MARCHING_CUBES_ID[257] and
# MARCHING_CUBES_IDS[2460] (triangle_extraction/constants.slang:1-142),
# recorded by meshtryoshka_gb300/csrc/gen_mc_tables.py.
FIRST_FNV1A = 0x5D8AF64EA65875FB
IDS_FNV1A = 0x2D8170C237B01F17


def test_mc_tables_round_trip_to_reference_checksums():
    first, ids = oracle.mc_checksums()
    assert first == FIRST_FNV1A
    assert ids == IDS_FNV1A


@pytest.mark.skipif(not os.path.exists(REFERENCE_CONSTANTS), reason="reference tree not mounted")
def test_mc_tables_match_reference_file():
    src = open(REFERENCE_CONSTANTS).read()

    def parse(name):
        m = re.search(name + r"\[[^\]]*\](?:\[[^\]]*\])?\s*=\s*\{(.*?)\};", src, re.S)
        return [int(x) for x in re.findall(r"-?\d+", m.group(1))]

    def fnv(values):
        h = 0xCBF29CE484222325
        for v in values:
            for b in int(v & 0xFFFFFFFF).to_bytes(4, "little"):
                h = ((h ^ b) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
        return h

    assert fnv(parse("FIRST_MARCHING_CUBES_ID")) == FIRST_FNV1A
    assert fnv(parse("MARCHING_CUBES_IDS")) == IDS_FNV1A


def _random_grid(rng, shape, density):
    i, j, k = shape
    return semantics.pack(rng.random((i, j, k)) < density)


GRIDS = [
    ("single_voxel", lambda rng: semantics.pack(np.pad(np.ones((1, 1, 1), bool), ((1, 2), (2, 1), (3, 28))))),
    ("random_sparse", lambda rng: _random_grid(rng, (5, 6, 64), 0.1)),
    ("random_dense", lambda rng: _random_grid(rng, (4, 3, 96), 0.6)),
    ("full", lambda rng: semantics.pack(np.ones((3, 4, 64), bool))),
    ("empty", lambda rng: semantics.pack(np.zeros((3, 3, 32), bool))),
    ("bit31_edges", lambda rng: semantics.pack(
        (np.arange(96)[None, None, :] % 32 >= 30) & (rng.random((4, 4, 96)) < 0.7))),
    ("one_word", lambda rng: _random_grid(rng, (2, 2, 32), 0.5)),
]


@pytest.mark.parametrize("name,make", GRIDS, ids=[g[0] for g in GRIDS])
def test_oracle_extract_voxels_matches_definition(name, make):
    occ = make(np.random.default_rng(7))
    got = oracle.extract_voxels(occ)
    want = semantics.voxels(occ)
    np.testing.assert_array_equal(got.vertices, want[0])
    np.testing.assert_array_equal(got.neighbors, want[1])
    np.testing.assert_array_equal(got.lower_corners, want[2])
    np.testing.assert_array_equal(got.upper_corners, want[3])
    np.testing.assert_array_equal(got.indices, want[4])


@pytest.mark.parametrize("d", [1, 2, 3, 7])
def test_oracle_dilate_matches_definition(d):
    occ = _random_grid(np.random.default_rng(d), (9, 8, 96), 0.01)
    np.testing.assert_array_equal(oracle.dilate_occupancy(occ, d), semantics.dilate(occ, d))


def test_oracle_scans():
    rng = np.random.default_rng(0)
    x = rng.integers(0, 4, 1000).astype(np.int32)
    np.testing.assert_array_equal(oracle.exclusive_cumsum(x), np.concatenate(([0], np.cumsum(x)[:-1])))
    np.testing.assert_array_equal(oracle.inclusive_cumsum_i64(x), np.cumsum(x.astype(np.int64)))


def _sphere_scene(n=32, levels=(0.04, 0.0, -0.04)):
    from meshtryoshka_gb300 import synthetic
    import torch

    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    d = np.sqrt(x * x + y * y + z * z) - 0.5
    occ = semantics.pack(np.abs(d) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    rng = np.random.default_rng(0)
    sdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    sh = rng.uniform(0, 1, (4, len(p), 3)).astype(np.float32)
    del synthetic, torch
    return vox, sdf, sh, np.array(levels, np.float32)


def test_oracle_tessellation_properties():
    """Every face references three vertices of its own shell, lying on edges
    of the face's voxel, with the interpolated sdf equal to the level set."""
    vox, sdf, sh, ls = _sphere_scene()
    tri = oracle.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, ls)
    assert tri.faces.shape[0] > 100
    assert (tri.faces >= 0).all()
    vb = np.concatenate(([0], tri.vertex_boundaries))
    fb = np.concatenate(([0], tri.face_boundaries))
    K = vox.grid_shape[2]
    J = vox.grid_shape[1]
    for s in range(len(ls)):
        f = tri.faces[fb[s]:fb[s + 1]]
        assert ((f >= vb[s]) & (f < vb[s + 1])).all()
        np.testing.assert_allclose(tri.signed_distances[vb[s]:vb[s + 1]], ls[s], atol=2e-6)
        # The three vertices lie in the closed cube of the face's voxel.
        lin = tri.voxel_indices[fb[s]:fb[s + 1]].astype(np.int64)
        vi, vj, vk = lin // (J * K), (lin // K) % J, lin % K
        pos = tri.vertices[f]  # [F, 3, 3] as (k, j, i) / extent
        scale = np.array([K, J, vox.grid_shape[0]], np.float64)
        cell = pos * scale
        lo = np.stack((vk, vj, vi), -1)[:, None, :]
        assert (cell >= lo - 1e-4).all() and (cell <= lo + 1 + 1e-4).all()
