"""CPU checks of the exactness arguments behind the compositing and key
speed-ups, with every float32 operation emulated one by one in numpy (IEEE
single precision, round to nearest, no fused multiply-add):

* warp-block edge exclusion: a block of pixel centres whose warp bit the
  mask kernel clears is rejected by the barycentric test's fast reject at
  every pixel centre (adversarial triangles: slivers, sub-pixel, repeated
  vertices, vertices on pixel centres, huge);
* the compositing forward's spans (edge_span): every pixel centre of a warp
  block that escapes the fast reject lies in its triangle's span;
* tile bounds with power-of-two tiles: division by 2^k equals multiplication
  by 2^-k for every float32, and the shifted integer division agrees with
  C's truncating one under max(., 0);
* the contribution list of the vertex-interpolation backward built per grid
  entry is the per-grid-vertex enumeration's list, written inside its bounds;
* the compositing forward's hit-bit reservations cover the batches each warp
  walks and together fit the bound the store is sized by.
"""

from __future__ import annotations

import numpy as np

f32 = np.float32
INF = f32(np.inf)


def _dot2(ax, ay, bx, by):
    return f32(f32(ax * bx) + f32(ay * by))


def _setup(p1, p2, p3):
    """Triangle-only part of the barycentric solve (setup_geometry)."""
    e12x, e12y = f32(p2[0] - p1[0]), f32(p2[1] - p1[1])
    e13x, e13y = f32(p3[0] - p1[0]), f32(p3[1] - p1[1])
    e23x, e23y = f32(p3[0] - p2[0]), f32(p3[1] - p2[1])
    d1212 = _dot2(e12x, e12y, e12x, e12y)
    d1223 = _dot2(e12x, e12y, e23x, e23y)
    d1213 = _dot2(e12x, e12y, e13x, e13y)
    d1313 = _dot2(e13x, e13y, e13x, e13y)
    d1323 = _dot2(e13x, e13y, e23x, e23y)
    d2323 = _dot2(e23x, e23y, e23x, e23y)
    a, b, c = abs(d1213), abs(d1223), abs(d1323)
    if a <= b and a <= c:
        denom = f32(f32(d1212 * d1313) - f32(d1213 * d1213))
    elif b <= a and b <= c:
        denom = f32(f32(d1212 * d2323) - f32(d1223 * d1223))
    elif c <= a and c <= b:
        denom = f32(f32(d1313 * d2323) - f32(d1323 * d1323))
    else:
        denom = f32(np.nan)
    dd = f32(denom + f32(1e-8))
    fast = dd > f32(2.0 ** -20) and dd < INF
    thr = -f32(dd * f32(2.0 ** -100)) if fast else -INF
    return dict(p1=p1, p2=p2, e12=(e12x, e12y), e13=(e13x, e13y), d1212=d1212, d1213=d1213, d1313=d1313,
                d1223=d1223, d1323=d1323, thr=thr, dd=dd)


def _numerators(g, px, py):
    """The three numerators of the barycentric test at pixel centres (arrays)."""
    q1x, q1y = (px - g["p1"][0]).astype(f32), (py - g["p1"][1]).astype(f32)
    q2x, q2y = (px - g["p2"][0]).astype(f32), (py - g["p2"][1]).astype(f32)
    e12x, e12y = g["e12"]
    e13x, e13y = g["e13"]

    def dot(ax, ay, bx, by):
        return ((ax * bx).astype(f32) + (ay * by).astype(f32)).astype(f32)

    d1x12, d1x13 = dot(q1x, q1y, e12x, e12y), dot(q1x, q1y, e13x, e13y)
    d2x12, d2x13 = dot(q2x, q2y, e12x, e12y), dot(q2x, q2y, e13x, e13y)

    def dop(a, x, c, y):
        return ((a * x).astype(f32) - (c * y).astype(f32)).astype(f32)

    vn = dop(g["d1313"], d1x12, g["d1213"], d1x13)
    wn = dop(g["d1212"], d1x13, g["d1213"], d1x12)
    un = dop(g["d1223"], d2x13, g["d1323"], d2x12)
    return un, vn, wn


def _edge_excludes(A, C, P, eX, eY, thr, x0, x1, y0, y1):
    """The mask kernel's exclusion by one numerator (edge_bound, edge_excludes)."""
    k = f32(2.0 ** -19)
    a = f32(f32(A * eX[0]) - f32(C * eY[0]))
    b = f32(f32(A * eX[1]) - f32(C * eY[1]))
    sx = f32(abs(f32(A * eX[0])) + abs(f32(C * eY[0])))
    sy = f32(abs(f32(A * eX[1])) + abs(f32(C * eY[1])))
    qx0, qx1 = f32(x0 - P[0]), f32(x1 - P[0])
    qy0, qy1 = f32(y0 - P[1]), f32(y1 - P[1])

    def term(c, s, q):
        return f32(f32(c * q) + f32(f32(k * s) * abs(q)))

    tx = max(term(a, sx, qx0), term(a, sx, qx1))
    ty = max(term(b, sy, qy0), term(b, sy, qy1))
    bm = f32(k * f32(f32(sx * max(abs(qx0), abs(qx1))) + f32(sy * max(abs(qy0), abs(qy1)))))
    hi = f32(f32(tx + ty) + bm)
    return bool(hi < thr)


def _block_excluded(g, x0, x1, y0, y1):
    if not g["thr"] > -INF:
        return False
    e12, e13 = g["e12"], g["e13"]
    return (_edge_excludes(g["d1313"], g["d1213"], g["p1"], e12, e13, g["thr"], x0, x1, y0, y1)
            or _edge_excludes(g["d1212"], g["d1213"], g["p1"], e13, e12, g["thr"], x0, x1, y0, y1)
            or _edge_excludes(g["d1223"], g["d1323"], g["p2"], e13, e12, g["thr"], x0, x1, y0, y1))


def _triangles(rng, n):
    out = []
    for kind in rng.integers(0, 6, n):
        c = rng.uniform(0, 200, 2)
        if kind == 0:  # small, well shaped
            p = c + rng.normal(0, 3, (3, 2))
        elif kind == 1:  # sliver
            d = rng.normal(0, 1, 2)
            d /= np.linalg.norm(d)
            p = c + rng.uniform(-20, 20, 3)[:, None] * d + rng.normal(0, 1e-3, (3, 2))
        elif kind == 2:  # repeated vertex
            p = np.stack((c, c + rng.normal(0, 5, 2), c))
        elif kind == 3:  # sub-pixel
            p = c + rng.normal(0, 0.3, (3, 2))
        elif kind == 4:  # large
            p = c + rng.normal(0, 60, (3, 2))
        else:  # vertices on pixel centres
            p = np.floor(c) + 0.5 + rng.integers(-4, 5, (3, 2)).astype(float)
        p = p.astype(f32)
        # Counter-clockwise in the sense of the back-face test (both orders
        # are exercised by the exclusion, which does not depend on it).
        out.append(p)
    return out


def test_excluded_blocks_are_fast_rejected_everywhere():
    rng = np.random.default_rng(0)
    checked = excluded = 0
    lx, ly = np.meshgrid(np.arange(8), np.arange(4))
    for p in _triangles(rng, 1500):
        g = _setup(p[0], p[1], p[2])
        lo = np.floor(p.min(0)).astype(int) - 9
        hi = np.floor(p.max(0)).astype(int) + 9
        for bx in range(lo[0] - lo[0] % 8, hi[0] + 1, 8):
            for by in range(lo[1] - lo[1] % 4, hi[1] + 1, 4):
                x0, x1 = f32(bx + 0.5), f32(bx + 7.5)
                y0, y1 = f32(by + 0.5), f32(by + 3.5)
                checked += 1
                if not _block_excluded(g, x0, x1, y0, y1):
                    continue
                excluded += 1
                px = (bx + lx + 0.5).astype(f32).ravel()
                py = (by + ly + 0.5).astype(f32).ravel()
                un, vn, wn = _numerators(g, px, py)
                rejected = (un < g["thr"]) | (vn < g["thr"]) | (wn < g["thr"])
                assert rejected.all(), (p, bx, by)
    assert checked > 10000 and excluded > checked // 4  # the exclusion is exercised


def _cull_box(g, p):
    """The accept box of the warp culling (bary.cuh: cull_box); None when open."""
    xmin, xmax = f32(p[:, 0].min()), f32(p[:, 0].max())
    ymin, ymax = f32(p[:, 1].min()), f32(p[:, 1].max())
    ext = max(f32(xmax - xmin), f32(ymax - ymin))
    if not ext < 8192 or not all(abs(v) < 1e6 for v in (xmin, xmax, ymin, ymax)) or not g["thr"] > -INF:
        return None
    e23 = (f32(p[2, 0] - p[1, 0]), f32(p[2, 1] - p[1, 1]))
    l23 = _dot2(e23[0], e23[1], e23[0], e23[1])
    worst = max(f32(g["d1212"] * g["d1313"]), f32(g["d1212"] * l23), f32(g["d1313"] * l23))
    if not g["dd"] >= f32(f32(1e-4) * worst):
        return None
    m = f32(f32(1) + f32(f32(1e-3) * ext))
    return (f32(xmin - m), f32(xmax + m), f32(ymin - m), f32(ymax + m))


def _edge_span(g, box, bx, by):
    """composite.cu edge_span: per row of the 8x4 block, the surviving column
    range (or None)."""
    if box is None:
        return [(0, 7)] * 4
    k2e = f32(2.0 ** -18)
    e12, e13 = g["e12"], g["e13"]
    edges = []
    for A, C, P, eX, eY in ((g["d1313"], g["d1213"], g["p1"], e12, e13), (g["d1212"], g["d1213"], g["p1"], e13, e12),
                            (g["d1223"], g["d1323"], g["p2"], e13, e12)):
        a = f32(f32(A * eX[0]) - f32(C * eY[0]))
        b = f32(f32(A * eX[1]) - f32(C * eY[1]))
        sx = f32(abs(f32(A * eX[0])) + abs(f32(C * eY[0])))
        sy = f32(abs(f32(A * eX[1])) + abs(f32(C * eY[1])))
        slack = f32(k2e * sx)
        with np.errstate(divide="ignore", over="ignore"):
            edges.append((a, b, sy, P, slack, f32(f32(1) / f32(a - slack)), f32(f32(1) / f32(a + slack))))
    rows = []
    for r in range(4):
        y = f32(by + f32(r))
        if not (box[2] <= y <= box[3]):
            rows.append(None)
            continue
        xl, xu, empty = box[0], box[1], False
        for a, b, sy, P, slack, inv_lo, inv_hi in edges:
            qy = f32(y - P[1])
            rr = f32(g["thr"] - f32(f32(b * qy) + f32(f32(k2e * sy) * abs(qy))))
            with np.errstate(over="ignore", invalid="ignore"):
                if a > slack:
                    q = f32(rr * (inv_lo if rr <= 0 else inv_hi))
                    pad = f32(f32(0.0625) + f32(f32(2.0 ** -16) * f32(abs(P[0]) + abs(q))))
                    xl = np.fmax(xl, f32(f32(P[0] + q) - pad))
                elif a < -slack:
                    q = f32(rr * (inv_hi if rr <= 0 else inv_lo))
                    pad = f32(f32(0.0625) + f32(f32(2.0 ** -16) * f32(abs(P[0]) + abs(q))))
                    xu = np.fmin(xu, f32(f32(P[0] + q) + pad))
                else:
                    qf = max(abs(f32(bx - P[0])), abs(f32(f32(bx + f32(7)) - P[0])))
                    empty = empty or f32(f32(f32(2.02) * slack) * qf) < rr
        c0 = max(int(np.ceil(np.fmax(f32(xl - bx), f32(-1)))), 0)
        c1 = min(int(np.floor(np.fmin(f32(xu - bx), f32(8)))), 7)
        rows.append(None if empty or c0 > c1 else (c0, c1))
    return rows


def test_forward_spans_hold_every_pixel_that_escapes_the_fast_reject():
    rng = np.random.default_rng(3)
    lx, ly = np.meshgrid(np.arange(8), np.arange(4))
    passing = in_span = 0
    for p in _triangles(rng, 1500):
        g = _setup(p[0], p[1], p[2])
        box = _cull_box(g, p)
        lo = np.floor(p.min(0)).astype(int) - 9
        hi = np.floor(p.max(0)).astype(int) + 9
        for bx in range(lo[0] - lo[0] % 8, hi[0] + 1, 8):
            for by in range(lo[1] - lo[1] % 4, hi[1] + 1, 4):
                px = (bx + lx + 0.5).astype(f32).ravel()
                py = (by + ly + 0.5).astype(f32).ravel()
                un, vn, wn = _numerators(g, px, py)
                escapes = ~((un < g["thr"]) | (vn < g["thr"]) | (wn < g["thr"]))
                if not escapes.any():
                    continue
                rows = _edge_span(g, box, f32(bx + 0.5), f32(by + 0.5))
                covered = np.array([rows[k // 8] is not None and rows[k // 8][0] <= k % 8 <= rows[k // 8][1]
                                    for k in range(32)])
                assert not (escapes & ~covered).any(), (p, bx, by, rows)
                passing += int(escapes.sum())
                in_span += int(covered.sum())
    print(f"pixel centres escaping the fast reject {passing}, in spans {in_span}")
    assert passing > 10000 and in_span < 8 * passing  # exercised, and the spans are tight


def test_power_of_two_tile_division_is_a_multiply():
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2 ** 32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(f32)
    x = x[np.isfinite(x)]
    extra = np.array([0.0, -0.0, 1e-45, -1e-45, 1.17549435e-38, 3.4028235e38, 7.5, -7.5, 8.0, 1023.9999],
                     dtype=f32)
    x = np.concatenate([x, extra])
    for k in range(0, 11):
        div = (x / f32(2 ** k)).astype(f32)
        mul = (x * f32(2.0 ** -k)).astype(f32)
        np.testing.assert_array_equal(div.view(np.uint32), mul.view(np.uint32))


def test_power_of_two_first_tile_shift():
    v = np.arange(-70000, 70000, dtype=np.int64)
    for k in range(0, 11):
        t = 1 << k
        trunc = np.where(v >= 0, v // t, -((-v) // t))  # C's truncating division
        np.testing.assert_array_equal(np.maximum(trunc, 0), np.maximum(v >> k, 0))


def _crossings(sdf, lower, levels):
    """[S, 3, G] edge crossings of every grid entry (crossing_mask)."""
    d0 = sdf[lower[0]]
    out = np.zeros((len(levels), 3, lower.shape[1]), bool)
    for a in range(3):
        da = np.where(lower[a + 1] >= 0, sdf[np.maximum(lower[a + 1], 0)], d0)
        for s, iso in enumerate(levels):
            out[s, a] = (d0 < iso) != (da < iso)
    return out


def _lists(lower, cross, capacity):
    """The contribution list enumerated per grid vertex (vertex_grad_list_kernel)
    and built per grid entry (entry_list_kernel: counts and segment lengths,
    scan, fill at offset + earlier segments); entries are (vertex, origin)."""
    S, _, G = cross.shape
    voff = np.concatenate([[0], np.cumsum(cross.sum(1).reshape(-1))])[:-1].reshape(S, G)
    inverse = np.full((4, G), -1, np.int64)
    for r in range(4):
        for e in range(G):
            if 0 <= lower[r, e] < G:
                inverse[r, lower[r, e]] = e

    def vertices(e):  # (shell, axis, vertex) of entry e in shell-then-axis order, capacity-checked
        out = []
        for s in range(S):
            for a in range(3):
                if cross[s, a, e]:
                    v = voff[s, e] + int(cross[s, :a, e].sum())
                    if v < capacity:
                        out.append((a, v))
        return out

    per_vertex = []
    for x in range(G):
        if inverse[0, x] >= 0:
            per_vertex += [(v, 1) for _, v in vertices(inverse[0, x])]
        for a in range(3):
            if inverse[a + 1, x] >= 0:
                per_vertex += [(v, 0) for b, v in vertices(inverse[a + 1, x]) if b == a]

    counts = np.zeros(G + 1, np.int64)
    segments = np.zeros((G, 4), np.int64)
    owners = []
    for e in range(G):
        xs = lower[:, e]
        owns = [0 <= xs[r] < G and inverse[r, xs[r]] == e for r in range(4)]
        owners.append((xs, owns))
        n = [0, 0, 0, 0]
        for a, _ in vertices(e):
            n[0] += 1
            n[a + 1] += 1
        for r in range(4):
            if owns[r] and n[r]:
                counts[xs[r]] += n[r]
                segments[xs[r], r] = n[r]
    assert segments.max() < 256  # one byte per segment
    offsets = np.concatenate([[0], np.cumsum(counts)])[:-1]
    per_entry = [None] * (2 * capacity)
    for e, (xs, owns) in enumerate(owners):
        pos = [offsets[xs[r]] + segments[xs[r], :r].sum() if owns[r] else 0 for r in range(4)]
        for a, v in vertices(e):
            for r, flag in ((0, 1), (a + 1, 0)):
                if owns[r]:
                    assert 0 <= pos[r] < 2 * capacity and per_entry[pos[r]] is None
                    per_entry[pos[r]] = (v, flag)
                pos[r] += 1
    assert offsets[-1] == len(per_vertex) <= 2 * capacity
    return per_vertex, per_entry[:len(per_vertex)]


def test_contribution_list_per_entry_equals_per_vertex():
    """The captured step builds the contribution list per grid entry; it is
    the per-vertex enumeration's list entry for entry, at full and at half
    vertex capacity, and with two entries sharing a corner (an input the
    corner inverse resolves to one owner), every write inside the list."""
    from oracle import oracle
    from tests import semantics

    n = 32
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    d = np.sqrt(x * x + y * y + z * z) - 0.5
    vox = oracle.extract_voxels(semantics.pack(np.abs(d) < 2.5 * 2 / n))
    p = 2 * vox.vertices.astype(np.float64) - 1
    sdf = (np.linalg.norm(p, axis=1) - 0.5 + np.random.default_rng(0).normal(0, 0.002, len(p))).astype(f32)
    lower = vox.lower_corners.astype(np.int64)
    levels = np.array([0.04, 0.0, -0.04], f32)
    shared = lower.copy()
    shared[2, 10:20] = shared[2, 30:40]  # axis-1 corners shared by two entries
    shared[0, 50] = shared[0, 60]        # an origin shared by two entries
    for topology in (lower, shared):
        cross = _crossings(sdf, topology, levels)
        total = int(cross.sum())
        for capacity in (total, total // 2):
            per_vertex, per_entry = _lists(topology, cross, capacity)
            assert per_entry == per_vertex and len(per_vertex) > 1000


def test_hit_bit_reservations_fit_the_store_bound():
    """The compositing forward reserves, per (tile, warp) work item, a bound
    on the batches the warp walks: ceil(tile keys / 32) when a tile has at
    most two warps, else ceil(keys with the warp's mask bit / 32). The sum
    over all items never exceeds the bound the store is sized by
    (K * warps / 32 + items: triangle_rasterization._hit_bits and
    mt_composite_hit_bits_bytes), and each reservation covers the batches
    the walk forms (one per 32 keys with the warp's bit)."""
    rng = np.random.default_rng(7)
    for warps in (1, 2, 4, 8):
        for _ in range(20):
            tiles = int(rng.integers(1, 400))
            counts = rng.choice([0, 0, 0, 1, 5, 31, 32, 33, 200, 1000], size=tiles)
            k = int(counts.sum())
            items = tiles * warps
            reserved = 0
            for n in counts:
                masks = rng.integers(0, 1 << warps, size=int(n)) | (1 << int(rng.integers(0, warps)))
                for wt in range(warps):
                    own = int(((masks >> wt) & 1).sum())
                    walked = -(-own // 32)
                    r = -(-int(n) // 32) if warps <= 2 else walked
                    assert r >= walked
                    reserved += r
            assert reserved <= k * warps // 32 + items
