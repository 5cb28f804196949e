"""Shared-memory bank model of the sweep kernels and the layout search behind
their slab tables (``pack_params`` in ``csrc/sf_laplace_line.cu``,
``dg_slabs`` and ``dg_inv_layout`` in ``csrc/sf_dg.cu``).

Model: shared memory has 32 banks of 4 bytes.  One warp-wide access takes as
many wavefronts as the largest number of distinct 4-byte words that its
active lanes touch in one bank (lanes reading the same word share it).  For
8-byte accesses each half-warp is served separately and a word occupies the
bank pair (2w, 2w+1) mod 32.

A kernel's slab traffic is a list of accesses: a slab (strides SX, SY, SZ,
per-cell stride RS), a pattern and a count per step.  Pattern ``z``: the lane
with line (a, b) reads the z column (a, b), entry m at SX a + SY b + SZ m;
``x``: the x line (y, z) = (a, b) (or (b, a) when the kernel swaps x lines),
entry m at SX m + SY y + SZ z; ``y``: the y line (x, z) likewise.  Lane t of
a group of W warps works on cell k and line l = a + n b with (k, l) =
(t / n^2, t % n^2) for the cell-major map or (t % K, t / K) for the
interleaved one; lanes past K n^2 repeat the last used lane.

``search`` is the exhaustive search the tables came from: stride triples
that are permutations of (1, P1, P2) with padded P1, P2 and every per-cell
stride up to 32 words above the slab's extent.
"""
from __future__ import annotations

import itertools
import os
import re

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")


def lane_map(n: int, warps: int, cells: int, interleaved: bool):
    """(cell, a, b) of every lane, each an array of shape (warps, 32)"""
    kn2 = cells * n * n
    t = np.arange(32 * warps)
    tt = np.where(t < kn2, t, kn2 - 1)
    if interleaved:
        k, l = tt % cells, tt // cells
    else:
        k, l = tt // (n * n), tt % (n * n)
    return k.reshape(warps, 32), (l % n).reshape(warps, 32), (l // n).reshape(warps, 32)


def wavefronts(addr: np.ndarray, elem: int) -> int:
    """total wavefronts of the warp accesses in the rows of addr (R, 32), in words"""
    groups = [addr] if elem == 4 else [addr[:, :16], addr[:, 16:]]
    nb = 32 if elem == 4 else 16
    total = 0
    for g in groups:
        s = np.sort(g, axis=1)
        first = np.ones_like(s, dtype=bool)
        first[:, 1:] = s[:, 1:] != s[:, :-1]
        cnt = np.zeros((s.shape[0], nb), dtype=np.int64)
        rows = np.broadcast_to(np.arange(s.shape[0])[:, None], s.shape)
        np.add.at(cnt, (rows[first], (s % nb)[first]), 1)
        total += int(cnt.max(axis=1).sum())
    return total


def pattern_addr(n, lanes, slab, pattern, xswap=False, yswap=False):
    """word addresses (R, 32) of one pattern over m = 0..n-1 and every warp"""
    sx, sy, sz, rs = slab
    k, a, b = (v[:, None, :] for v in lanes)
    m = np.arange(n)[None, :, None]
    if pattern == "z":
        v = sx * a + sy * b + sz * m
    elif pattern == "x":
        y, z = (b, a) if xswap else (a, b)
        v = sx * m + sy * y + sz * z
    else:
        x, z = (b, a) if yswap else (a, b)
        v = sx * x + sy * m + sz * z
    return (k * rs + v).reshape(-1, 32)


def slab_cost(n, elem, lanes, slab, weights, xswap=False, yswap=False):
    """weighted wavefronts of one slab: weights = accesses per step in (z, x, y)"""
    return sum(w * wavefronts(pattern_addr(n, lanes, slab, p, xswap, yswap), elem)
               for p, w in zip("zxy", weights) if w)


def ideal(n, elem, warps, accesses):
    return accesses * warps * n * (1 if elem == 4 else 2)


# accesses per step of the line kernel's slabs B0, B1, B2 in (z, x, y)
LINE_WEIGHTS = ((3, 4, 1), (3, 5, 3), (2, 0, 2))
# dg_kernel's slabs B0, B1, B2
DG_WEIGHTS = ((2, 3, 1), (3, 3, 3), (1, 0, 1))
# the inverse mass kernel's regions ZX and XY
INV_WEIGHTS = ((2, 2, 0), (0, 2, 2))


def line_cost(n, elem, pp):
    """slab wavefronts per step of one group of the line kernel for a
    pack_params entry (W, K, GROUPS, MINB, INTER, XS, YS, B0, B1, B2)"""
    w, k, _, _, inter, xs, ys, *slabs = pp
    lanes = lane_map(n, w, k, bool(inter))
    return sum(slab_cost(n, elem, lanes, s, wt, xs, ys) for s, wt in zip(slabs, LINE_WEIGHTS))


def line_geometry_cost(n, elem, w, k, walk_ordered=True, gs=None):
    """wavefronts per step of the 6 geometry reads of the quadrature-point
    operation: walk-ordered blocks (lane t reads word c K n^2 + t) or
    per-cell blocks gs words apart (point (l, c) at c n^2 + l)"""
    lanes = lane_map(n, w, k, False)
    kk, a, b = (v[:, None, :] for v in lanes)
    c = np.arange(n)[None, :, None]
    if walk_ordered:
        t = np.minimum(np.arange(32 * w), k * n * n - 1).reshape(w, 1, 32)
        addr = c * k * n * n + t
    else:
        addr = kk * gs + c * n * n + a + n * b
    return 6 * wavefronts(addr.reshape(-1, 32), elem)


def search(n, elem, lanes, weights, xswap=False, yswap=False, rs_slack=33):
    """best (cost, slab) over padded stride permutations and per-cell strides"""
    best = None
    for p1 in range(n, n + 13):
        for p2 in range((n - 1) * p1 + n, (n - 1) * p1 + 4 * n):
            for s in set(itertools.permutations((1, p1, p2))):
                g = np.arange(n)
                v = (s[0] * g[:, None, None] + s[1] * g[None, :, None] + s[2] * g[None, None, :]).ravel()
                if len(np.unique(v)) != v.size:
                    continue
                ext = int(v.max()) + 1
                for rs in range(ext, ext + rs_slack):
                    c = slab_cost(n, elem, lanes, s + (rs,), weights, xswap, yswap)
                    if best is None or (c, rs) < (best[0], best[1][3]):
                        best = (c, s + (rs,))
    return best


def _ints(txt):
    return [int(v) for v in re.findall(r"-?\d+", txt)]


def pack_params_from_source(path=None):
    """{(elem, n): (W, K, GROUPS, MINB, INTER, XS, YS, B0, B1, B2)} parsed
    from pack_params in sf_laplace_line.cu"""
    src = open(path or os.path.join(CSRC, "sf_laplace_line.cu")).read()
    body = src[src.index("constexpr PackParams pack_params"):]
    body = body[:body.index("\n}\n")]
    f32, f64 = re.split(r"\n\s*: \(n == 2", body, maxsplit=1)
    f64 = "n == 2" + f64
    out = {}
    for elem, part in ((4, f32), (8, f64)):
        for m in re.finditer(r"(?:n == (\d)\s*\?\s*)?PackParams\{([^}]*\{[^}]*\}[^}]*\{[^}]*\}[^}]*\{[^}]*\})\}", part):
            vals = _ints(m.group(2))
            n = int(m.group(1)) if m.group(1) else 9
            out[(elem, n)] = tuple(vals[:7]) + (tuple(vals[7:11]), tuple(vals[11:15]), tuple(vals[15:19]))
    return out
