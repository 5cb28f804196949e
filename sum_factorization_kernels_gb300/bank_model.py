"""Shared-memory bank model of the sweep kernels and the layout search behind
their slab tables (``pack_params`` in ``csrc/sf_laplace_line.cu``,
``dg_slabs`` and ``dg_inv_layout`` in ``csrc/sf_dg.cu``, ``faces_layout`` in
``csrc/sf_cell_faces.cu``, ``ta_slabs`` in ``csrc/sf_dg_advect_tensor.cu``).

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


# ---- the DO_FACES kernel (csrc/sf_cell_faces.cu) ----
# cells per block (n^2 threads per cell, cell-major lanes)
FACES_CPB = {2: 32, 3: 14, 4: 8, 5: 5, 6: 7, 7: 5, 8: 2, 9: 3}


def faces_padded(n):
    """the padded layout (SX, SY, SZ, RS, FN, FA, CW): strides (1, n + 1,
    n (n + 1) + 1), dense face arrays"""
    sz = n * (n + 1) + 1
    return (1, n + 1, sz, n * sz, n, n * n, 4 * n * sz + 4 * n * n)


def faces_cost(n, elem, layout, conv=False):
    """wavefronts per cell of every shared access of cell_faces_kernel with
    the layout (SX, SY, SZ, RS, FN, FA, CW): the cell term's z, x and y line
    patterns on the slabs X, Sa, Sb, Sc, and per face direction the layer
    reads and row / column passes over the face arrays, the point phase, the
    injections into the output slab and the final column read.  Lanes without
    work in a pass repeat an active lane of their warp."""
    sx, sy, sz, rs, fn, fa, cw = layout
    cpb = FACES_CPB[n]
    nt = cpb * n * n
    warps = (nt + 31) // 32
    t = np.arange(32 * warps)
    act = t < nt
    tt = np.minimum(t, nt - 1)
    k, l = tt // (n * n), tt % (n * n)
    a, b = l % n, l // n
    base = k * cw
    X, Sa, Sb, Sc, Fb = 0, rs, 2 * rs, 3 * rs, 4 * rs
    acc = []

    def add(addr, mask=None, count=1):
        m = act if mask is None else (act & mask)
        acc.extend([(addr, m)] * count)

    line = {"z": lambda m: sx * a + sy * b + sz * m, "x": lambda m: sx * m + sy * a + sz * b,
            "y": lambda m: sx * a + sy * m + sz * b}
    if conv:
        ops = [(X, "z", 1), (Sa, "z", 1), (Sa, "x", 2), (Sa, "y", 2), (Sc, "y", 1), (Sa, "x", 1), (Sc, "x", 2),
               (Sa, "z", 1), (Sc, "z", 2), (Sc, "y", 2), (Sc, "x", 2), (Sc, "z", 1)]
    else:
        ops = [(X, "z", 1), (Sa, "z", 1), (Sa, "x", 2), (Sa, "y", 2), (Sc, "y", 1), (Sa, "x", 1), (Sb, "x", 1),
               (Sa, "z", 1), (Sb, "z", 2), (Sc, "z", 2), (Sa, "z", 1), (Sb, "x", 1), (Sa, "x", 2), (Sc, "y", 1),
               (Sa, "y", 2), (Sa, "x", 2), (Sa, "z", 2), (Sa, "z", 1)]
    for off, pat, cnt in ops:
        for m in range(n):
            add(base + off + line[pat](m), count=cnt)
    nl, nb = (2, 2) if conv else (4, 3)
    st = (sx, sy, sz)
    for f in range(3):
        so, s1, s2 = st[f], st[(f + 1) % 3], st[(f + 2) % 3]
        for ntask, kind in ((nl, "layers"), (nl, "cols"), (nb, "rows"), (nb, "cols")):
            for rep in range((ntask * n + n * n - 1) // (n * n)):
                task = l + rep * n * n
                busy = task < ntask * n
                kk, r = np.minimum(task, ntask * n - 1) // n, np.minimum(task, ntask * n - 1) % n
                layer = np.choose(np.minimum(kk, 3), [n - 1, 0, max(n - 2, 0), 1])
                for j in range(n):
                    if kind == "layers":
                        add(base + X + layer * so + r * s2 + j * s1, busy)
                        add(base + Fb + kk * fa + r * fn + j, busy)
                    elif kind == "cols":
                        add(base + Fb + kk * fa + j * fn + r, busy, 2)
                    else:
                        add(base + Fb + kk * fa + r * fn + j, busy, 2)
        q = b * fn + a
        add(base + Fb + q, count=2)
        add(base + Fb + fa + q, count=2)
        if not conv:
            add(base + Fb + 2 * fa + q, count=3)
            add(base + Fb + 3 * fa + q)
        y_slab = Sc if conv else Sa
        for layer in ([n - 1, 0] if conv else [n - 1, n - 2, 0, 1]):
            add(base + y_slab + layer * so + b * s2 + a * s1, count=2)
    y_slab = Sc if conv else Sa
    for m in range(n):
        add(base + y_slab + line["z"](m))
    rows = []
    for addr, m in acc:
        A, M = addr.reshape(warps, 32).copy(), m.reshape(warps, 32)
        for w in range(warps):
            if M[w].any():
                row = A[w]
                row[~M[w]] = row[M[w]][0]
                rows.append(row)
    return wavefronts(np.array(rows), elem) / cpb


def faces_layout_from_source(path=None):
    """{(elem, n): (SX, SY, SZ, RS, FN, FA, CW)} parsed from faces_layout in
    sf_cell_faces.cu"""
    src = open(path or os.path.join(CSRC, "sf_cell_faces.cu")).read()
    body = src[src.index("constexpr FacesLayout faces_layout"):]
    body = body[:body.index("\n}\n")]
    f32, f64 = re.split(r"\n\s*: \(n == 2", body, maxsplit=1)
    f64 = "n == 2" + f64
    out = {}
    for elem, part in ((4, f32), (8, f64)):
        for m in re.finditer(r"(?:n == (\d)\s*\?\s*)?FacesLayout\{([^}]*)\}", part):
            n = int(m.group(1)) if m.group(1) else 9
            out[(elem, n)] = tuple(_ints(m.group(2)))
    return out
