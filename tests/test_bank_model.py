"""The shared-memory bank model behind the line kernel's slab tables: it
reproduces the ncu wavefront count of the p=4 FP32 kernel, and the committed
tables (parsed from the CUDA source) cost no more than the single padded
layout each degree started from."""
import numpy as np

from sum_factorization_kernels_gb300 import bank_model as B

# the line kernel's layouts before the search: (W, K) and one padded layout
# (1, P1, P2) shared by B0 and B1 (per-cell stride 2 n P2 + skew) and B2
# (1, Q1, Q2), cell-major lanes, no line swaps
PADDED_F32 = {
    2: (1, 8, (1, 2, 5, 20), (1, 2, 6, 12)),
    3: (2, 7, (1, 3, 9, 59), (1, 3, 11, 41)),
    4: (1, 2, (1, 4, 19, 176), (1, 4, 20, 80)),
    5: (4, 5, (1, 5, 25, 253), (1, 5, 37, 185)),
    6: (7, 6, (1, 7, 42, 508), (1, 6, 38, 228)),
    7: (5, 3, (1, 7, 56, 785), (1, 7, 52, 369)),
    8: (2, 1, (1, 9, 72, 1152), (1, 8, 72, 576)),
    9: (8, 3, (1, 9, 81, 1465), (1, 9, 85, 785)),
}


def test_wavefront_rules():
    lanes = np.arange(32)[None, :]
    assert B.wavefronts(lanes, 4) == 1                 # 32 consecutive words
    assert B.wavefronts(lanes * 2, 4) == 2             # stride 2: two words per bank
    assert B.wavefronts(np.zeros((1, 32), int), 4) == 1  # one word: broadcast
    assert B.wavefronts(lanes * 32, 4) == 32           # one bank
    assert B.wavefronts(lanes, 8) == 2                 # 8-byte words: two half-warps


def test_source_tables_parse_and_fit():
    t = B.pack_params_from_source()
    assert sorted(t) == [(e, n) for e in (4, 8) for n in range(2, 10)]
    for (elem, n), pp in t.items():
        for sx, sy, sz, rs in pp[7:]:
            g = np.arange(n)
            v = (sx * g[:, None, None] + sy * g[None, :, None] + sz * g[None, None, :]).ravel()
            assert len(np.unique(v)) == v.size and v.max() < rs, (elem, n)


def test_model_reproduces_ncu_p4():
    """ncu on the 64^3 p=4 FP32 apply (one colour launch, 32,768 cells):
    5,089,427 shared wavefronts = 155.3 per cell.  Model: slabs + the six
    walk-ordered geometry reads + the geometry block written by the bulk copy
    (15,000 bytes per step in 128-byte wavefronts), per cell of the 5-cell
    step."""
    pp = B.pack_params_from_source()[(4, 5)]
    slabs = B.line_cost(5, 4, pp)
    geo = B.line_geometry_cost(5, 4, 4, 5)
    tma = 15000 / 128
    per_cell = (slabs + geo + tma) / 5
    assert slabs == 540 and geo == B.ideal(5, 4, 4, 6)
    assert abs(per_cell - 5089427 / 32768) < 0.02 * per_cell


def test_tables_no_worse_than_padded_layout():
    t = B.pack_params_from_source()
    for n, (w, k, b01, b2) in PADDED_F32.items():
        lanes = B.lane_map(n, w, k, False)
        old = (B.slab_cost(n, 4, lanes, b01, (6, 9, 4)) + B.slab_cost(n, 4, lanes, b2, (2, 0, 2)))
        new = B.line_cost(n, 4, t[(4, n)])
        assert new <= old, (n, new, old)
    # p=4: 540 weighted wavefronts per step against 660 and the ideal 460
    lanes = B.lane_map(5, 4, 5, False)
    old5 = B.slab_cost(5, 4, lanes, (1, 5, 25, 253), (6, 9, 4)) + B.slab_cost(5, 4, lanes, (1, 5, 37, 185), (2, 0, 2))
    assert (B.line_cost(5, 4, t[(4, 5)]), old5, B.ideal(5, 4, 4, 23)) == (540, 660, 460)


def test_faces_layouts():
    """the DO_FACES kernel's layout table (parsed from the CUDA source): every
    entry fits, costs no more than the padded layout in both variants and
    holds the per-cell words within 8 of it; the padded layout's model count
    at p=4 FP32 is within 4 % of ncu's 532 wavefronts per cell, and the
    searched one gives the 382 quoted in the source"""
    t = B.faces_layout_from_source()
    assert sorted(t) == [(e, n) for e in (4, 8) for n in range(2, 10)]
    for (elem, n), L in t.items():
        sx, sy, sz, rs, fn, fa, cw = L
        g = np.arange(n)
        v = (sx * g[:, None, None] + sy * g[None, :, None] + sz * g[None, None, :]).ravel()
        assert len(np.unique(v)) == v.size and v.max() < rs
        assert fn >= n and fa >= n * fn and cw >= 4 * rs + 4 * fa
        pad = B.faces_padded(n)
        assert cw <= pad[6] + 8, (elem, n)
        for conv in (False, True):
            assert B.faces_cost(n, elem, L, conv) <= B.faces_cost(n, elem, pad, conv), (elem, n, conv)
    assert abs(B.faces_cost(5, 4, B.faces_padded(5)) - 532) < 0.04 * 532
    assert round(B.faces_cost(5, 4, t[(4, 5)])) == 382


def test_line_operator_kernel_layouts():
    """The FP32 slab table of the line-operator kernel (ta_slabs in
    csrc/sf_dg_advect_tensor.cu), parsed from the source: per degree its
    weighted wavefronts (X: z stores, x and y loads; R1: x stores, z loads;
    R2: y stores, z loads; cell-major lanes) beat the padded layout of
    dg_layout it replaced, and p = 4 costs the 190 the search found"""
    import os
    import re
    src = open(os.path.join(B.CSRC, "sf_dg_advect_tensor.cu")).read()
    body = src[src.index("constexpr TASlabs ta_slabs(int n, int elem, int cpb)"):]
    body = body[:body.index("default: break;")]
    rows = re.findall(r"case (\d): return ta_slabs3\(\{([^}]*)\}, \{([^}]*)\}, \{([^}]*)\}, cpb\);", body)
    assert len(rows) == 8
    padded = {2: (2, 5, 6), 3: (3, 9, 10), 4: (4, 19, 12), 5: (5, 25, 2), 6: (7, 42, 8), 7: (7, 56, 25),
              8: (9, 72, 0), 9: (9, 81, 6)}
    cells = {2: 32, 3: 14, 4: 8, 5: 5, 6: 7, 7: 5, 8: 2, 9: 3}
    weights = ((1, 1, 1), (1, 1, 0), (1, 0, 1))
    for case, *slabs in rows:
        n = int(case)
        k = cells[n]
        lanes = B.lane_map(n, (k * n * n + 31) // 32, k, False)
        table = sum(B.slab_cost(n, 4, lanes, tuple(B._ints(sl)[:4]), w) for sl, w in zip(slabs, weights))
        p1, p2, skew = padded[n]
        old = sum(B.slab_cost(n, 4, lanes, (1, p1, p2, 3 * p2 * n + skew), w) for w in weights)
        assert table < old, (n, table, old)
        if n == 5:
            assert table == 190
