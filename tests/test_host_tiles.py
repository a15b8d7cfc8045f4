"""The FAST tensor-core tiling rule, on a hand-built view-factor list
(workloads.tc_tile_structure, the numpy statement of build_tc and
k_tc_rowneed that the GPU tests compare the device's tiles with): 128 x 64
tiles keyed row block * column blocks + column block, 16-wide K slices, and
residual tiles V - bf16(V) where a tile holds a view factor >= 1e-4 or where,
for some facet row, the tile's share of the row's mass is at least 1 % of the
row's mean mass per column block it touches.  Cells with fewer entries than
the threshold form no tile: their entries are the sparse remainder (tile -1),
summed in FP32 outside the tensor cores."""
import numpy as np

from binarytpm_gb300 import workloads

NF = 200  # row blocks 0 (facets 0-127) and 1 (128-199); column blocks 0-3


def _csr(rows):
    ptr, idx, vf = [0], [], []
    for f in range(NF):
        for j, v in rows.get(f, []):
            idx.append(j)
            vf.append(v)
        ptr.append(len(idx))
    return np.array(ptr, np.int32), np.array(idx, np.int32), np.array(vf, np.float32)


ROWS = {
    0: [(5, 0.5), (70, 1e-6), (130, 2e-7)],  # block 0 large; blocks 1 and 2 below 1 % of its mean
    1: [(66, 5e-5), (67, 5e-5)],             # all of row 1's mass in block 1, each value < 1e-4
    150: [(10, 3e-5), (190, 0.9)],           # block 0 is 0.003 % of row 150's mass
}


def test_tiles_slices_and_residual_rule():
    ptr, idx, vf = _csr(ROWS)
    tiles, inv, slices, has_lo = workloads.tc_tile_structure(NF, ptr, idx, vf, min_entries=1)
    assert tiles.tolist() == [0, 1, 2, 4, 6]
    rows = np.repeat(np.arange(NF), np.diff(ptr))
    assert np.array_equal(tiles[inv], (rows // 128) * 4 + idx // 64)
    assert np.array_equal(slices, idx % 64 // 16)
    # tile 0: value 0.5; tile 1: row 1 needs it although every value < 1e-4;
    # tile 2: 2e-7 is a negligible share of row 0; tile 4: row 150's 3e-5 is
    # negligible beside its 0.9; tile 6: value 0.9
    assert has_lo.tolist() == [True, True, False, False, True]


def test_a_row_with_only_small_entries_keeps_its_residual():
    rows = dict(ROWS)
    rows[151] = [(20, 2e-5)]  # all of row 151's mass sits in tile 4
    ptr, idx, vf = _csr(rows)
    tiles, _, _, has_lo = workloads.tc_tile_structure(NF, ptr, idx, vf, min_entries=1)
    assert tiles.tolist() == [0, 1, 2, 4, 6]
    assert has_lo.tolist() == [True, True, False, True, True]


def test_empty_list_has_no_tiles():
    ptr, idx, vf = _csr({})
    tiles, inv, slices, has_lo = workloads.tc_tile_structure(NF, ptr, idx, vf, min_entries=1)
    assert tiles.size == inv.size == slices.size == has_lo.size == 0


def test_sparse_cells_go_to_the_remainder():
    """With a threshold of 2 entries per cell only cell (row block 0,
    column block 1) qualifies: it holds row 0's entry 70 and row 1's entries
    66 and 67.  Every other cell holds one entry, so those entries are the
    remainder."""
    ptr, idx, vf = _csr(ROWS)
    tiles, inv, _, has_lo = workloads.tc_tile_structure(NF, ptr, idx, vf, min_entries=2)
    assert tiles.tolist() == [1]
    rows = np.repeat(np.arange(NF), np.diff(ptr))
    assert inv.tolist() == [-1, 0, -1, 0, 0, -1, -1]
    assert np.array_equal(np.flatnonzero(inv < 0), np.flatnonzero(~((rows == 1) | (rows == 0) & (idx == 70))))
    assert has_lo.tolist() == [True]


def test_default_threshold_matches_the_library():
    import re
    from pathlib import Path

    src = (Path(__file__).resolve().parents[1] / "binarytpm_gb300" / "csrc" / "atpm_capi.cpp").read_text()
    m = re.search(r"int tc_min_entries\(\) \{.*?\? v : (\d+);", src, re.S)
    assert m and int(m.group(1)) == workloads.TC_MIN_ENTRIES
