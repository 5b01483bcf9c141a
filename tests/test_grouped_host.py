"""Grouped-product host logic without a GPU: shape defaults, save/load round trips of class tables
(v1) and of tables with measured costs (v2), and rejection of malformed tables."""
import os

import blaze_gb300 as G


def lib():
    if not os.path.exists(G.LIB_PATH):
        G.build()
    return G.lib()


def test_default_shapes_follow_problem_size():
    lib()
    small = G.grouped_shape_for(8, 5, 6, 10)
    large = G.grouped_shape_for(8, 250, 250, 250)
    assert small[1] * small[2] < large[1] * large[2]
    # FP64 keeps at most 16 accumulators per lane (16x32 or 32x16 warp tiles)
    assert large[1] * large[2] <= 512


def test_tuning_save_load_roundtrip(tmp_path):
    L = lib()
    # a class table without costs (an earlier autotune in this process would save as v2)
    reset = tmp_path / "reset.txt"
    reset.write_text("gb300-grouped-tune v1\n")
    assert L.gb300_grouped_tuning_load(str(reset).encode()) == 0
    p = tmp_path / "t.txt"
    assert L.gb300_grouped_tuning_save(str(p).encode()) == 0
    text = p.read_text().splitlines()
    assert text[0] == "gb300-grouped-tune v1" and len(text) == 1 + 2 * 6 * 6 * 3
    # a loaded table (no costs) makes plans use its class shapes
    assert L.gb300_grouped_tuning_load(str(p).encode()) == 0
    before = G.grouped_shape_for(8, 100, 20, 300)
    # rewrite one class and load it back
    lines = [ln for ln in text[1:]]
    d, a, b, c, s = (int(x) for x in lines[0].split())
    lines[0] = f"{d} {a} {b} {c} {0 if s else 1}"
    p.write_text("\n".join([text[0]] + lines) + "\n")
    assert L.gb300_grouped_tuning_load(str(p).encode()) == 0
    assert G.grouped_shape_for(8, 5, 5, 5)[0] == (0 if s else 1)
    # restore the original table
    p.write_text("\n".join(text) + "\n")
    assert L.gb300_grouped_tuning_load(str(p).encode()) == 0
    assert G.grouped_shape_for(8, 100, 20, 300) == before


def test_malformed_tuning_files_are_rejected(tmp_path):
    L = lib()
    p = tmp_path / "bad.txt"
    p.write_text("not a table\n")
    assert L.gb300_grouped_tuning_load(str(p).encode()) == G.ERR_INVALID_ARG
    p.write_text("gb300-grouped-tune v1\n0 0 0 0 9\n")
    assert L.gb300_grouped_tuning_load(str(p).encode()) == G.ERR_INVALID_ARG


def test_costed_table_picks_per_product(tmp_path):
    """A v2 table carries the autotuner's time per padded multiply-add of every shape: a plan then
    takes, for each product's own m and n, the shape with the least padded work times that cost."""
    L = lib()
    p = tmp_path / "v2.txt"
    rows = ["gb300-grouped-tune v2"]
    for d in range(2):
        for a in range(6):
            for b in range(6):
                for c in range(3):
                    # shape 0 (8 x 8) four times dearer than the others per padded multiply-add
                    rows.append(f"{d} {a} {b} {c} 1 4 1 1 1 1 1")
    p.write_text("\n".join(rows) + "\n")
    assert L.gb300_grouped_tuning_load(str(p).encode()) == 0
    # 16 x 16 (shape 1) wastes nothing on a 16 x 16 product and costs a quarter of 8 x 8
    assert G.grouped_shape_for(8, 16, 16, 16)[0] == 1
    # 9 x 9: 8 x 8 tiles pad to 16 x 16 too, at four times the cost: never chosen
    assert G.grouped_shape_for(8, 9, 9, 9)[0] != 0
    q = tmp_path / "v2b.txt"
    assert L.gb300_grouped_tuning_save(str(q).encode()) == 0
    assert q.read_text().splitlines()[0] == "gb300-grouped-tune v2"
    # a cost line with a missing value is rejected and leaves the table as it was
    bad = tmp_path / "bad2.txt"
    bad.write_text("gb300-grouped-tune v2\n0 0 0 0 1 1 1\n")
    assert L.gb300_grouped_tuning_load(str(bad).encode()) == G.ERR_INVALID_ARG
    assert G.grouped_shape_for(8, 16, 16, 16)[0] == 1
    # back to a class table for the other tests of this process
    p1 = tmp_path / "v1.txt"
    p1.write_text("gb300-grouped-tune v1\n")
    assert L.gb300_grouped_tuning_load(str(p1).encode()) == 0
