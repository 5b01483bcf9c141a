"""Grouped-product host logic without a GPU: tuning-table defaults, save/load round trip and
rejection of malformed tables."""
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
    p = tmp_path / "t.txt"
    assert L.gb300_grouped_tuning_save(str(p).encode()) == 0
    text = p.read_text().splitlines()
    assert text[0] == "gb300-grouped-tune v1" and len(text) == 1 + 2 * 6 * 6 * 3
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
