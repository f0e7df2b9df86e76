"""CPU tests of the autotuner's committed table and its nearest-shape lookup."""
import json

from blaze103 import autotune


def test_committed_table_is_well_formed():
    table = json.load(open(autotune.TUNING_PATH))
    assert set(table["shapes"]) == set(autotune.SHAPES)
    for name, entry in table["shapes"].items():
        t = entry["tuning"]
        assert set(t) <= {"stage_bytes", "max_warps_per_block", "tile_residues", "launch_mode", "batch_launch"}
        assert 0 < t["stage_bytes"] <= 16384 and 0 <= t["max_warps_per_block"] <= 32 and t["tile_residues"] >= 0
        assert entry["kind"] == autotune.SHAPES[name][0]
        assert entry["ms"] <= entry["default_ms"] * 1.05  # the chosen setting is no slower than the default


def test_lookup_takes_the_nearest_shape_of_its_kind():
    shapes = autotune.load_table()["shapes"]
    for name, entry in shapes.items():
        got = autotune.lookup(entry["kind"], entry["n_queries"], entry["median_qlen"], entry["db_residues"])
        assert got == entry["tuning"], name
    # a 500-query batch near the 512-query shape, a 60-query one near the 64-query shape
    b512, b64 = shapes["batched-512"], shapes["batched-64"]
    assert autotune.lookup("batched", 500, b512["median_qlen"], b512["db_residues"]) == b512["tuning"]
    assert autotune.lookup("batched", 60, b64["median_qlen"], b64["db_residues"]) == b64["tuning"]
    assert autotune.lookup("no-such-kind", 1, 1.0, 1) is None
