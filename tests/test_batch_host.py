"""Host logic of the batched runner and the autotuner cache (no GPU)."""
import numpy as np

from augur_gb300 import autotune
from augur_gb300.batch import grid_for, make_batch


def test_grid_rule_gives_about_eight_cells_per_body():
    assert grid_for(10_000) == 64
    assert grid_for(32_768) == 64
    assert grid_for(32_769) == 96
    assert grid_for(110_592) == 96
    assert grid_for(110_593) == 128
    assert grid_for(1_000_000) == 128


def test_batch_is_seeded_and_log_uniform():
    a = make_batch(count=6, nmin=1000, nmax=20000, seed=7, grids=(32, 48, 64))
    b = make_batch(count=6, nmin=1000, nmax=20000, seed=7, grids=(32, 48, 64))
    assert [x["n"] for x in a] == [x["n"] for x in b]
    assert all(np.array_equal(x["pos"], y["pos"]) for x, y in zip(a, b))
    assert all(1000 <= x["n"] <= 20000 for x in a)
    assert [x["kind"] for x in a[:5]] == ["plummer", "uniform", "clumpy", "disk", "flyby"]
    for x in a:
        assert x["pos"].shape == (x["n"], 3) and x["pos"].dtype == np.float32
        assert (x["pos"] >= -0.5).all() and (x["pos"] < 0.5).all()


def test_cache_lookup_takes_the_nearest_bucket_of_the_same_grid():
    cache = {"entries": {"G64_n16384": {"tiles": {"c2r_rows": 4}}, "G64_n32768": {"tiles": {"c2r_rows": 8}},
                         "G128_n1048576": {"tiles": {"c2r_rows": 16}}}}
    assert autotune.tiles_for(64, 20000, cache) == {"c2r_rows": 4}
    assert autotune.tiles_for(64, 30000, cache) == {"c2r_rows": 8}
    assert autotune.tiles_for(64, 10 ** 6, cache) == {"c2r_rows": 8}
    assert autotune.tiles_for(96, 10 ** 5, cache) is None
    assert autotune.key(128, 900_000) == "G128_n1048576"


def test_candidates_divide_the_grid():
    for G in (64, 96, 128, 256):
        c = autotune.candidates(G)
        assert all(G % d["deposit_rows_y"] == 0 and G % d["deposit_rows_z"] == 0 for d in c["deposit"])
        assert all(G % d["green_tile_y"] == 0 for d in c["green_tile_y"])
        assert all(1 <= d["fft_rows"] <= 256 for d in c["fft_rows"])


def test_batch_shapes_cover_the_workload():
    shapes = autotune.batch_shapes()
    ns = [n for _, n in shapes]
    assert min(ns) <= 10_000 and max(ns) >= 1_000_000
    assert {g for g, _ in shapes} == {64, 96, 128}
