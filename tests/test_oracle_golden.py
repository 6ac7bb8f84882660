"""The oracle pinned against outputs of the reference itself (tests/golden/, made by
tests/golden/make_golden.py from the reference's own functions)."""
import numpy as np
import pytest

from oracle import pm_oracle as O


@pytest.mark.parametrize("tag", ["G96_E1", "G256_E1", "G64_E1", "G128_E64"])
def test_cell_index_bit_exact_vs_reference(golden, tag):
    g = golden["cell_index"]
    pos, i0, w = g[tag + "_pos"], g[tag + "_i0"], g[tag + "_w"]
    G = int(tag.split("_")[0][1:])
    E = float(tag.split("_")[1][1:])
    oi, ow = O.cell_index(pos, G, E)
    assert np.array_equal(oi, i0.astype(np.int64))
    assert np.array_equal(ow.view(np.uint32), w.view(np.uint32))


def test_reciprocal_multiply_would_break_g96(golden):
    """The reference divides by fp32(h); multiplying by fp32(1/h) moves floor() for G=96."""
    g = golden["cell_index"]
    pos, i0 = g["G96_E1_pos"], g["G96_E1_i0"]
    p = pos.astype(np.float32)
    t = (p + np.float32(0.5)).astype(np.float32)
    u = ((t * np.float32(96.0)).astype(np.float32) - np.float32(0.5)).astype(np.float32)
    assert not np.array_equal(np.floor(u).astype(np.int64), i0)


def test_deposit_matches_reference_scatter(golden):
    g = golden["scatter_gather_2d"]
    G, E = int(g["G"]), float(g["E"])
    ref = g["grid"][0]  # mass channel, (G, G) [y][x]
    ours = O.deposit_ref(g["pos"], g["mass"], g["mask"], G, E, periodic=False)
    assert np.abs(ours - ref).max() <= 1e-6 * np.abs(ref).max()
    fixed = O.deposit_fixed(g["pos"], g["mass"], g["mask"], G, E, periodic=False)
    assert np.abs(fixed - ref).max() <= 2e-6 * np.abs(ref).max()
    # mass on the grid = mass of the corners that land on it
    assert abs(fixed.sum() * (E / G) ** 2 - ref.sum() * (E / G) ** 2) < 1e-4


def test_gather_bit_exact_vs_reference(golden):
    g = golden["scatter_gather_2d"]
    G, E = int(g["G"]), float(g["E"])
    field = g["field"]  # (4, G, G)
    F4 = np.zeros((G, G, 4), np.float32)
    F4[..., 0], F4[..., 1], F4[..., 3] = field[0], field[1], field[2]
    a, ph = O.gather_f32(F4, g["pos"], G, E, periodic=False)
    ref = g["gather"]
    assert np.array_equal(a[:, 0], ref[:, 0]) and np.array_equal(a[:, 1], ref[:, 1])
    assert np.array_equal(ph, ref[:, 2])


@pytest.mark.parametrize("key", ["plummer_n300", "plummer_n1000", "two_clump_n300", "exp_disk_n300"])
def test_isolated_pm_matches_reference_pm_acc(golden, key):
    g = golden["pm_acc_2d"]
    pos, acc = g[key + "_pos"], g[key + "_acc"]
    for s in range(min(4, len(pos))):
        n = pos.shape[1]
        ours = O.pm_acc_isolated_2d(pos[s], np.ones(n), np.ones(n), 128, 64.0, 0.5)
        assert O.rel_rms(ours, acc[s]) < 1e-5


@pytest.mark.parametrize("key", ["plummer_n300", "two_clump_n300", "exp_disk_n300"])
def test_isolated_pm_reproduces_published_medians(golden, key):
    """results/pm_baseline_force_error.json plain_pm medians (FP64 direct-sum truth, eps 0.5)."""
    g = golden["pm_acc_2d"]
    pos = g[key + "_pos"]
    es = []
    for s in range(len(pos)):
        n = pos.shape[1]
        a = O.pm_acc_isolated_2d(pos[s], np.ones(n), np.ones(n), 128, 64.0, 0.5, f32=True)
        at = O.direct_sum(pos[s].astype(np.float64), pos[s].astype(np.float64), 0.5, target_index=np.arange(n))
        es.append(O.errs(a, at)[0])
    med = O.median_lower(np.concatenate(es))
    assert abs(med - float(g[key + "_median_published"])) < 5e-6
    assert abs(med - float(g[key + "_median_here"])) < 2e-6


@pytest.mark.parametrize("d", [2, 3])
def test_direct_sum_matches_reference_exact_acc(golden, d):
    g = golden["exact_acc"]
    pos, ref, eps = g[f"d{d}_pos"], g[f"d{d}_acc"], float(g[f"d{d}_eps"])
    ours = O.direct_sum(pos, pos, eps, target_index=np.arange(len(pos)))
    assert np.abs(ours - ref).max() <= 1e-12 * np.abs(ref).max()
