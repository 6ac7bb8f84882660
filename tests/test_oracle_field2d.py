"""The oracle's float64 restatement of the production 2D model and of the chunked large-N tick
(oracle/field2d_oracle.py) against the reference's own outputs (tests/golden/field2d.npz,
tick2d.npz). No GPU."""
import numpy as np
import pytest

from oracle import field2d_oracle as F


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


@pytest.fixture(scope="module")
def weights(golden):
    g = golden["field2d"]
    return {k: g["w_" + k].astype(np.float64) for k in g["names"]}


def test_oracle_unet(golden, weights):
    g = golden["field2d"]
    y = F.unet(weights, g["unet_x"].astype(np.float64))
    assert rel(y, g["unet_y"]) < 1e-6  # the golden output is stored in float32


@pytest.mark.parametrize("n", (30, 100))
def test_oracle_scatter_and_force(golden, weights, n):
    g = golden["field2d"]
    pos, vel = g[f"n{n}_pos0"].astype(np.float64), g[f"n{n}_vel0"].astype(np.float64)
    one = np.ones(n)
    x = F.scatter3(pos, vel, one, one, 128, 64.0)
    assert rel(x, g[f"n{n}_scatter"]) < 1e-6
    m = F.Model2D(weights)
    a, f = m.force(pos, vel, one, one, np.zeros((1, 128, 128)))
    assert rel(a, g[f"n{n}_acc0"]) < 1e-9
    assert rel(f[0], g[f"n{n}_field1"]) < 1e-6


def test_oracle_verlet_rollout(golden, weights):
    g = golden["field2d"]
    n = 30
    pos, vel = g[f"n{n}_pos0"].astype(np.float64), g[f"n{n}_vel0"].astype(np.float64)
    one = np.ones(n)
    m = F.Model2D(weights)
    state = (np.zeros((1, 128, 128)), None)
    for t in range(int(g["steps"])):
        pos, vel, state, _ = m.step(pos, vel, one, one, state)
        assert np.abs(pos - g[f"n{n}_pos"][t]).max() < 1e-9
        assert np.abs(vel - g[f"n{n}_vel"][t]).max() < 1e-9


def test_oracle_tick(golden, weights):
    """float32 state: the oracle's float64 arithmetic rounded where the reference stores state."""
    g = golden["tick2d"]
    n = int(g["n"])
    sim = F.Tick2D(F.Model2D(weights, pair=False), n, c=float(g["c"]), dt=float(g["dt"]), state_dtype=np.float32)
    pos, mom = g["f32_pos0"].copy(), g["f32_mom0"].copy()
    _, x = sim.scatter_pass(pos, mom, False)
    assert rel(x, g["f32_x0"]) < 2e-5  # the reference's fp32 cell weights vs float64 here
    pos, mom = sim.init_kick(pos, mom)
    assert rel(mom, g["f32_mom_ik"]) < 1e-5
    for t in range(int(g["ticks"])):
        pos, mom = sim.tick(pos, mom)
        assert rel(pos, g["f32_pos"][t]) < 1e-5 and rel(mom, g["f32_mom"][t]) < 1e-5, t


def test_oracle_tick_fp16_state(golden, weights):
    """float16 state: the oracle rounds to float16 where the reference stores (pos after the drift,
    momentum after the kick); most stored values are the reference's own."""
    g = golden["tick2d"]
    n = int(g["n"])
    sim = F.Tick2D(F.Model2D(weights, pair=False), n, c=float(g["c"]), dt=float(g["dt"]), state_dtype=np.float16)
    pos, mom = g["f16_pos0"].copy(), g["f16_mom0"].copy()
    pos, mom = sim.init_kick(pos, mom)
    assert np.mean(mom == g["f16_mom_ik"]) > 0.85
    for t in range(int(g["ticks"])):
        pos, mom = sim.tick(pos, mom)
        for a, b in ((pos, g["f16_pos"][t]), (mom, g["f16_mom"][t])):
            assert np.mean(a == b) > 0.85, t
            assert rel(a, b) < 5e-4, t


def test_oracle_prior_cell_unit_variant(golden):
    """The prior + cell-unit variant with kpad "ext" (grid 64, U-Net levels 4, width 16) against the reference."""
    g = golden["field2d_variant"]
    sd = {k: g["w_" + k].astype(np.float64) for k in g["names"]}
    m = F.Model2D(sd, grid=64, extent=64.0, levels=int(g["levels"]), prior=True, cu=True, kpad="ext")
    pos, vel = g["pos0"].astype(np.float64), g["vel0"].astype(np.float64)
    one = np.ones(len(pos))
    a, f = m.force(pos, vel, one, one, np.zeros((1, 64, 64)))
    assert rel(a, g["acc0"]) < 1e-9
    assert rel(f[0], g["field1"]) < 1e-6
    state = (np.zeros((1, 64, 64)), None)
    for t in range(int(g["steps"])):
        pos, vel, state, _ = m.step(pos, vel, one, one, state)
        assert np.abs(pos - g["pos"][t]).max() < 1e-9 and np.abs(vel - g["vel"][t]).max() < 1e-9
