"""Batched uneven scenes in one CUDA graph, tile shapes and the autotuner, on the GPU.

Every kernel is deterministic and tile shapes change launch geometry only, so the batched
graph must reproduce per-scene runs bit for bit, and any valid tile shape the same
trajectory as the defaults."""
import json

import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan, autotune, scenes
from augur_gb300.batch import BatchedPM, make_batch
from augur_gb300.cnn import GridCNN
from augur_gb300.learned import CorrectedPM, FallbackMonitor

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _run(plan, pos, vel, mass, dt, nsteps):
    p, v = _t(pos), _t(vel)
    plan.run(p, v, _t(mass), torch.ones(len(mass), device=DEV), dt=dt, nsteps=nsteps)
    return p, v


@pytest.mark.parametrize("G,kind", [(64, "plummer"), (96, "clumpy")])
def test_tile_shapes_leave_the_trajectory_bit_identical(G, kind):
    n, dt = 60000, 5e-4
    pos, vel, mass = scenes.make_scene(kind, n, seed=21)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    ref = _run(plan, pos, vel, mass, dt, 4)
    shapes = [{"deposit_rows_y": 8, "deposit_rows_z": 1, "deposit_chunk": 2048, "green_tile_y": 8,
               "c2r_rows": 4, "fft_rows": 8, "deposit_aggregate": 1},
              {"deposit_rows_y": 32, "deposit_rows_z": 2, "deposit_chunk": 65536, "green_tile_y": 16,
               "c2r_rows": 32, "fft_rows": 64, "deposit_aggregate": 0},
              {"deposit_rows_y": 4, "deposit_rows_z": 4, "deposit_chunk": 4096, "green_tile_y": 16,
               "c2r_rows": 2, "fft_rows": 1, "deposit_aggregate": 1}]
    for t in shapes:
        plan.set_tiles(t)
        assert plan.tiles == t
        p, v = _run(plan, pos, vel, mass, dt, 4)
        assert torch.equal(p, ref[0]) and torch.equal(v, ref[1]), t
    plan.check()


def test_set_tiles_rejects_shapes_that_do_not_fit():
    plan = PMPlan(3, 96, 1000, "periodic", 1.0, device=DEV)
    before = plan.tiles
    for bad in ({"deposit_rows_y": 5}, {"deposit_rows_z": 16}, {"deposit_rows_z": 5}, {"deposit_chunk": 100},
                {"green_tile_y": 12}, {"c2r_rows": 3}, {"c2r_rows": 64}, {"fft_rows": 0}, {"deposit_aggregate": 2},
                {"deposit_rows_y": 96, "deposit_rows_z": 12}):
        with pytest.raises(RuntimeError):
            plan.set_tiles(bad)
        assert plan.tiles == before


def test_plans_of_different_grids_share_kernels_safely():
    """A plan with small tiles created after a large one must not lower the shared-memory
    opt-in the large plan's launches need."""
    n, dt = 30000, 5e-4
    pos, vel, mass = scenes.make_scene("plummer", n, seed=3)
    big = PMPlan(3, 256, n, "periodic", 1.0, device=DEV)
    ref = _run(big, pos, vel, mass, dt, 2)
    small = PMPlan(3, 32, n, "periodic", 1.0, device=DEV)
    _run(small, pos, vel, mass, dt, 2)
    again = _run(big, pos, vel, mass, dt, 2)
    assert torch.equal(again[0], ref[0]) and torch.equal(again[1], ref[1])


def test_bound_force_grid_is_the_one_the_run_loop_uses():
    n, G, dt = 20000, 32, 5e-4
    pos, vel, mass = scenes.make_scene("disk", n, seed=4)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    ref = _run(plan, pos, vel, mass, dt, 3)
    big = torch.full((3, G, G, G, 4), float("nan"), device=DEV)
    plan.bind_force_grid(big[1])
    p, v = _run(plan, pos, vel, mass, dt, 3)
    assert torch.equal(p, ref[0]) and torch.equal(v, ref[1])
    assert torch.isfinite(big[1]).all() and torch.isnan(big[0]).all() and torch.isnan(big[2]).all()
    plan.bind_force_grid(None)
    assert plan.force_grid().data_ptr() != big[1].data_ptr()


def _small_batch(count=8, seed=9100):
    return make_batch(count=count, nmin=3000, nmax=60000, seed=seed, grids=(32, 48, 64))


def test_batched_graph_equals_per_scene_runs():
    batch = _small_batch()
    assert len({b["grid"] for b in batch}) >= 2
    dt, k = 5e-4, 6
    sim = BatchedPM(batch, dt=dt, streams=4, tiles=None)
    sim.begin()
    sim.steps(k - 2)
    sim.steps(2)
    out = sim.end()
    for sc, (p, v) in zip(batch, out):
        plan = PMPlan(3, sc["grid"], sc["n"], "periodic", 1.0, device=DEV)
        # begin + k merged steps + end = k + 1 force evaluations = run(nsteps=k + 1)
        pr, vr = _run(plan, sc["pos"], sc["vel"], sc["mass"], dt, k + 1)
        assert torch.equal(p, pr) and torch.equal(v, vr), (sc["kind"], sc["n"], sc["grid"])
    sim.close()


@pytest.mark.parametrize("tiles", [None, "mixed"])
def test_fused_batch_equals_per_scene_runs(tiles):
    """One launch per stage for all scenes (augur_pm_batch_run_steps) against each scene's own
    run: positions and velocities bit-identical, with scenes of different body counts, grids and
    (second case) tile shapes, including a one-body scene."""
    batch = _small_batch(count=9, seed=9400)
    pos1, vel1, mass1 = scenes.make_scene("plummer", 1, seed=5)
    batch.append({"kind": "plummer", "n": 1, "seed": 5, "grid": 32, "pos": pos1, "vel": vel1, "mass": mass1})
    tl = None
    if tiles == "mixed":
        tl = {32: {"deposit_rows_y": 8, "c2r_rows": 16, "fft_rows": 8, "deposit_chunk": 1024},
              48: {"deposit_rows_y": 16, "deposit_rows_z": 2, "c2r_rows": 8},
              64: {"deposit_rows_y": 4, "fft_rows": 32, "c2r_rows": 32, "deposit_chunk": 4096}}
    dt, k = 5e-4, 6
    sim = BatchedPM(batch, dt=dt, tiles=tl, fused=True)
    sim.begin()
    sim.steps(k - 2)
    sim.steps(2)
    out = sim.end()
    for sc, (p, v) in zip(batch, out):
        plan = PMPlan(3, sc["grid"], sc["n"], "periodic", 1.0, device=DEV)
        if tl:
            plan.set_tiles(tl[sc["grid"]])
        pr, vr = _run(plan, sc["pos"], sc["vel"], sc["mass"], dt, k + 1)
        assert torch.equal(p, pr) and torch.equal(v, vr), (sc["kind"], sc["n"], sc["grid"])
    sim.close()


def _net(seed=1, scale=0.05):
    net = GridCNN(DEV, seed=seed, phi_scale=0.1, out_scale=1.0)
    g = torch.Generator().manual_seed(seed + 1)
    net.view["w_out"].copy_(torch.randn(3, 27, 32, generator=g) * scale)
    net.prepare()
    return net


def test_batched_cnn_groups_equal_per_scene_corrected_runs():
    """Scenes of one grid share a batched force grid and one network launch per layer; the
    result equals CorrectedPM scene by scene (the batched convolution computes every sample
    as the unbatched one does)."""
    batch = _small_batch(count=7, seed=9200)
    dt, k = 5e-4, 4
    net = _net()
    nets = {48: net, 64: net}
    sim = BatchedPM(batch, dt=dt, nets=nets, streams=3, tiles=None, check_every=0)
    sim.begin()
    assert sim.groups and sum(g["B"] for g in sim.groups.values()) >= 2
    sim.steps(k)
    out = sim.end()
    for sc, (p, v) in zip(batch, out):
        plan = PMPlan(3, sc["grid"], sc["n"], "periodic", 1.0, device=DEV)
        if sc["grid"] in nets:
            # the batched runner's monitor watches energy only: no correction-size check here either
            cp = CorrectedPM(plan, net, FallbackMonitor(corr_max=1e30), check_every=0)
            pr, vr = _t(sc["pos"]), _t(sc["vel"])
            cp.begin(pr, vr, _t(sc["mass"]), torch.ones(sc["n"], device=DEV), dt=dt)
            cp.steps(k)
            cp.end(pr, vr)
        else:
            pr, vr = _run(plan, sc["pos"], sc["vel"], sc["mass"], dt, k + 1)
        assert torch.equal(p, pr) and torch.equal(v, vr), (sc["kind"], sc["n"], sc["grid"])
    sim.close()


def test_batched_fallback_reverts_scenes_and_recaptures():
    """A drift bound no run can meet trips every CNN scene at the first check; they leave the
    group, the graph is captured again, and each scene then follows the same trajectory as
    CorrectedPM reverting at the same step."""
    batch = _small_batch(count=5, seed=9300)
    dt = 5e-4
    net = _net(seed=5, scale=0.2)
    nets = {48: net, 64: net}
    sim = BatchedPM(batch, dt=dt, nets=nets, streams=2, tiles=None, check_every=2, drift_max=1e-12)
    sim.begin()
    cnn0 = [s["cnn"] for s in sim.scenes]
    assert any(cnn0)
    sim.steps(6)
    out = sim.end()
    assert not any(s["cnn"] for s in sim.scenes)
    assert not sim.groups
    for sc, s, c0, (p, v) in zip(batch, sim.scenes, cnn0, out):
        assert torch.isfinite(p).all() and torch.isfinite(v).all()
        if c0:
            assert s["monitor"].reverted and "energy drift" in s["monitor"].reason
            plan = PMPlan(3, sc["grid"], sc["n"], "periodic", 1.0, device=DEV)
            cp = CorrectedPM(plan, net, FallbackMonitor(drift_max=1e-12, corr_max=1e30), check_every=2)
            pr, vr = _t(sc["pos"]), _t(sc["vel"])
            cp.begin(pr, vr, _t(sc["mass"]), torch.ones(sc["n"], device=DEV), dt=dt)
            cp.steps(6)
            cp.end(pr, vr)
            assert cp.monitor.reverted
            assert torch.equal(p, pr) and torch.equal(v, vr), (sc["kind"], sc["n"], sc["grid"])
    sim.close()


def test_autotuner_picks_valid_tiles_and_caches_them(tmp_path):
    n, G = 40000, 64
    pos, vel, mass = scenes.make_scene("plummer", n, seed=11)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    r = autotune.tune_plan(plan, _t(pos), _t(vel), _t(mass), steps=2, reps=1, rounds=1)
    assert plan.tiles == r["tiles"] and r["ms"] <= r["default_ms"] and r["evaluated"] > 5
    path = tmp_path / "tiles.json"
    cache = autotune.tune([(32, 5000)], path=path, log=None)
    assert "G32_n4096" in cache["entries"]
    assert autotune.tiles_for(32, 6000, json.loads(path.read_text())) == cache["entries"]["G32_n4096"]["tiles"]
