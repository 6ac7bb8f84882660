"""The learned correction on the GPU: a short training run beats plain PM on held-out
snapshots (force error vs the FP64 Ewald direct sum), the corrected leapfrog and its
fallback, and the split run loop."""
import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan, energy_fp64, scenes
from augur_gb300.cnn import GridCNN
from augur_gb300.learned import (CorrectedPM, FallbackMonitor, evaluate, label_snapshots, make_dataset, make_truth,
                                 train)

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def test_training_reduces_force_error_on_held_out_snapshots():
    G, n = 32, 40000
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    net = GridCNN(DEV, seed=4738, phi_scale=0.1)
    data = make_dataset(plan, net, n, 100, 4738, n_targets=2048, eps=1.0 / 64)
    held = make_dataset(plan, net, n, 10, 9100, n_targets=2048, eps=1.0 / 64)
    net.out_scale = float(torch.cat([d["label"] for d in data]).pow(2).sum(1).mean().sqrt())
    before = evaluate(net, plan, held)
    assert before["cnn"]["rel_rms"] == pytest.approx(before["plain_pm"]["rel_rms"])  # zero-initialised output
    hist = train(net, plan, data, steps=1000, batch=4, lr=1e-3, log_every=100)
    after = evaluate(net, plan, held)
    assert hist[-1]["loss"] < min(hist[0]["loss"], 1.0)
    # what the trained network gains over plain PM, scene by scene and overall; the uniform
    # box's forces are shot noise the grid cannot predict, so it only must not get worse by 5%
    for kind, r in after["by_kind"].items():
        bound = 1.05 if kind == "uniform" else 1.0
        assert r["cnn"]["rel_rms"] < bound * r["plain_pm"]["rel_rms"], (kind, r)
    assert after["cnn"]["rel_rms"] < 0.85 * after["plain_pm"]["rel_rms"], after


def test_training_resumes_from_a_sigterm_checkpoint(tmp_path):
    """Six AdamW steps in one run against three steps stopped by SIGTERM (saved atomically) plus a
    fresh run that resumes from the checkpoint: the same parameters, AdamW state and step count (up
    to the fp32 atomics of the gather transpose)."""
    import os
    import signal

    G, n = 32, 20000
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    net0 = GridCNN(DEV, seed=4738, phi_scale=0.1)
    truth = make_truth(n, 8, 4738, DEV, n_targets=1024, eps=1.0 / 64)
    data = label_snapshots(plan, net0, truth)
    scale = float(torch.cat([d["label"] for d in data]).pow(2).sum(1).mean().sqrt())

    def fresh():
        net = GridCNN(DEV, seed=4738, phi_scale=0.1, out_scale=scale)
        net.view["w_out"].normal_(0.0, 1e-3)  # non-zero output layer: every parameter moves
        net.prepare()
        return net

    a = fresh()
    train(a, plan, data, steps=6, batch=2, lr=1e-3, log_every=3)
    a2 = fresh()
    train(a2, plan, data, steps=6, batch=2, lr=1e-3, log_every=3)
    floor = float((a2.params - a.params).norm() / a.params.norm())  # run-to-run spread
    ck = str(tmp_path / "g32.ckpt")
    b = fresh()
    kill = lambda m: os.kill(os.getpid(), signal.SIGTERM) if m.startswith("step 3 ") else None  # noqa: E731
    hist = train(b, plan, data, steps=6, batch=2, lr=1e-3, log_every=3, log=kill, checkpoint=ck)
    assert hist[-1].get("stopped") and hist[-1]["step"] == 3 and b.adam_step == 3
    c = fresh()
    hist = train(c, plan, data, steps=6, batch=2, lr=1e-3, log_every=3, checkpoint=ck)
    assert c.adam_step == 6 and [h["step"] for h in hist if "loss" in h] == [3, 6]
    rel = float((c.params - a.params).norm() / a.params.norm())
    print(f"resumed vs straight {rel:.3e}, straight vs straight {floor:.3e}")
    assert rel < 1e-5 + 3.0 * floor, (rel, floor)


def test_split_run_loop_equals_run():
    n, G, dt = 20000, 32, 5e-4
    pos, vel, mass = scenes.make_scene("clumpy", n, seed=5)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    ones = torch.ones(n, device=DEV)
    p1, v1 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    m = torch.from_numpy(mass).to(DEV)
    plan.run(p1, v1, m, ones, dt=dt, nsteps=4)
    p2, v2 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    plan.run_load(p2, v2, m, ones, dt=dt)
    plan.run_grid()
    plan.run_kick(0.5 * dt, True)
    for _ in range(3):
        plan.run_grid()
        plan.run_kick(dt, True)
    plan.run_grid()
    plan.run_kick(0.5 * dt, False)
    plan.run_unload(p2, v2)
    assert torch.equal(p1, p2) and torch.equal(v1, v2)


def test_split_loop_with_density_output_equals_run():
    """run_grid(rho_out) (deposit writing the density grid beside the x R2C) leaves the
    trajectory unchanged and writes the density of the current state."""
    n, G, dt = 50000, 64, 5e-4
    pos, vel, mass = scenes.make_scene("plummer", n, seed=6)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    ones = torch.ones(n, device=DEV)
    m = torch.from_numpy(mass).to(DEV)
    p1, v1 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    plan.run(p1, v1, m, ones, dt=dt, nsteps=3)
    p2, v2 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    rho = torch.empty((G,) * 3, device=DEV)
    plan.run_load(p2, v2, m, ones, dt=dt)
    plan.run_grid(rho, with_phi=True)
    assert torch.equal(rho, plan.deposit(torch.from_numpy(pos).to(DEV), m, ones))
    plan.run_load(p2, v2, m, ones, dt=dt)
    for k, (kick, drift) in enumerate([(0.5 * dt, True), (dt, True), (dt, True), (0.5 * dt, False)]):
        plan.run_grid(rho, with_phi=True)
        plan.run_kick(kick, drift)
    plan.run_unload(p2, v2)
    assert torch.equal(p1, p2) and torch.equal(v1, v2)


def test_energy_tap_matches_fp64_reduction():
    n, G = 30000, 32
    pos, vel, mass = scenes.make_scene("plummer", n, seed=8)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    p, v, m = (torch.from_numpy(x).to(DEV) for x in (pos, vel, mass))
    ones = torch.ones(n, device=DEV)
    e = torch.zeros(2, dtype=torch.float64, device=DEV)
    plan.run_load(p, v, m, ones, dt=1e-3)
    plan.run_grid(with_phi=True)
    plan.run_kick(0.0, False, energy_out=e, esync=0.0)
    _, phi = plan.force(p, m, ones, with_phi=True)
    ref = energy_fp64(v, m, ones, phi)
    ke, pe = e.tolist()
    assert abs(ke - ref["ke"]) < 1e-5 * abs(ref["ke"])
    assert abs(pe - ref["pe"]) < 1e-5 * abs(ref["pe"])


def test_corrected_step_runs_and_falls_back_to_plain_pm():
    n, G, dt = 20000, 32, 5e-4
    pos, vel, mass = scenes.make_scene("plummer", n, seed=9)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    net = GridCNN(DEV, seed=1, phi_scale=0.1, out_scale=1.0)
    g = torch.Generator().manual_seed(2)
    net.view["w_out"].copy_(torch.randn(3, 27, 32, generator=g) * 0.5)
    net.prepare()
    m = torch.from_numpy(mass).to(DEV)
    ones = torch.ones(n, device=DEV)
    # a correction far larger than the force trips the monitor on the first check
    mon = FallbackMonitor(corr_max=1e-6)
    sim = CorrectedPM(plan, net, mon, check_every=2)
    p, v = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    sim.begin(p, v, m, ones, dt=dt)
    sim.steps(4)
    sim.end(p, v)
    assert mon.reverted and "correction" in mon.reason
    # after the revert the scene runs plain PM: the same trajectory as a plain run from then on
    assert torch.isfinite(p).all() and torch.isfinite(v).all()
    # an untrained (zero output layer) net leaves the trajectory identical to plain PM
    net0 = GridCNN(DEV, seed=1, phi_scale=0.1)
    sim0 = CorrectedPM(plan, net0, FallbackMonitor(), check_every=0)
    p0, v0 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    sim0.begin(p0, v0, m, ones, dt=dt)
    sim0.steps(3)
    sim0.end(p0, v0)
    p1, v1 = torch.from_numpy(pos).to(DEV), torch.from_numpy(vel).to(DEV)
    plan.run(p1, v1, m, ones, dt=dt, nsteps=4)
    assert torch.equal(p0, p1) and torch.equal(v0, v1)
