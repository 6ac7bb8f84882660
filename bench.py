"""Benchmark of the plain-PM gravity step at 3M bodies on a 256^3 periodic grid.

One step = one leapfrog step of the whole scene on the GPU: re-sort by grid row, CIC
deposit + x R2C, y/z FFTs with the Green's function and spectral gradient, C2R, gather +
kick-drift. Inputs (3M-body Plummer sphere, a=0.05, in a unit periodic box; seeded,
synthetic) are resident in HBM before the timed region; the per-step working set
(~1.5 GB of traffic over ~0.8 GB of buffers) is larger than the 129 MB L2, so no flush.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload pm|batch64|pm1e9|pair|field2d|tick1e9]

The default workload is the one above; --workload batch64 steps 64 uneven scenes in one CUDA
graph, pm1e9 one 10^9-body scene on 1024^3, and pair / field2d / tick1e9 time the pair term,
the production 2D model and its 10^9-body fp16-state tick.

Prints one JSON line (rank 0). Under torchrun each rank runs an independent replica
(scenes are independent; the PM step has no inter-GPU exchange) and value is the
whole-job rate over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "body-steps/s at 3M bodies: CNN-corrected vs plain PM at equal force error"
STAGES = ("sort", "deposit_r2c", "fft_y_fwd", "fft_z_green", "fft_y_inv", "c2r", "gather_kd")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_bytes(n: int, G: int) -> dict:
    """Algorithmic bytes per launch of each stage (unpadded, FP32). C = half spectrum."""
    C = 8 * (G // 2 + 1) * G * G
    G3 = G ** 3
    return {
        "sort": 0,  # implementation overhead, not algorithmic
        "deposit_r2c": 16 * n + C,  # read bodies (x, y, z, m), write the x-transformed spectrum
        "fft_y_fwd": 2 * C,
        "fft_z_green": 4 * C,  # read 1 spectrum, write 3 gradient spectra
        "fft_y_inv": 6 * C,
        "c2r": 3 * C + 12 * G3,
        "gather_kd": 12 * G3 + 64 * n,  # force grid + body state read and written
    }


def step_bytes(n: int, G: int) -> int:
    """Algorithmic bytes of one PM step: 48 N + 32 G^3 + 8 C."""
    C = 8 * (G // 2 + 1) * G * G
    return 48 * n + 32 * G ** 3 + 8 * C


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.proc = None
        try:
            uuid = str(torch.cuda.get_device_properties(device).uuid)
            ident = uuid if uuid.startswith("GPU-") else f"GPU-{uuid}"
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={ident}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            return None
        sm, mx, pw, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
                pw.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        load = [s for s, p in zip(sm, pw) if p > 0.3 * max(pw)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_inputs(n: int, seed: int, scene: str = "plummer"):
    from augur_gb300 import scenes

    return scenes.make_scene(scene, n, seed=seed)


def cpu_baseline_run(n, G, dt, budget_s=20.0, warmup=0, steps=None):
    """The reference-idiom torch CPU step (oracle/pm_torch_cpu.py) on this host's cores, on the full
    workload: `warmup` untimed steps, then `steps` timed steps, cut short where they would exceed
    budget_s (at least one). Returns the steps and warm-up steps actually run."""
    from oracle.pm_torch_cpu import TorchCPUPM

    torch.set_num_threads(os.cpu_count() or 1)
    pos, vel, mass = make_inputs(n, 9100)
    p, v, m = torch.from_numpy(pos), torch.from_numpy(vel), torch.from_numpy(mass)
    sim = TorchCPUPM(G)
    sim.begin(p, v, m, dt)
    for _ in range(warmup):
        sim.step(p, v, m, dt)
    t0 = time.perf_counter()
    sim.step(p, v, m, dt)
    t1 = time.perf_counter() - t0
    done = 1
    want = steps if steps is not None else 10
    extra = max(0, min(want - 1, int(budget_s / max(t1, 1e-3)) - 1))
    t0 = time.perf_counter()
    for _ in range(extra):
        sim.step(p, v, m, dt)
    if extra:
        t1 = (t1 + time.perf_counter() - t0)
        done += extra
    return {"value": n * done / t1, "unit": "body-steps/s", "cores": torch.get_num_threads(), "kind": "port",
            "sample": f"{done} timed step(s) after {warmup} warm-up step(s) of the full {n}-body / {G}^3 workload "
                      f"(oracle/pm_torch_cpu.py, float32)",
            "s_per_step": t1 / done, "steps": done, "warmup": warmup}


def run_reference_widened(args, world):
    """CPU reference arm of the widened workloads: the oracle's float64 restatement of the
    reference's pair term, 2D model and large-N tick (oracle/pm_oracle.py, oracle/field2d_oracle.py)
    on a bounded sample of the same workload, single-threaded numpy."""
    from oracle import field2d_oracle as F
    from oracle import pm_oracle as O

    rng = np.random.default_rng(9100)
    sd = {k: v.numpy().astype(np.float64) for k, v in seeded_field2d_state().items()}
    t0 = time.time()
    if args.workload == "pair":
        n, q = args.bodies, 50
        pos = rng.normal(0.0, 10.7, (n, 2))
        params = np.concatenate([sd[f"ppmlp.{i}.{w}"].reshape(-1) for i in (0, 2, 4) for w in ("weight", "bias")])
        params[-65:] = np.linspace(-0.2, 0.2, 65)
        idx = np.arange(0, n, n // q)[:q]
        O.pair_acc_2d(pos, np.ones(n), np.ones(n), params, 2, [], 0, 0.5, 0.5, 0.5, 16, queries=idx)
        dt_s = time.time() - t0
        value, unit, sample = q / dt_s, "bodies/s", f"{q} query bodies of the {n}-body scene (brute-force top-knn)"
        metric = "pair-term bodies/s (knn 16, pair-weight MLP), 1e6 Gaussian bodies"
    elif args.workload == "field2d":
        n = args.bodies
        m = F.Model2D(sd)
        pos, vel = rng.uniform(-20, 20, (n, 2)), rng.normal(0, 1, (n, 2))
        one = np.ones(n)
        state = (np.zeros((1, 128, 128)), None)
        pos, vel, state, _ = m.step(pos, vel, one, one, state)  # the first step computes a_prev
        t0 = time.time()
        m.step(pos, vel, one, one, state)
        dt_s = time.time() - t0
        value, unit, sample = n / dt_s, "body-steps/s", f"one Verlet step of the {n}-body scene"
        metric = "body-steps/s of the production 2D model (U-Net, kernel and pair terms, Verlet)"
    else:
        n = 100_000
        m = F.Model2D(sd, pair=False)
        sim = F.Tick2D(m, n, c=10.0, dt=0.1, state_dtype=np.float16)
        pos = np.clip(rng.normal(0, 8.0, (n, 2)), -29, 29).astype(np.float16)
        mom = rng.normal(0, 3.0, (n, 2)).astype(np.float16)
        pos, mom = sim.init_kick(pos, mom)
        t0 = time.time()
        sim.tick(pos, mom)
        dt_s = time.time() - t0
        value, unit, sample = n / dt_s, "body-ticks/s", f"one tick of a {n}-body sample of the scene, fp16 state"
        metric = "body-ticks/s, 1e9-body 2D scene, fp16 state (chunked large-N tick)"
    cb = {"value": value, "unit": unit, "cores": 1, "kind": "port",
          "sample": sample + " (oracle float64 numpy restatement of the reference)"}
    print(json.dumps({"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": world,
                      "steps": 1, "warmup": 0, "ms_per_step": dt_s * 1e3, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": args.workload, "bodies": args.bodies}, "cpu_baseline": cb,
                      "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def run_reference(args, world, rank):
    if rank != 0:
        return
    if args.workload in ("pair", "field2d", "tick1e9"):
        run_reference_widened(args, world)
        return
    if args.workload != "pm":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm times the single-scene "
                                                              "workloads only"}), flush=True)
        return
    n, G = args.bodies, args.grid
    cb = cpu_baseline_run(n, G, args.dt, budget_s=120.0, warmup=min(args.warmup, 3), steps=args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "body-steps/s", "n_gpus": world,
            "steps": cb["steps"], "warmup": cb["warmup"], "requested_steps": args.steps,
            "requested_warmup": args.warmup, "ms_per_step": 1e3 * cb["s_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config(args):
    kind = {"plummer": "Plummer sphere (a=0.05)", "uniform": "uniform box", "clumpy": "64-clump scene",
            "disk": "exponential disk", "flyby": "Plummer flyby"}[args.scene]
    return {"workload": f"plain PM step, {args.bodies}-body {kind} in a unit periodic box, "
                        f"{args.grid}^3 FP32 grid, leapfrog dt={args.dt}",
            "bodies": args.bodies, "grid": args.grid, "scene": args.scene, "seed": 9100, "dt": args.dt,
            "l2": "per-step traffic ~1.5 GB over ~0.8 GB of buffers > 129 MB L2; no flush"}


def fp64_truth(pos_d, mass_d, n, ns=4096, seed=9100):
    """FP64 periodic (minimum image + Ewald) direct sum at ns sampled bodies, eps = 1/256."""
    from augur_gb300 import direct_sum_fp64

    idx = torch.from_numpy(np.random.default_rng(seed).choice(n, ns, replace=False)).to(pos_d.device)
    src = pos_d.double()
    truth = direct_sum_fp64(src[idx].contiguous(), src, mass_d.double(), eps=1.0 / 256, box=1.0,
                            target_index=idx.contiguous())
    return idx, truth


def force_error(a, truth):
    d = (a.double() - truth).norm(dim=1)
    rms = truth.norm(dim=1).pow(2).mean().sqrt()
    e = (d / rms).cpu().numpy()
    return {"vs": "FP64 periodic direct sum (min-image + Ewald), eps=1/256, 4096 sampled bodies",
            "rel_rms": float((d.pow(2).mean().sqrt() / rms).item()),
            "median_norm_by_rms": float(np.sort(e)[(len(e) - 1) // 2]), "p90_norm_by_rms": float(np.quantile(e, 0.9))}


def cnn_form(args, pos, vel, mass, dev, idx, truth, st):
    """The CNN-corrected step at 128^3 (trained weights) on the same bodies: body-steps/s, the
    network's share of the step against the tensor-pipe roofline, an end-to-end rate through the
    public API with pinned host buffers, and the force error at t = 0 and after the timed steps,
    beside plain PM at 128^3."""
    from augur_gb300 import PMPlan
    from augur_gb300.cnn import GridCNN
    from augur_gb300.learned import CorrectedPM, FallbackMonitor

    ck = ROOT / "augur_gb300" / "weights" / "scatter_cnn_g128.pt"
    if not ck.exists():
        return {"unavailable": f"no trained weights at {ck.relative_to(ROOT)}"}
    d = torch.load(ck, map_location="cpu", weights_only=False)
    G = int(d["grid"])
    n = args.bodies
    plan = PMPlan(3, G, n, "periodic", 1.0, device=dev)
    net = GridCNN(dev)
    net.load_state_dict(d["net"])
    p, v, m = (torch.from_numpy(x).to(dev) for x in (pos, vel, mass))
    ones = torch.ones(n, device=dev)

    def accuracy(pp, tgt, tr):
        rho = plan.deposit(pp, m, ones)
        F4 = plan.poisson(rho)
        tp = pp[tgt].contiguous()
        pm, _ = plan.gather(F4, tp)
        field = torch.zeros(G ** 3 * 4, device=dev)
        net.forward(net.input(rho, F4), 1, G, field)
        corr, _ = plan.gather(field.view(G, G, G, 4), tp)
        return force_error(pm + corr, tr), force_error(pm, tr), (rho, F4)

    acc0, pm0, (rho, F4) = accuracy(p, idx, truth)
    # the network alone on this grid (CUDA events), for its tensor-pipe roofline
    x = net.input(rho, F4)
    field = torch.zeros(G ** 3 * 4, device=dev)
    for _ in range(3):
        net.forward(x, 1, G, field)
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(st)
    for _ in range(10):
        net.forward(x, 1, G, field)
    a1.record(st)
    torch.cuda.synchronize(dev)
    net_ms = a0.elapsed_time(a1) / 10
    flop = 174528.0 * G ** 3  # forward flops per voxel x voxels (2 x 27 x (2*32 + 3*32*32 + 32*3))
    pk = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak_s, peak_b = float(pk.get("bf16_tflops_sustained", 1700.0)), float(pk.get("bf16_tflops", 1900.0))
    tflops = flop / (net_ms * 1e-3) / 1e12
    # throughput of the corrected leapfrog (monitor checks every 10 steps)
    sim = CorrectedPM(plan, net, FallbackMonitor(), check_every=10)
    pe, ve = p.clone(), v.clone()
    sim.begin(pe, ve, m, ones, dt=args.dt)
    sim.steps(3)
    torch.cuda.synchronize(dev)
    k = max(10, min(200, args.steps // 5))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    sim.steps(k)
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / k
    sim.end(pe, ve)
    net.check()
    # accuracy after the timed steps, against a fresh FP64 truth at the evolved positions
    idx1, truth1 = fp64_truth(pe, m, n, seed=9101)
    acc1, pm1, _ = accuracy(pe, idx1, truth1)
    # end to end through the public API: one corrected step per call on caller tensors copied in from
    # and out to pinned host memory (CorrectedPM.begin / steps(1) / end)
    h_pos, h_vel = torch.from_numpy(pos).pin_memory(), torch.from_numpy(vel).pin_memory()
    d_pos, d_vel = torch.empty_like(p), torch.empty_like(v)
    sim2 = CorrectedPM(plan, net, FallbackMonitor(), check_every=10)

    def e2e_step():
        d_pos.copy_(h_pos, non_blocking=True)
        d_vel.copy_(h_vel, non_blocking=True)
        sim2.begin(d_pos, d_vel, m, ones, dt=args.dt)
        sim2.steps(1)
        sim2.end(d_pos, d_vel)
        h_pos.copy_(d_pos, non_blocking=True)
        h_vel.copy_(d_vel, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize(dev)
    ke = 5
    e0.record(st)
    for _ in range(ke):
        e2e_step()
    e1.record(st)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1) / ke
    return {"form": "CNN-corrected PM", "grid": G, "value": n / (ms * 1e-3), "unit": "body-steps/s",
            "ms_per_step": ms, "steps": k, "monitor_check_every": 10, "reverted_to_plain_pm": sim.monitor.reverted,
            "roofline": {"bound": "tensor", "kernel": "GridCNN.forward (5 tcgen05 conv layers)", "achieved": tflops,
                         "peak": peak_s, "unit": "TFLOP/s", "frac": tflops / peak_s, "peak_kind": "measured sustained",
                         "frac_of_burst": tflops / peak_b, "forward_ms": net_ms, "flop_per_forward": flop,
                         "share_of_step": net_ms / ms, "traffic": None},
            "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "body-steps/s", "h2d_bytes_per_step": 24 * n,
                    "d2h_bytes_per_step": 24 * n,
                    "api": "augur_gb300.learned.CorrectedPM begin / steps(1) / end on pinned host buffers"},
            "accuracy": acc0, "plain_pm_same_grid_accuracy": pm0,
            "accuracy_after_steps": {"steps": k + 3, "cnn": acc1, "plain_pm_same_grid": pm1},
            "weights": str(ck.relative_to(ROOT)), "trained": {k2: d.get(k2) for k2 in ("bodies", "grid", "eps")}}


def run_ours(args, world, rank, local):
    from augur_gb300 import PMPlan

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    n, G, dt = args.bodies, args.grid, args.dt
    pos, vel, mass = make_inputs(n, 9100 + rank, args.scene)
    pos_d, vel_d, mass_d = (torch.from_numpy(x).to(dev) for x in (pos, vel, mass))
    ones = torch.ones(n, device=dev)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=dev)
    st = torch.cuda.current_stream(dev)

    p, v = pos_d.clone(), vel_d.clone()
    plan.run_begin(p, v, mass_d, ones, dt=dt)
    plan.run_steps(args.warmup)
    torch.cuda.synchronize(dev)

    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    plan.run_steps(args.steps)
    e1.record(st)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    launches = plan.last_launches
    plan.check()
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms = ms_total / args.steps

    stages = plan.run_profile(20)
    plan.run_end(p, v)
    torch.cuda.synchronize(dev)

    # end to end through the public API: a velocity-Verlet step on caller tensors that live in
    # pinned host memory, copied in and out every step
    h_pos, h_vel = torch.from_numpy(pos).pin_memory(), torch.from_numpy(vel).pin_memory()
    h_acc = torch.zeros_like(h_pos).pin_memory()
    d_pos, d_vel, d_acc = torch.empty_like(pos_d), torch.empty_like(vel_d), torch.empty_like(pos_d)
    k_e2e = max(3, min(args.steps, 50))

    def e2e_step(first):
        # the host-buffer entry point: chunked copies in and out overlap the step's kernels
        plan.step_host(h_pos, h_vel, h_acc, mass_d, ones, dt=dt, have_acc=not first)

    def copy_step(first):
        # the same step through the device entry point with whole-array copies around it
        d_pos.copy_(h_pos, non_blocking=True)
        d_vel.copy_(h_vel, non_blocking=True)
        d_acc.copy_(h_acc, non_blocking=True)
        plan.step(d_pos, d_vel, d_acc, mass_d, ones, dt=dt, have_acc=not first)
        h_pos.copy_(d_pos, non_blocking=True)
        h_vel.copy_(d_vel, non_blocking=True)
        h_acc.copy_(d_acc, non_blocking=True)

    def time_e2e(fn):
        fn(True)
        fn(False)
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(k_e2e):
            fn(False)
        e1.record(st)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / k_e2e

    e2e_ms = time_e2e(e2e_step)
    copy_ms = time_e2e(copy_step)

    acc_info, cnn_info = None, None
    if not args.no_accuracy and rank == 0:
        idx, truth = fp64_truth(pos_d, mass_d, n)
        acc_info = force_error(plan.force(pos_d, mass_d, ones)[idx], truth)
        if not args.no_cnn:
            cnn_info = cnn_form(args, pos, vel, mass, dev, idx, truth, st)
            if "accuracy" in cnn_info:
                cnn_info["equal_or_lower_error_than_plain_pm"] = \
                    cnn_info["accuracy"]["rel_rms"] <= acc_info["rel_rms"]

    if rank != 0:
        return
    peak, peak_kind = peaks()
    sb = stage_bytes(n, G)
    dom = max(stages, key=stages.get)
    ach = sb[dom] / (stages[dom] * 1e-3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "ncu_traffic.json"
    if tp.exists():
        tr = json.loads(tp.read_text()).get(f"{n}x{G}", {})
        traffic = tr.get(dom)
    B = step_bytes(n, G)
    cb = cpu_baseline_run(n, G, dt) if (world == 1 and not args.no_cpu) else None
    line = {
        "metric": METRIC, "value": world * n / (ms * 1e-3), "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(args),
        "form": "plain PM",
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": sb[dom]},
        "step_roofline": {"bound": "hbm", "algorithmic_bytes": B, "achieved": B / (ms * 1e-3) / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": B / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind},
        "stages_ms": stages,
        "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": "body-steps/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": 36 * n, "ms_per_step": e2e_ms,
                "api": "augur_gb300.PMPlan.step_host (augur_pm_step_host) on pinned host buffers",
                "copies_around_device_step": {"value": world * n / (copy_ms * 1e-3), "ms_per_step": copy_ms,
                                              "api": "PMPlan.step (augur_pm_step) with whole-array copies"}},
        "gpu_launches": launches,
        "clocks": clk,
        "accuracy": acc_info,
        "cnn_corrected": cnn_info,
        "cpu_baseline": None if cb is None else {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
    }
    print(json.dumps(line), flush=True)


def run_batch(args, world, rank, local):
    """64 independent scenes, N log-uniform in [1e4, 1e6], grids 64/96/128 at ~8 cells per body,
    stepped together by CUDA-graph replay (two merged steps per replay); plain PM for all and the
    CNN-corrected form for the 128^3 scenes (trained weights), beside the same scenes run one after
    another without the graph. Replicas only under torchrun (each rank its own batch)."""
    from augur_gb300 import PMPlan
    from augur_gb300.batch import BatchedPM, make_batch
    from augur_gb300.cnn import GridCNN

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    st = torch.cuda.current_stream(dev)
    K = args.steps + (args.steps % 2)
    W = args.warmup + (args.warmup % 2)
    t0 = time.time()
    batch = make_batch(64, 1e4, 1e6, seed=9100 + rank)
    gen_s = time.time() - t0

    def timed(fn):
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b)

    # plain PM, all scenes on per-scene graph branches (16 capture streams)
    simb = BatchedPM(batch, dt=args.dt, streams=args.streams)
    simb.begin()
    branch_launches = sum(s["plan"].last_launches for s in simb.scenes)
    simb.steps(W)
    branch_ms = timed(lambda: simb.steps(K)) / K
    simb.end()
    simb.close()
    # plain PM, one launch per stage for all scenes
    sim = BatchedPM(batch, dt=args.dt, fused=True)
    sim.begin()
    launches_per_step = 11
    sim.steps(W)
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    ms_total = timed(lambda: sim.steps(K))
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    sim.end()
    for s in sim.scenes:
        s["plan"].check()
    ms = ms_total / K
    bodies = sim.bodies
    nbytes = sum(step_bytes(s["n"], s["grid"]) for s in sim.scenes)
    tiles_cached = sum(1 for s in sim.scenes if s["tuned"])
    plain_err = sim.force_errors(ntarget=1024) if not args.no_accuracy else None
    sim.close()

    # the same scenes one after another on one stream, no graph
    seq_ms = 0.0
    for sc in batch:
        plan = PMPlan(3, sc["grid"], sc["n"], "periodic", 1.0, device=dev)
        from augur_gb300 import autotune
        tl = autotune.tiles_for(sc["grid"], sc["n"])
        if tl:
            plan.set_tiles(tl)
        p, v, m = (torch.from_numpy(x).to(dev) for x in (sc["pos"], sc["vel"], sc["mass"]))
        plan.run_begin(p, v, m, dt=args.dt)
        plan.run_steps(W)
        seq_ms += timed(lambda: plan.run_steps(K))
        plan.close()
    seq_ms /= K

    # CNN-corrected form on the scenes whose grid has trained weights
    cnn = None
    nets = {}
    for ck in sorted((ROOT / "augur_gb300" / "weights").glob("scatter_cnn_g*.pt")):
        d = torch.load(ck, map_location="cpu", weights_only=False)
        net = GridCNN(dev)
        net.load_state_dict(d["net"])
        nets[int(d["grid"])] = net
    if nets and not args.no_cnn:
        simc = BatchedPM(batch, dt=args.dt, nets=nets, streams=args.streams, check_every=10)
        simc.begin()
        simc.steps(W)
        cms = timed(lambda: simc.steps(K)) / K
        simc.end()
        errs = simc.force_errors(ntarget=1024) if not args.no_accuracy else None
        ncnn = sum(1 for s in simc.scenes if s["monitor"] is not None)
        cnn = {"form": "CNN-corrected PM on the scenes whose grid has trained weights "
                       f"({sorted(nets)}), plain PM on the others",
               "value": bodies / (cms * 1e-3), "unit": "body-steps/s", "ms_per_step": cms,
               "cnn_scenes": ncnn, "reverted_to_plain_pm": sum(1 for s in simc.scenes if s["monitor"] is not None
                                                                and s["monitor"].reverted),
               "monitor_check_every": 10, "per_scene_error": errs}
        simc.close()

    if rank != 0:
        return
    peak, peak_kind = peaks()

    def summary(rows, key):
        v = [r[key] for r in rows if key in r]
        return None if not v else {"mean": float(np.mean(v)), "max": float(np.max(v)), "scenes": len(v)}

    line = {
        "metric": "aggregate body-steps/s of 64 uneven periodic scenes stepped together", "value":
            world * bodies / (ms * 1e-3), "unit": "body-steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "64 scenes (plummer/uniform/clumpy/disk/flyby in turn), N log-uniform in [1e4, 1e6], "
                               "grid 64/96/128 at >= 8 cells per body, leapfrog dt=%g, one launch per stage"
                               % args.dt, "bodies": bodies, "seed": 9100,
                   "grids": {str(g): sum(1 for s in batch if s["grid"] == g) for g in (64, 96, 128)},
                   "streams": args.streams, "scene_generation_s": round(gen_s, 1),
                   "l2": "per-step traffic %.2f GB > 129 MB L2; no flush" % (nbytes / 1e9)},
        "form": "plain PM",
        "step_roofline": {"bound": "hbm", "algorithmic_bytes": nbytes, "achieved": nbytes / (ms * 1e-3) / 1e9,
                          "peak": peak, "unit": "GB/s", "frac": nbytes / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind},
        "form_detail": "one launch per stage for all 64 scenes (augur_pm_batch_run_steps), 2 steps per graph",
        "graph_branches": {"value": bodies / (branch_ms * 1e-3), "ms_per_step": branch_ms,
                           "launches_per_step": branch_launches,
                           "what": "one plan per scene, run_steps on 16 capture streams in one CUDA graph"},
        "sequential_no_graph": {"value": bodies / (seq_ms * 1e-3), "ms_per_step": seq_ms,
                                "what": "the same plans one after another on one stream, run_steps per scene"},
        "gpu_launches": launches_per_step * K,
        "tiles": {"autotuned_scenes": tiles_cached, "source": "augur_gb300/tiles_gb300.json"},
        "clocks": clk,
        "accuracy_plain_pm": None if plain_err is None else {
            "vs": "FP64 periodic direct sum (min-image + Ewald), eps=1/256, 1024 sampled bodies per scene, "
                  "state after the run", "rel_rms": summary(plain_err, "plain_pm"), "per_scene": plain_err},
        "cnn_corrected": cnn,
    }
    print(json.dumps(line), flush=True)


def run_1e9(args, world, rank, local):
    """One 10^9-body Plummer sphere on a 1024^3 grid, generated on the GPU; 20 merged steps timed;
    force error at 4096 targets vs the FP64 periodic direct sum over a 10^6-body subsample."""
    from augur_gb300 import PMPlan, direct_sum_fp64, scenes

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n, G, dt = args.bodies, args.grid, args.dt
    st = torch.cuda.current_stream(dev)
    t0 = time.time()
    pos = torch.empty(n, 3, device=dev)
    vel = torch.empty(n, 3, device=dev)
    scenes.plummer_device(pos, vel, seed=9100 + rank)
    mass = torch.full((n,), 1.0 / n, device=dev)
    mask = torch.ones(n, device=dev)
    torch.cuda.synchronize(dev)
    gen_s = time.time() - t0
    plan = PMPlan(3, G, n, "periodic", 1.0, device=dev)
    acc = None
    if not args.no_accuracy:
        # the sub-op path (deposit, Poisson solve, gather at the targets) before the run is loaded
        ns, nt = 1_000_000, 4096
        g = torch.Generator(device=dev)
        g.manual_seed(9300)
        sub = torch.randint(0, n, (ns,), device=dev, generator=g)
        src = pos[sub].double().contiguous()
        rho = plan.deposit(pos, mass, mask)
        F4 = plan.poisson(rho)
        del rho
        pm = plan.gather(F4, pos[sub[:nt]].contiguous())[0]
        del F4
        torch.cuda.empty_cache()
        truth = direct_sum_fp64(src[:nt].contiguous(), src, torch.full((ns,), 1.0 / ns, dtype=torch.float64,
                                device=dev), eps=1.0 / G, box=1.0,
                                target_index=torch.arange(nt, device=dev, dtype=torch.int64))
        acc = force_error(pm, truth)
        acc["vs"] = ("FP64 periodic direct sum (min-image + Ewald), eps=1/%d, over a 10^6-body random subsample "
                     "(masses scaled to the total), %d targets; the subsample's shot noise is part of the error" % (G, nt))
        del src, sub
    plan.run_begin(pos, vel, mass, mask, dt=dt)
    plan.run_steps(args.warmup)
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    plan.run_steps(args.steps)
    b.record(st)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    ms = a.elapsed_time(b) / args.steps
    launches = plan.last_launches
    stages = plan.run_profile(2)
    plan.check()
    if rank != 0:
        return
    peak, peak_kind = peaks()
    B = step_bytes(n, G)
    sb = stage_bytes(n, G)
    dom = max(stages, key=stages.get)
    ach = sb[dom] / (stages[dom] * 1e-3) / 1e9 if sb[dom] else None
    line = {
        "metric": "body-steps/s, one 1e9-body scene", "value": world * n / (ms * 1e-3), "unit": "body-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain PM step, {n}-body Plummer sphere (a=0.05, generated on the GPU) in a unit "
                               f"periodic box, {G}^3 FP32 grid, leapfrog dt={dt}", "bodies": n, "grid": G,
                   "scene_generation_s": round(gen_s, 1), "workspace_gb": plan.workspace_bytes / 1e9,
                   "l2": "per-step traffic %.0f GB >> L2; no flush" % (B / 1e9)},
        "form": "plain PM",
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": None if ach is None else ach / peak, "peak_kind": peak_kind, "algorithmic_bytes": sb[dom]},
        "step_roofline": {"bound": "hbm", "algorithmic_bytes": B, "achieved": B / (ms * 1e-3) / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": B / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind},
        "stages_ms": stages, "gpu_launches": launches, "clocks": clk, "accuracy": acc,
        "e2e": None, "e2e_note": "not measured: the 24 GB body state does not round-trip through host memory per step",
    }
    print(json.dumps(line), flush=True)


def seeded_field2d_state(seed: int = 4738) -> dict:
    """Parameters of the production 2D model under the reference's names, drawn as torch's default
    Linear / Conv2d initialisation does (uniform, bound 1/sqrt(fan_in)), with the output layers of
    the pair MLP, the kernel MLP and the U-Net zeroed as the reference initialises them
    (scripts/scatter_field.py:123-136). The work per step does not depend on the values."""
    g = torch.Generator().manual_seed(seed)
    shapes = {}
    for pre in ("ppmlp", "kmlp"):
        shapes.update({f"{pre}.0.weight": (64, 2), f"{pre}.0.bias": (64,), f"{pre}.2.weight": (64, 64),
                       f"{pre}.2.bias": (64,), f"{pre}.4.weight": (1, 64), f"{pre}.4.bias": (1,)})
    shapes.update({"net.inp.weight": (32, 6, 3, 3), "net.inp.bias": (32,)})
    for blk, cin in [(f"enc.{l}", 32) for l in range(6)] + [(f"dec.{l}", 64) for l in range(5)]:
        shapes.update({f"net.{blk}.0.weight": (32, cin, 3, 3), f"net.{blk}.0.bias": (32,),
                       f"net.{blk}.2.weight": (32, 32, 3, 3), f"net.{blk}.2.bias": (32,)})
    shapes.update({"net.out.weight": (1, 32, 3, 3), "net.out.bias": (1,)})
    sd = {}
    for k, shp in shapes.items():
        wshape = shapes[k.replace(".bias", ".weight")]
        fan_in = int(np.prod(wshape[1:]))
        b = 1.0 / math.sqrt(fan_in)
        sd[k] = (torch.rand(shp, generator=g) * 2 - 1) * b
    for k in ("ppmlp.4.weight", "ppmlp.4.bias", "kmlp.4.weight", "kmlp.4.bias", "net.out.weight", "net.out.bias"):
        sd[k].zero_()
    return sd


def _line(args, world, metric, value, unit, ms, config, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
         "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic",
         "config": config}
    d.update(extra)
    return d


def run_widened(args, world, rank, local):
    """The widened rows: the pair term (--workload pair), the production 2D model's Verlet step
    (--workload field2d) and its chunked large-N tick at 10^9 bodies in fp16 (--workload tick1e9)."""
    from augur_gb300 import ChunkedTick2D, PMPlan, UNetScatterField

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream(dev)
    K, W = args.steps, args.warmup
    g = torch.Generator(device=dev)
    g.manual_seed(9100 + rank)

    def timed(fn):
        for _ in range(W):
            fn()
        torch.cuda.synchronize(dev)
        clocks = Clocks(local)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(K):
            fn()
        b.record(st)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / K
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms, clocks.stop()

    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12  # nominal FP32 FMA rate, TFLOP/s (no measured FP32 peak)
    if args.workload == "pair":
        n, ppe, knn, sigma = args.bodies, 0.5, 16, 10.7
        pos = (torch.randn(n, 2, device=dev, generator=g) * sigma).contiguous()
        mass, mask = torch.ones(n, device=dev), torch.ones(n, device=dev)
        params = torch.cat([t.reshape(-1) for k, t in seeded_field2d_state().items() if k.startswith("ppmlp")]).to(dev)
        params[-65:] = torch.linspace(-0.2, 0.2, 65)  # non-zero output layer
        plan = PMPlan(2, 128, n, "isolated", 64.0, eps=0.5, device=dev)
        plan.pair_acc(pos, mass, mask, ppe=ppe, knn=knn, params=params, ncol=2)
        ms, clk = timed(lambda: plan.pair_acc(pos, mass, mask, ppe=ppe, knn=knn, params=params, ncol=2))
        launches = plan.last_launches
        # end to end: host buffers in, accelerations back, every step
        hp, hm = pos.cpu().pin_memory(), mass.cpu().pin_memory()
        ha = torch.empty(n, 2).pin_memory()

        def e2e():
            p, m_ = hp.to(dev, non_blocking=True), hm.to(dev, non_blocking=True)
            a = plan.pair_acc(p, m_, m_, ppe=ppe, knn=knn, params=params, ncol=2)
            ha.copy_(a, non_blocking=True)
        ems, _ = timed(e2e)
        flop = n * knn * 2 * (64 * 2 + 64 * 64 + 64 + 64 + 64)  # MLP FMAs of the knn pairs (an upper bound)
        cpu = None
        if rank == 0 and not args.no_cpu:
            from oracle import pm_oracle as O
            q = np.arange(0, n, n // 100)[:100]
            pn, mn = pos.cpu().numpy(), np.ones(n, np.float32)
            t0 = time.time()
            O.pair_acc_2d(pn, mn, mn, params.cpu().numpy(), 2, [], 0, ppe, 0.5, 0.5, knn, queries=q)
            cpu = {"value": len(q) / (time.time() - t0), "unit": "bodies/s", "cores": 1, "kind": "port",
                   "sample": "100 query bodies of the same scene, float64 brute-force top-knn (oracle/pm_oracle.py)"}
        if rank:
            return
        print(json.dumps(_line(
            args, world, "pair-term bodies/s (knn 16, pair-weight MLP), 1e6 Gaussian bodies", world * n / (ms * 1e-3),
            "bodies/s", ms, {"workload": f"pair term of ScatterField.pp_acc: {n} bodies N(0, {sigma}^2) in 2D, "
                                         f"ppe {ppe}, knn {knn}, MLP 2-64-64-1", "bodies": n},
            dtype="f32", gpu_launches=launches * K, clocks=clk,
            roofline={"bound": "fp32", "kernel": "pair_weight_tc_kernel (with the search)",
                      "achieved": flop / (ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                      "frac": flop / (ms * 1e-3) / 1e12 / fp32_peak,
                      "peak_kind": "nominal FP32 (152 SMs x 128 FMA x 2.07 GHz); achieved counts the MLP as fp32 "
                                   "flops although its 64x64 layer runs on tcgen05 (3 BF16 products) and only the "
                                   "GELUs and layers 1 and 3 on the CUDA cores, which bound it", "traffic": None},
            e2e={"value": world * n / (ems * 1e-3), "unit": "bodies/s", "h2d_bytes_per_step": 12 * n,
                 "d2h_bytes_per_step": 8 * n},
            cpu_baseline=cpu)), flush=True)
        return
    m = UNetScatterField(device=dev)
    m.load_state_dict(seeded_field2d_state())
    if args.workload == "field2d":
        n = args.bodies
        pos = (torch.rand(1, n, 2, device=dev, generator=g) * 40 - 20).contiguous()
        vel = torch.randn(1, n, 2, device=dev, generator=g).contiguous()
        mass, mask = torch.ones(1, n, device=dev), torch.ones(1, n, device=dev)
        state = {"p": pos, "v": vel, "f": m.init_field(1)}

        def step():
            state["p"], state["v"], state["f"], _ = m.step(state["p"], state["v"], mass, mask, state["f"])
        ms, clk = timed(step)
        flop = 2 * 1_039_000_000 * 2  # U-Net MACs per forward (levels 5, width 32, 128^2) x 2 flop
        # a batch of 64 small scenes (100 bodies each, the reference's training scale) in one call
        B, nb = 64, 100
        bst = {"p": (torch.rand(B, nb, 2, device=dev, generator=g) * 20 - 10).contiguous(),
               "v": torch.randn(B, nb, 2, device=dev, generator=g).contiguous(), "f": m.init_field(B)}
        bm = torch.ones(B, nb, device=dev)

        def bstep():
            bst["p"], bst["v"], bst["f"], _ = m.step(bst["p"], bst["v"], bm, bm, bst["f"])
        bms, _ = timed(bstep)
        # the same batch with the step captured in a CUDA graph (graph=True)
        mg = UNetScatterField(device=dev, graph=True)
        mg.load_state_dict(seeded_field2d_state())
        gst = {"p": bst["p"].clone(), "v": bst["v"].clone(), "f": mg.init_field(B)}

        def gstep():
            gst["p"], gst["v"], gst["f"], _ = mg.step(gst["p"], gst["v"], bm, bm, gst["f"])
        gstep()  # the first step computes a_prev eagerly; the next ones replay the graph
        gms, _ = timed(gstep)
        if rank:
            return
        print(json.dumps(_line(
            args, world, "body-steps/s of the production 2D model (U-Net, kernel and pair terms, Verlet)",
            world * n / (ms * 1e-3), "body-steps/s", ms,
            {"workload": f"ScatterField(grid=128, extent=64, net=unet, kernel, pp=2, split, potential, verlet): one "
                         f"scene of {n} uniform bodies, dt 0.1, seeded weights (reference init)", "bodies": n},
            dtype="f32", clocks=clk,
            roofline={"bound": "fp32", "kernel": "U-Net (f2_conv3_kernel)", "achieved": flop / 2 / (ms * 1e-3) / 1e12,
                      "peak": fp32_peak, "unit": "TFLOP/s", "frac": flop / 2 / (ms * 1e-3) / 1e12 / fp32_peak,
                      "peak_kind": "nominal FP32; achieved counts the U-Net's flops over the whole step", "traffic": None},
            batch64={"scenes": B, "bodies_per_scene": nb, "ms_per_step": bms,
                     "value": world * B * nb / (bms * 1e-3), "unit": "body-steps/s",
                     "what": "64 scenes stepped together: one U-Net launch sequence for the batch",
                     "graph_ms_per_step": gms, "graph_value": world * B * nb / (gms * 1e-3)},
            cpu_baseline=None, cpu_note="the reference's own CPU path cannot run on this host (it is not installed here); "
                                               "--impl reference times the oracle's restatement of it")),
            flush=True)
        return
    # tick1e9: the reference's initial conditions (scripts/scatter_bh_1b.py:66-104, gaussian), fp16 state
    n, c, sigma = args.bodies, 10.0, 8.0
    pos = torch.empty(n, 2, device=dev, dtype=torch.float16)
    mom = torch.empty(n, 2, device=dev, dtype=torch.float16)
    vscale = 0.3 * math.sqrt(n / (4 * sigma))
    chunk = 50_000_000
    for s0 in range(0, n, chunk):
        e0 = min(n, s0 + chunk)
        p = (torch.randn(e0 - s0, 2, device=dev, generator=g) * sigma).clamp_(-29.0, 29.0)
        v = torch.randn(e0 - s0, 2, device=dev, generator=g) * vscale
        vmag = v.norm(dim=-1, keepdim=True).clamp(max=0.99 * c)
        v = v / v.norm(dim=-1, keepdim=True).clamp_min(1e-30) * vmag
        pos[s0:e0] = p.half()
        mom[s0:e0] = (v * (1 - (vmag / c) ** 2).clamp(min=1e-6).rsqrt()).half()
        del p, v, vmag
    sim = ChunkedTick2D(m, n, c=c, dt=0.1, pos_dtype=torch.float16, mom_dtype=torch.float16)
    sim.init_kick(pos, mom)
    ms, clk = timed(lambda: sim.tick(pos, mom))
    ok = bool(torch.isfinite(mom[: 1 << 20].float()).all())
    peak, peak_kind = peaks()
    B = 16 * n  # fp16 pos and momentum read once and written once
    if rank:
        return
    print(json.dumps(_line(
        args, world, "body-ticks/s, 1e9-body 2D scene, fp16 state (chunked large-N tick)", world * n / (ms * 1e-3),
        "body-ticks/s", ms,
        {"workload": f"Sim.tick of scripts/scatter_bh_1b.py: {n} unit-mass bodies, Gaussian sigma {sigma} clipped "
                     f"to +-29, relativistic c={c}, dt 0.1, fp16 pos and momentum, production 2D model without "
                     f"the pair term, seeded weights (reference init)", "bodies": n,
         "l2": "per-tick traffic %.0f GB >> L2; no flush" % (B / 1e9)},
        dtype="f16 state / f32 arithmetic", clocks=clk, finite=ok,
        step_roofline={"bound": "hbm", "algorithmic_bytes": B, "achieved": B / (ms * 1e-3) / 1e9, "peak": peak,
                       "unit": "GB/s", "frac": B / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind},
        reference_published={"ms_per_tick": 1325.0, "hardware": "H200 NVL", "source": "results/scatter_bh_1b.json"},
        cpu_baseline=None, cpu_note="the reference's Sim.tick cannot run on this host (it is not installed here); "
                                               "--impl reference times the oracle's restatement of it")),
        flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", choices=("pm", "batch64", "pm1e9", "pair", "field2d", "tick1e9"), default="pm",
                    help="pm: one 3M-body scene on 256^3 (default); batch64: 64 uneven scenes in one graph; "
                         "pm1e9: one 1e9-body scene on 1024^3; pair: the pair term at 1e6 bodies; field2d: the "
                         "production 2D model; tick1e9: its chunked large-N tick at 1e9 bodies, fp16 state")
    ap.add_argument("--streams", type=int, default=16)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--bodies", type=int, default=None)
    ap.add_argument("--grid", type=int, default=None)
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-cnn", action="store_true")
    ap.add_argument("--scene", default="plummer", choices=("plummer", "uniform", "clumpy", "disk", "flyby"))
    args = ap.parse_args()
    defaults = {"pm": (2000, 3_000_000, 256, 5e-4), "batch64": (100, None, None, 5e-4),
                "pm1e9": (20, 1_000_000_000, 1024, 2.5e-4), "pair": (20, 1_000_000, 128, 0.1),
                "field2d": (50, 10_000, 128, 0.1), "tick1e9": (10, 1_000_000_000, 128, 0.1)}[args.workload]
    for k, v in zip(("steps", "bodies", "grid", "dt"), defaults):
        if getattr(args, k) is None:
            setattr(args, k, v)
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "batch64":
        run_batch(args, world, rank, local)
    elif args.workload == "pm1e9":
        run_1e9(args, world, rank, local)
    elif args.workload in ("pair", "field2d", "tick1e9"):
        run_widened(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
