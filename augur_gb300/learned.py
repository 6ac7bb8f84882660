"""CNN-corrected PM: training data, training, evaluation, and the corrected leapfrog step.

The correction is learned from pairs the method generates itself: for each seeded snapshot
the plain-PM force and the FP64 (Ewald-periodic) direct-sum force at sampled bodies; the
label is their difference (the role of the reference's truth-vs-model force error,
scripts/pm_baseline_force_error.py:88-92, turned into a training target). The network sees
the CIC density and PM potential grids and outputs a 3-channel correction field that is
CIC-gathered at the bodies and added to the PM force.

Plain PM is the fallback and the yardstick: FallbackMonitor reverts a scene to plain PM when its
relative energy drift exceeds 5% or the predicted correction grows beyond a fraction of the
PM force (the reference's energy drift diagnostic, scripts/scatter_field.py:759-765, :874).
"""
from __future__ import annotations

import math
import os
import signal
import threading
import time

import numpy as np
import torch

from . import scenes
from .cnn import GridCNN
from .pm import PMPlan, direct_sum_fp64


# ---------------------------------------------------------------------------------------------
# data
# ---------------------------------------------------------------------------------------------
def make_snapshot(plan: PMPlan, net: GridCNN, kind: str, n: int, seed: int, n_targets: int = 8192,
                  eps: float = 1.0 / 256, box: float = 1.0) -> dict:
    """One labelled snapshot on plan's grid: CNN input x (bf16), target positions and the
    (FP64 direct sum - PM) force at them."""
    dev = plan.device
    pos, _, mass = scenes.make_scene(kind, n, seed=seed, box=box)
    p = torch.from_numpy(pos).to(dev)
    m = torch.from_numpy(mass).to(dev)
    ones = torch.ones(n, device=dev)
    rho = plan.deposit(p, m, ones)
    F4 = plan.poisson(rho)
    rng = np.random.default_rng(seed + 17)
    idx = torch.from_numpy(rng.choice(n, size=min(n_targets, n), replace=False)).to(dev)
    tpos = p[idx].contiguous()
    pm, _ = plan.gather(F4, tpos)
    src = p.double()
    truth = direct_sum_fp64(src[idx].contiguous(), src, m.double(), eps=eps, box=box, target_index=idx.contiguous())
    x = net.input(rho, F4)
    return {"kind": kind, "seed": seed, "x": x, "tpos": tpos, "pm": pm, "truth": truth.float(),
            "label": (truth - pm.double()).float()}


def _scene_job(args):
    kind, n, seed = args
    pos, _, mass = scenes.make_scene(kind, n, seed=seed)
    return pos, mass


def make_truth(n: int, count: int, seed0: int, device, kinds=scenes.SCENES, n_targets: int = 8192,
               eps: float = 1.0 / 256, workers: int = 0, log=None) -> list:
    """The grid-independent half of a dataset: seeded scenes (kind i % len(kinds), seed seed0 + i)
    kept on the device, the sampled target indices and the FP64 periodic direct-sum force at them.
    label_snapshots() adds a grid's PM force and CNN input, so one truth serves every grid.
    workers > 0 samples the scenes on that many host processes (spawned; no CUDA in them)."""
    jobs = [(kinds[i % len(kinds)], n, seed0 + i) for i in range(count)]
    if workers > 0:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor

        ex = ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"))
        it = ex.map(_scene_job, jobs, chunksize=4)
    else:
        ex, it = None, map(_scene_job, jobs)
    out = []
    t0 = time.time()
    try:
        for i, ((kind, _, seed), (pos, mass)) in enumerate(zip(jobs, it)):
            p = torch.from_numpy(pos).to(device)
            m = torch.from_numpy(mass).to(device)
            rng = np.random.default_rng(seed + 17)
            idx = torch.from_numpy(rng.choice(n, size=min(n_targets, n), replace=False)).to(device)
            src = p.double()
            truth = direct_sum_fp64(src[idx].contiguous(), src, m.double(), eps=eps, box=1.0,
                                    target_index=idx.contiguous())
            out.append({"kind": kind, "seed": seed, "pos": p, "mass": m, "idx": idx, "truth64": truth})
            if log and (i + 1) % max(1, count // 10) == 0:
                log(f"truth {i + 1}/{count} ({time.time() - t0:.1f} s)")
    finally:
        if ex is not None:
            ex.shutdown()
    return out


def label_snapshots(plan: PMPlan, net: GridCNN, truths: list) -> list:
    """Snapshots on plan's grid from make_truth() entries: CNN input, target positions, PM force and
    the (FP64 direct sum - PM) label, as make_snapshot() returns them."""
    out = []
    for t in truths:
        p, m = t["pos"], t["mass"]
        ones = torch.ones(p.shape[0], device=p.device)
        rho = plan.deposit(p, m, ones)
        F4 = plan.poisson(rho)
        tpos = p[t["idx"]].contiguous()
        pm, _ = plan.gather(F4, tpos)
        out.append({"kind": t["kind"], "seed": t["seed"], "x": net.input(rho, F4), "tpos": tpos, "pm": pm,
                    "truth": t["truth64"].float(), "label": (t["truth64"] - pm.double()).float()})
    return out


def make_dataset(plan, net, n, count, seed0, kinds=scenes.SCENES, n_targets=8192, eps=1.0 / 256, log=None):
    out = []
    t0 = time.time()
    for i in range(count):
        out.append(make_snapshot(plan, net, kinds[i % len(kinds)], n, seed0 + i, n_targets, eps))
        if log and (i + 1) % max(1, count // 10) == 0:
            log(f"snapshots {i + 1}/{count} ({time.time() - t0:.1f} s)")
    return out


# ---------------------------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------------------------
def _predict(plan: PMPlan, field: torch.Tensor, B: int, snaps) -> list:
    G = plan.grid
    f = field.view(B, G, G, G, 4)
    return [plan.gather(f[b], s["tpos"])[0] for b, s in enumerate(snaps)]


def save_checkpoint(path: str, state: dict) -> None:
    """Writes state with torch.save to path + '.tmp' and renames it over path, so a reader (or a
    resumed run) sees the previous checkpoint or the new one, never a partial file
    (save_atomic, scripts/train_scatter_field.py:132-134)."""
    tmp = str(path) + ".tmp"
    torch.save(state, tmp)
    os.replace(tmp, path)


def load_checkpoint(path: str):
    """The state save_checkpoint wrote, or None when there is none."""
    if not path or not os.path.exists(path):
        return None
    return torch.load(path, map_location="cpu", weights_only=False)


class _StopFlag:
    """Set by SIGTERM while installed (main thread only): the loop saves and returns."""

    def __init__(self):
        self.set = False
        self._prev = None

    def __enter__(self):
        if threading.current_thread() is threading.main_thread():
            self._prev = signal.signal(signal.SIGTERM, self._handler)
        return self

    def _handler(self, signum, frame):
        self.set = True

    def __exit__(self, *exc):
        if self._prev is not None:
            signal.signal(signal.SIGTERM, self._prev)
        return False


def train(net: GridCNN, plan: PMPlan, data: list, steps: int, batch: int = 4, lr: float = 3e-4,
          weight_decay: float = 0.01, seed: int = 4738, log=None, log_every: int = 100, clip: float = 1.0,
          warmup: int = 50, checkpoint: str | None = None, checkpoint_every: int = 1000) -> list:
    """AdamW on loss = mean over the batch's snapshots of sum |pred - label|^2 / sum |label|^2, with
    linear warm-up then cosine decay of the learning rate, gradient-norm clipping and skipping
    of non-finite steps (scripts/train_scatter_field.py:190, :228-235).

    checkpoint: a path; every checkpoint_every steps, at the end, and on SIGTERM the parameters,
    AdamW moments, step counter, batch sampler state and loss history are written there atomically,
    and a run that finds the file resumes from it (scripts/train_scatter_field.py:132-134,
    :165-168). On SIGTERM the function returns after saving, with hist[-1]["stopped"] set."""
    G = plan.grid
    rng = np.random.default_rng(seed)
    hist = []
    field = torch.zeros(batch * G ** 3 * 4, device=plan.device)
    dfield = torch.zeros_like(field)
    t0 = time.time()
    window, skipped = [], 0
    start = 1
    ck = load_checkpoint(checkpoint) if checkpoint else None
    if ck is not None:
        net.load_state_dict(ck["net"])
        rng.bit_generator.state = ck["rng"]
        hist, skipped, start = list(ck["hist"]), int(ck["skipped"]), int(ck["it"]) + 1
        if log:
            log(f"resumed from {checkpoint} at step {start - 1}")

    def state(it):
        return {"net": net.state_dict(), "rng": rng.bit_generator.state, "hist": hist, "skipped": skipped, "it": it,
                "steps": steps}

    with _StopFlag() as stop:
        for it in range(start, steps + 1):
            loss, gn = _train_step(net, plan, data, batch, G, rng, field, dfield, clip)
            if loss is None:  # non-finite loss or gradient: no update
                skipped += 1
            else:
                sched = min(1.0, it / max(1, warmup)) * (0.55 + 0.45 * math.cos(math.pi * it / steps))
                net.adamw(lr=lr * sched, weight_decay=weight_decay)
                window.append(loss)
            if it % log_every == 0 or it == steps:
                net.check()
                hist.append({"step": it, "loss": float(np.mean(window)) if window else float("nan"),
                             "grad_norm": gn, "skipped": skipped, "s": time.time() - t0})
                window = []
                if log:
                    log(f"step {it} loss {hist[-1]['loss']:.4f} |g| {gn:.3g} ({time.time() - t0:.1f} s)")
            if checkpoint and (it % checkpoint_every == 0 or it == steps or stop.set):
                save_checkpoint(checkpoint, state(it))
            if stop.set:
                hist.append({"step": it, "stopped": True, "s": time.time() - t0})
                if log:
                    log(f"SIGTERM: saved at step {it}")
                return hist
    return hist


def _train_step(net, plan, data, batch, G, rng, field, dfield, clip):
    """Forward, loss and backward of one batch with gradient-norm clipping; returns (loss, |g|), or
    (None, |g|) when the loss or the gradient is not finite (the caller then skips the update)."""
    pick = rng.choice(len(data), size=batch, replace=len(data) < batch)
    snaps = [data[i] for i in pick]
    x = torch.cat([s["x"] for s in snaps])
    field.zero_()
    net.forward(x, batch, G, field, train=True)
    preds = _predict(plan, field, batch, snaps)
    loss = 0.0
    dfield.zero_()
    d4 = dfield.view(batch, G ** 3 * 4)
    for b, (s, pr) in enumerate(zip(snaps, preds)):
        # each snapshot normalised by its own residual energy, so that scenes with small
        # forces (a uniform box) weigh as much as concentrated ones
        den = batch * max(float((s["label"] ** 2).sum()), 1e-30)
        diff = pr - s["label"]
        loss += float((diff ** 2).sum()) / den
        g = (2.0 / den) * diff
        net._call("augur_cnn_gather_transpose", s["tpos"].data_ptr(), g.contiguous().data_ptr(),
                  s["tpos"].shape[0], G, plan.extent, d4[b].data_ptr())
    net.backward(dfield, batch, G)
    gn = net.clip_grad_norm(clip)
    if not (math.isfinite(loss) and math.isfinite(gn)):
        return None, gn
    return loss, gn


# ---------------------------------------------------------------------------------------------
# evaluation
# ---------------------------------------------------------------------------------------------
def errors(a: torch.Tensor, truth: torch.Tensor) -> dict:
    d = (a.double() - truth.double()).norm(dim=1)
    rms = truth.double().norm(dim=1).pow(2).mean().sqrt()
    e = (d / rms).cpu().numpy()
    return {"rel_rms": float(d.pow(2).mean().sqrt() / rms), "median_norm_by_rms": float(np.sort(e)[(len(e) - 1) // 2]),
            "p90_norm_by_rms": float(np.quantile(e, 0.9))}


def evaluate(net: GridCNN, plan: PMPlan, data: list) -> dict:
    """Force error vs the FP64 direct sum with and without the learned correction: per scene
    kind (bodies of all that kind's snapshots pooled) and over all kinds (mean of the kinds)."""
    G = plan.grid
    field = torch.zeros(G ** 3 * 4, device=plan.device)
    pooled: dict = {}
    for s in data:
        field.zero_()
        net.forward(s["x"], 1, G, field)
        corr = plan.gather(field.view(G, G, G, 4), s["tpos"])[0]
        d = pooled.setdefault(s["kind"], {"pm": [], "cnn": [], "truth": []})
        d["pm"].append(s["pm"])
        d["cnn"].append(s["pm"] + corr)
        d["truth"].append(s["truth"])
    out = {"by_kind": {}}
    for kind, d in pooled.items():
        t = torch.cat(d["truth"])
        out["by_kind"][kind] = {"plain_pm": errors(torch.cat(d["pm"]), t), "cnn": errors(torch.cat(d["cnn"]), t)}
    for form in ("plain_pm", "cnn"):
        rows = [v[form] for v in out["by_kind"].values()]
        out[form] = {m: float(np.mean([r[m] for r in rows])) for m in rows[0]}
    return out


# ---------------------------------------------------------------------------------------------
# fallback and the corrected leapfrog
# ---------------------------------------------------------------------------------------------
class FallbackMonitor:
    """Reverts to plain PM when |E - E0| / |E0| > drift_max or when the rms predicted correction
    exceeds corr_max times the rms PM force. Once reverted, the scene stays on plain PM."""

    def __init__(self, drift_max: float = 0.05, corr_max: float = 0.5):
        self.drift_max, self.corr_max = drift_max, corr_max
        self.e0 = None
        self.reverted = False
        self.reason = None
        self.history = []

    def observe(self, energy: float | None = None, corr_ratio: float | None = None) -> bool:
        """Record one check; returns True while the learned correction stays enabled."""
        if self.reverted:
            return False
        if energy is not None:
            if self.e0 is None:
                self.e0 = energy
            drift = abs(energy - self.e0) / max(abs(self.e0), 1e-300)
            self.history.append(("drift", drift))
            if not math.isfinite(energy) or drift > self.drift_max:
                self.reverted, self.reason = True, f"energy drift {drift:.3g} > {self.drift_max}"
        if corr_ratio is not None:
            self.history.append(("corr", corr_ratio))
            if not math.isfinite(corr_ratio) or corr_ratio > self.corr_max:
                self.reverted, self.reason = True, f"correction/force {corr_ratio:.3g} > {self.corr_max}"
        return not self.reverted


class CorrectedPM:
    """Leapfrog of one scene on the PM run loop with the CNN correction added to the force grid
    between the Poisson solve and the gather. check_every: steps between monitor checks (the
    check step also solves for the potential lane for the energy)."""

    def __init__(self, plan: PMPlan, net: GridCNN | None, monitor: FallbackMonitor | None = None,
                 check_every: int = 10):
        self.plan, self.net = plan, net
        self.monitor = monitor or FallbackMonitor()
        self.check_every = check_every
        G = plan.grid
        self.rho = torch.empty((G,) * 3, device=plan.device)
        # (kinetic, potential, sum |correction|^2, sum |PM force|^2): read back together, once per check
        self.energy = torch.zeros(4, dtype=torch.float64, device=plan.device)
        self.nstep = 0
        self.last_energy = None
        self._stats_due = False

    def _grid(self, check: bool):
        use = self.net is not None and not self.monitor.reverted
        F4 = self.plan.run_grid(self.rho if use else None, with_phi=use or check)
        if use:
            stats = None
            if check:
                stats = self.energy[2:]
                stats.zero_()
                self._stats_due = True
            x = self.net.input(self.rho, F4)
            self.net.forward(x, 1, self.plan.grid, F4.view(-1), stats=stats)
        return F4

    def begin(self, pos, vel, mass=None, mask=None, dt: float = 5e-4):
        self.dt = dt
        self.plan.run_load(pos, vel, mass, mask, dt=dt)
        self._grid(True)
        self.plan.run_kick(0.5 * dt, True, energy_out=self.energy[:2], esync=0.0)
        self._record()

    def steps(self, k: int):
        for _ in range(k):
            self.nstep += 1
            check = self.check_every > 0 and self.nstep % self.check_every == 0
            self._grid(check)
            if check:
                self.plan.run_kick(self.dt, True, energy_out=self.energy[:2], esync=0.5 * self.dt)
                self._record()
            else:
                self.plan.run_kick(self.dt, True)

    def end(self, pos, vel):
        self._grid(True)
        self.plan.run_kick(0.5 * self.dt, False, energy_out=self.energy[:2], esync=0.5 * self.dt)
        self._record()
        self.plan.run_unload(pos, vel)

    def _record(self):
        """One host read per check: the energy taps and, when the network ran, the correction
        and PM-force norms accumulated by its output layer."""
        ke, pe, c2, f2 = self.energy.tolist()
        self.last_energy = ke + pe
        corr = None
        if self._stats_due:
            corr = math.sqrt(c2 / max(f2, 1e-300))
            self._stats_due = False
        self.monitor.observe(energy=self.last_energy, corr_ratio=corr)
