"""Train the scatter-field CNN on (FP64 direct sum - PM) force residuals and evaluate it.

    python -m augur_gb300.train_cnn --bodies 1000000 --grid 128 --snapshots 200 --steps 2000 \
        --out augur_gb300/weights/scatter_cnn_g128.pt --log run.json

Training snapshots use seeds 4738 + i over the five scene types; held-out evaluation uses
seeds 9100 + i, 9200 + i and 9300 + i. Writes the weights (with their input/output scales)
and a JSON record of the loss curve and of the held-out errors with and without the CNN.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import torch

from .cnn import GridCNN
from .learned import evaluate, make_dataset, train
from .pm import PMPlan


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--bodies", type=int, default=1_000_000)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--snapshots", type=int, default=200)
    ap.add_argument("--eval-snapshots", type=int, default=15)
    ap.add_argument("--targets", type=int, default=8192)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--eps", type=float, default=1.0 / 256)
    ap.add_argument("--out", default="")
    ap.add_argument("--log", default="")
    a = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.time()
    plan = PMPlan(3, a.grid, a.bodies, "periodic", 1.0, device=dev)
    net = GridCNN(dev, seed=4738, rho_scale=1.0, phi_scale=0.1, out_scale=1.0)
    log = lambda m: print(f"[{time.time() - t0:7.1f}s] {m}", flush=True)  # noqa: E731
    data = make_dataset(plan, net, a.bodies, a.snapshots, 4738, n_targets=a.targets, eps=a.eps, log=log)
    held = []
    for s0 in (9100, 9200, 9300):
        held += make_dataset(plan, net, a.bodies, a.eval_snapshots // 3, s0, n_targets=a.targets, eps=a.eps)
    lab = torch.cat([d["label"] for d in data])
    net.out_scale = float(lab.pow(2).sum(1).mean().sqrt())
    log(f"data ready; label rms {net.out_scale:.4g}")
    before = evaluate(net, plan, held)
    hist = train(net, plan, data, a.steps, batch=a.batch, lr=a.lr, log=log)
    after = evaluate(net, plan, held)
    rec = {"config": vars(a), "out_scale": net.out_scale, "loss": hist, "held_out_before": before,
           "held_out_after": after, "seconds": time.time() - t0}
    log(json.dumps({"plain_pm": after["plain_pm"], "cnn": after["cnn"]}))
    if a.out:
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        torch.save({"net": net.state_dict(), "grid": a.grid, "bodies": a.bodies, "eps": a.eps}, a.out)
    if a.log:
        Path(a.log).parent.mkdir(parents=True, exist_ok=True)
        Path(a.log).write_text(json.dumps(rec, indent=1))
    return rec


if __name__ == "__main__":
    main()
