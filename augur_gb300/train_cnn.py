"""Train the scatter-field CNN on (FP64 direct sum - PM) force residuals and evaluate it.

    python -m augur_gb300.train_cnn --bodies 1000000 --grids 64,96,128 --snapshots 2000 \
        --targets 8192 --steps 20000 --out-dir augur_gb300/weights --workers 12

One set of seeded snapshots (their FP64 periodic direct-sum forces at the sampled targets) serves
every grid; each grid then gets its PM forces, CNN inputs and labels, and its own network, trained
with AdamW and evaluated on held-out snapshots. Training snapshots use seeds 4738 + i over the five
scene types; held-out evaluation uses seeds 9100 + i, 9200 + i and 9300 + i. Writes, per grid,
scatter_cnn_g<G>.pt (weights with their input/output scales) and scatter_cnn_g<G>.json (the
configuration, the loss curve and the held-out errors with and without the CNN). With
--checkpoint-dir, training saves every --checkpoint-every steps and on SIGTERM, and a rerun with
the same arguments resumes each grid where it stopped.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import torch

from .cnn import GridCNN
from .learned import evaluate, label_snapshots, make_truth, train
from .pm import PMPlan


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--bodies", type=int, default=1_000_000)
    ap.add_argument("--grids", default="128", help="comma-separated grid sizes, e.g. 64,96,128")
    ap.add_argument("--snapshots", type=int, default=2000)
    ap.add_argument("--eval-snapshots", type=int, default=15)
    ap.add_argument("--targets", type=int, default=8192)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--eps", type=float, default=1.0 / 256)
    ap.add_argument("--workers", type=int, default=0, help="host processes sampling the scenes")
    ap.add_argument("--out-dir", default="")
    ap.add_argument("--checkpoint-dir", default="")
    ap.add_argument("--checkpoint-every", type=int, default=1000)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.time()
    log = lambda m: print(f"[{time.time() - t0:7.1f}s] {m}", flush=True)  # noqa: E731
    grids = [int(g) for g in a.grids.split(",") if g]
    truth = make_truth(a.bodies, a.snapshots, 4738, dev, n_targets=a.targets, eps=a.eps, workers=a.workers, log=log)
    held_truth = []
    for s0 in (9100, 9200, 9300):
        held_truth += make_truth(a.bodies, a.eval_snapshots // 3, s0, dev, n_targets=a.targets, eps=a.eps,
                                 workers=a.workers)
    t_truth = time.time() - t0
    log(f"truth ready: {len(truth)} training and {len(held_truth)} held-out snapshots")
    records = {}
    for G in grids:
        tg = time.time()
        plan = PMPlan(3, G, a.bodies, "periodic", 1.0, device=dev)
        net = GridCNN(dev, seed=4738, rho_scale=1.0, phi_scale=0.1, out_scale=1.0)
        data = label_snapshots(plan, net, truth)
        held = label_snapshots(plan, net, held_truth)
        lab = torch.cat([d["label"] for d in data])
        net.out_scale = float(lab.pow(2).sum(1).mean().sqrt())
        log(f"grid {G}: labels ready; label rms {net.out_scale:.4g}")
        before = evaluate(net, plan, held)
        ck = str(Path(a.checkpoint_dir) / f"train_g{G}.ckpt") if a.checkpoint_dir else None
        if ck:
            Path(a.checkpoint_dir).mkdir(parents=True, exist_ok=True)
        hist = train(net, plan, data, a.steps, batch=a.batch, lr=a.lr, log=log, log_every=500, checkpoint=ck,
                     checkpoint_every=a.checkpoint_every)
        if hist and hist[-1].get("stopped"):
            log(f"grid {G}: stopped by SIGTERM; rerun to resume")
            return records
        after = evaluate(net, plan, held)
        cfg = {k: v for k, v in vars(a).items() if k not in ("out_dir", "checkpoint_dir")}
        cfg["grid"] = G
        rec = {"config": cfg, "out_scale": net.out_scale, "loss": hist, "held_out_before": before,
               "held_out_after": after, "truth_seconds_all_grids": t_truth, "grid_seconds": time.time() - tg}
        log(f"grid {G}: " + json.dumps({"plain_pm": after["plain_pm"], "cnn": after["cnn"]}))
        if a.out_dir:
            out = Path(a.out_dir)
            out.mkdir(parents=True, exist_ok=True)
            torch.save({"net": net.state_dict(), "grid": G, "bodies": a.bodies, "eps": a.eps},
                       out / f"scatter_cnn_g{G}.pt")
            (out / f"scatter_cnn_g{G}.json").write_text(json.dumps(rec, indent=1))
        records[G] = rec
        del data, held, net, plan
        torch.cuda.empty_cache()
    return records


if __name__ == "__main__":
    main()
