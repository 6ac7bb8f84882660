"""Tile-shape autotuner for PM plans.

The tile shapes of a plan (augur_pm_tiles: deposit row block and chunk, z-transform tile,
C2R and y-transform row batches) change launch geometry only -- every output is
bit-identical for any valid shape -- so they are chosen by speed alone: coordinate descent
over each shape's candidates, timing a few merged steps of a real scene with CUDA events.

Results are cached per (grid, body-count bucket) in a JSON file (tiles_gb300.json beside
this module, written by ``python -m augur_gb300.autotune``); tiles_for() looks a plan up
there and the batched runner applies what it finds. The reference has no counterpart (its
kernels are cuFFT's and torch's), the closest being its DEFAULT_OPT table of fixed launch
options (scripts/scatter_field.py:1223).
"""
from __future__ import annotations

import argparse
import json
import math
import time
from pathlib import Path

import numpy as np
import torch

from . import scenes
from .pm import PMPlan

CACHE = Path(__file__).resolve().parent / "tiles_gb300.json"


def bucket(n: int) -> int:
    """Body-count bucket: the nearest power of two."""
    return 1 << max(0, int(round(math.log2(max(1, n)))))


def key(grid: int, n: int) -> str:
    return f"G{int(grid)}_n{bucket(n)}"


def candidates(grid: int) -> dict:
    """Candidate values per tile group; invalid combinations are rejected by the plan."""
    G = grid
    dep = [(ry, rz) for ry in (2, 4, 8, 16, 32) for rz in (1, 2, 3, 4, 6, 8)
           if G % ry == 0 and G % rz == 0 and ry * rz <= 64]
    base = 4096 // G
    return {
        "deposit": [{"deposit_rows_y": ry, "deposit_rows_z": rz} for ry, rz in dep],
        "deposit_chunk": [{"deposit_chunk": c} for c in (1024, 2048, 4096, 8192, 16384, 65536)],
        "deposit_aggregate": [{"deposit_aggregate": a} for a in (0, 1)],
        "green_tile_y": [{"green_tile_y": t} for t in (8, 16) if G % t == 0],
        "c2r_rows": [{"c2r_rows": r} for r in (2, 4, 8, 16, 32)],
        "fft_rows": [{"fft_rows": r} for r in sorted({max(1, min(256, base * f // 4)) for f in (1, 2, 4, 8)})],
    }


def _time_steps(plan: PMPlan, steps: int, reps: int) -> float:
    """Median device ms per merged step over reps timings of `steps` (even) steps."""
    s = torch.cuda.current_stream(plan.device)
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        plan.run_steps(steps)
        b.record(s)
        b.synchronize()
        out.append(a.elapsed_time(b) / steps)
    return float(np.median(out))


def tune_plan(plan: PMPlan, pos: torch.Tensor, vel: torch.Tensor, mass: torch.Tensor, dt: float = 5e-4,
              steps: int = 4, reps: int = 3, rounds: int = 2, log=None) -> dict:
    """Coordinate descent over candidates() on an active run of (pos, vel, mass); leaves the best
    shapes applied to plan and returns {"tiles", "ms", "default_ms", "evaluated"}."""
    plan.run_begin(pos, vel, mass, dt=dt)
    plan.run_steps(2)
    best = plan.tiles
    best_ms = default_ms = _time_steps(plan, steps, reps)
    evaluated = 1
    for _ in range(rounds):
        improved = False
        for group, opts in candidates(plan.grid).items():
            for o in opts:
                t = dict(best, **o)
                if t == best:
                    continue
                try:
                    plan.set_tiles(t)
                except RuntimeError:
                    continue
                plan.run_steps(2)
                ms = _time_steps(plan, steps, reps)
                evaluated += 1
                if ms < 0.98 * best_ms:
                    best, best_ms, improved = t, ms, True
                    if log:
                        log(f"  {group}: {o} -> {ms * 1e3:.1f} us/step")
            plan.set_tiles(best)
        if not improved:
            break
    plan.set_tiles(best)
    p2, v2 = torch.empty_like(pos), torch.empty_like(vel)
    plan.run_end(p2, v2)
    torch.cuda.synchronize(plan.device)
    return {"tiles": best, "ms": best_ms, "default_ms": default_ms, "evaluated": evaluated}


def load_cache(path: Path | str = CACHE) -> dict:
    p = Path(path)
    if not p.exists():
        return {"entries": {}}
    return json.loads(p.read_text())


_loaded: dict | None = None


def cached_tiles(grid: int, n: int) -> dict | None:
    """tiles_for() on the cache file, read once per process."""
    global _loaded
    if _loaded is None:
        _loaded = load_cache()
    return tiles_for(grid, n, _loaded)


def tiles_for(grid: int, n: int, cache: dict | None = None) -> dict | None:
    """Cached tiles for this grid and the nearest body-count bucket (None if the grid is absent)."""
    cache = load_cache() if cache is None else cache
    ent = cache.get("entries", {})
    same = [(k, v) for k, v in ent.items() if k.startswith(f"G{int(grid)}_n")]
    if not same:
        return None
    want = math.log2(bucket(n))
    k, v = min(same, key=lambda kv: abs(math.log2(int(kv[0].split("_n")[1])) - want))
    return dict(v["tiles"])


def tune(shapes, kind: str = "plummer", seed: int = 4738, dt: float = 5e-4, log=print, path: Path | str = CACHE):
    """Tune every (grid, n) in shapes on a seeded scene of `kind` and merge into the cache file."""
    cache = load_cache(path)
    cache.setdefault("entries", {})
    cache["device"] = torch.cuda.get_device_name()
    for grid, n in shapes:
        pos, vel, mass = scenes.make_scene(kind, int(n), seed=seed)
        dev = torch.device("cuda", torch.cuda.current_device())
        p, v, m = (torch.from_numpy(a).to(dev) for a in (pos, vel, mass))
        plan = PMPlan(3, int(grid), int(n), "periodic", 1.0, tiles=None)
        t0 = time.time()
        r = tune_plan(plan, p, v, m, dt=dt, log=log)
        r["scene"], r["n"], r["seconds"] = kind, int(n), round(time.time() - t0, 1)
        cache["entries"][key(grid, n)] = r
        if log:
            log(f"G={grid} n={n}: {r['default_ms'] * 1e3:.1f} -> {r['ms'] * 1e3:.1f} us/step "
                f"({r['evaluated']} shapes, {r['seconds']} s) {r['tiles']}")
        plan.close()
    Path(path).write_text(json.dumps(cache, indent=1, sort_keys=True) + "\n")
    return cache


def batch_shapes(grids=(64, 96, 128), nmin: float = 1e4, nmax: float = 1e6, cells_per_body: float = 8.0):
    """(grid, n) pairs covering the batched workload: every body-count bucket of [nmin, nmax]
    on the grid the batch rule assigns it."""
    from .batch import grid_for
    out = []
    for b in range(int(math.floor(math.log2(nmin))), int(math.ceil(math.log2(nmax))) + 1):
        n = 1 << b
        out.append((grid_for(n, grids, cells_per_body), n))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="tune PM tile shapes and write the cache file")
    ap.add_argument("--shapes", default="batch", help="'batch' or a list like 256:3000000,128:1000000")
    ap.add_argument("--out", default=str(CACHE))
    a = ap.parse_args(argv)
    if a.shapes == "batch":
        shapes = batch_shapes() + [(256, 3_000_000), (256, 1_000_000), (128, 1_000_000)]
    else:
        shapes = [tuple(int(float(x)) for x in s.split(":")) for s in a.shapes.split(",")]
    tune(shapes, path=a.out)


if __name__ == "__main__":
    main()
