"""Batched stepping of independent periodic scenes of uneven size and grid.

The reference batches scenes by padding them to one (B, Nmax, D) tensor with a mask and
one grid size (to_tensors, scripts/scatter_field.py:779-794) and removes Python launch
overhead by capturing its step in a CUDA graph (_graphed, :567-589). Here every scene
keeps its own body count and grid: one PM plan per scene, and one CUDA graph holds two
merged steps of all of them. The graph's branches (one per capture stream) are
independent, so small scenes run side by side and fill the GPU, and one replay costs one
launch. Scenes of one grid size share a batched force grid (B, G, G, G, 4) -- each plan
writes its slice -- so the learned correction of all of them is one network launch per
layer; plain PM stays the fallback: a scene whose energy drifts by more than 5% leaves
the CNN group and the graph is captured again. (The monitor here watches the energy only,
read every check_every steps from taps inside the graph; CorrectedPM's check of the
correction's size needs the grid before and after the network and is not made.)

A step swaps each plan's two body buffers, so the graph holds an even number of steps
and replays leave the plans' host state unchanged.

fused=True (plain PM only) steps all scenes with one launch per stage instead of one plan per
graph branch: augur_pm_batch_run_steps deals each stage's blocks to the scenes by a table of
block offsets, so a step is 11 launches whatever the number of scenes, bit-identical to the
per-scene steps.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib, autotune, scenes
from .learned import FallbackMonitor
from .pm import PMPlan, direct_sum_fp64


def grid_for(n: int, grids=(64, 96, 128), cells_per_body: float = 8.0) -> int:
    """Smallest grid with at least cells_per_body cells per body, else the largest."""
    for g in sorted(grids):
        if g ** 3 >= cells_per_body * n:
            return int(g)
    return int(max(grids))


def make_batch(count: int = 64, nmin: float = 1e4, nmax: float = 1e6, seed: int = 9100, grids=(64, 96, 128),
               cells_per_body: float = 8.0, kinds=scenes.SCENES) -> list:
    """Seeded uneven batch: N log-uniform in [nmin, nmax], scene kinds in turn, grid by grid_for."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(np.int64)
    out = []
    for i, n in enumerate(ns):
        kind = kinds[i % len(kinds)]
        pos, vel, mass = scenes.make_scene(kind, int(n), seed=seed + 1 + i)
        out.append({"kind": kind, "n": int(n), "seed": seed + 1 + i, "grid": grid_for(int(n), grids, cells_per_body),
                    "pos": pos, "vel": vel, "mass": mass})
    return out


class BatchedPM:
    """Leapfrog of a list of scenes (dicts with pos, vel (n, 3), mass (n,), grid) on one GPU.

    nets: {grid: GridCNN} for the CNN-corrected form (scenes whose grid has no net run plain
    PM); None for plain PM. tiles: "cache" (autotune cache), None (plan defaults) or a
    {grid: tiles dict} map. streams: capture streams (graph branches).
    """

    def __init__(self, batch: list, dt: float = 5e-4, nets: dict | None = None, streams: int = 16,
                 tiles="cache", check_every: int = 10, device=None, extent: float = 1.0, drift_max: float = 0.05,
                 fused: bool = False):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.dt, self.nets, self.check_every = float(dt), dict(nets or {}), int(check_every)
        if fused and self.nets:
            raise ValueError("fused stepping covers plain PM batches (no nets)")
        self.fused = bool(fused)
        self._batch = None
        self.scenes = []
        cache = autotune.load_cache() if tiles == "cache" else None
        for sc in batch:
            t = lambda a: (a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))) \
                .to(self.device, torch.float32).contiguous()
            pos, vel, mass = t(sc["pos"]), t(sc["vel"]), t(sc["mass"])
            n, G = pos.shape[0], int(sc["grid"])
            plan = PMPlan(3, G, n, "periodic", extent, device=self.device, tiles=None)
            tl = autotune.tiles_for(G, n, cache) if cache is not None else (tiles or {}).get(G)
            if tl:
                plan.set_tiles(tl)
            self.scenes.append({"plan": plan, "pos": pos, "vel": vel, "mass": mass,
                                "mask": torch.ones(n, device=self.device), "n": n, "grid": G,
                                "kind": sc.get("kind"), "cnn": G in self.nets, "tuned": bool(tl),
                                "monitor": FallbackMonitor(drift_max=drift_max) if G in self.nets else None})
        # longest first, dealt round-robin over the streams (balanced branches)
        cost = [s["n"] + 2 * s["grid"] ** 3 for s in self.scenes]
        self.order = sorted(range(len(self.scenes)), key=lambda i: -cost[i])
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max(1, min(streams, len(self.scenes))))]
        for j, i in enumerate(self.order):
            self.scenes[i]["stream"] = self.streams[j % len(self.streams)]
        self.energy = torch.zeros(len(self.scenes), 2, 2, dtype=torch.float64, device=self.device)
        self.graph = None
        self.nstep = 0
        self.bodies = sum(s["n"] for s in self.scenes)

    # ---- groups of CNN-corrected scenes sharing one batched grid -------------------------
    def _build_groups(self):
        self.groups = {}
        for G in sorted(self.nets):
            idx = [i for i, s in enumerate(self.scenes) if s["grid"] == G and s["cnn"]]
            if not idx:
                continue
            B = len(idx)
            grp = {"idx": idx, "B": B, "G": G, "net": self.nets[G],
                   "field": torch.zeros(B, G, G, G, 4, device=self.device),
                   "rho": torch.zeros(B, G, G, G, device=self.device),
                   "x": torch.empty(B * G ** 3 * 2, dtype=torch.bfloat16, device=self.device),
                   "stream": torch.cuda.Stream(self.device)}
            for b, i in enumerate(idx):
                self.scenes[i]["plan"].bind_force_grid(grp["field"][b])
                self.scenes[i]["group"], self.scenes[i]["slot"] = G, b
            self.groups[G] = grp
        for s in self.scenes:
            if not s["cnn"]:
                s["plan"].bind_force_grid(None)
                s.pop("group", None)

    # ---- one merged step of everything, inside the capture -------------------------------
    def _step(self, j: int):
        """Merged step j (0 or 1) of all scenes on their streams (forked from the capture stream
        beforehand); CNN scenes write energy slot j. Stream order alone chains a scene's steps."""
        for i in self.order:
            sc = self.scenes[i]
            if not sc["cnn"]:
                with torch.cuda.stream(sc["stream"]):
                    sc["plan"].run_steps(1)
        # CNN groups: every scene's grid into its slice, the net over the group, then the kicks
        for G, grp in self.groups.items():
            gs = grp["stream"]
            mine = [self.scenes[i] for i in grp["idx"]]
            sts = list({id(sc["stream"]): sc["stream"] for sc in mine}.values())
            for st in sts:  # fork the group's scene streams, all at once so their grids overlap
                st.wait_stream(gs)
            for b, sc in enumerate(mine):
                with torch.cuda.stream(sc["stream"]):
                    sc["plan"].run_grid(grp["rho"][b], with_phi=True)
            for st in sts:
                gs.wait_stream(st)
            with torch.cuda.stream(gs):
                net = grp["net"]
                net.input(grp["rho"], grp["field"], out=grp["x"])
                net.forward(grp["x"], grp["B"], G, grp["field"].view(-1))
            for st in sts:
                st.wait_stream(gs)
            for b, (sc, i) in enumerate(zip(mine, grp["idx"])):
                with torch.cuda.stream(sc["stream"]):
                    sc["plan"].run_kick(self.dt, True, energy_out=self.energy[i, j], esync=0.5 * self.dt)
            for st in sts:
                gs.wait_stream(st)

    # ---- public -------------------------------------------------------------------------
    def begin(self):
        """Load every scene, apply the opening half kick and capture the two-step graph."""
        if self.fused:
            # one launch per stage needs one z-transform tile and one deposit variant for all plans
            ty = 16 if all(s["grid"] % 16 == 0 for s in self.scenes) else 8
            for s in self.scenes:
                t = s["plan"].tiles
                if t["green_tile_y"] != ty or t["deposit_aggregate"] != 0:
                    s["plan"].set_tiles({"green_tile_y": ty, "deposit_aggregate": 0})
                s["plan"].bind_force_grid(None)
                s["plan"].run_begin(s["pos"], s["vel"], s["mass"], s["mask"], dt=self.dt)
            lib = _lib.load()
            arr = (C.c_void_p * len(self.scenes))(*[s["plan"]._p for s in self.scenes])
            h = C.c_void_p()
            with torch.cuda.device(self.device):
                rc = lib.augur_pm_batch_create(C.byref(h), arr, len(self.scenes))
            _lib.check(rc, "augur_pm_batch_create")
            self._batch = h
            self.groups = {}
            torch.cuda.synchronize(self.device)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                st = torch.cuda.current_stream(self.device).cuda_stream
                _lib.check(lib.augur_pm_batch_run_steps(self._batch, 2, st), "augur_pm_batch_run_steps")
            torch.cuda.synchronize(self.device)
            return
        self._build_groups()
        for s in self.scenes:
            if not s["cnn"]:
                s["plan"].run_begin(s["pos"], s["vel"], s["mass"], s["mask"], dt=self.dt)
        for G, grp in self.groups.items():
            for b, i in enumerate(grp["idx"]):
                s = self.scenes[i]
                s["plan"].run_load(s["pos"], s["vel"], s["mass"], s["mask"], dt=self.dt)
                s["plan"].run_grid(grp["rho"][b], with_phi=True)
            net = grp["net"]
            net.input(grp["rho"], grp["field"], out=grp["x"])
            net.forward(grp["x"], grp["B"], G, grp["field"].view(-1))
            for b, i in enumerate(grp["idx"]):
                self.scenes[i]["plan"].run_kick(0.5 * self.dt, True, energy_out=self.energy[i, 0])
        torch.cuda.synchronize(self.device)
        e0 = self.energy[:, 0].sum(-1).tolist()
        for i, s in enumerate(self.scenes):
            if s["monitor"] is not None:
                s["monitor"].observe(energy=e0[i])
        self._capture()

    def _capture(self):
        for G, grp in self.groups.items():  # workspaces exist before the capture
            grp["net"]._workspace(grp["B"], G, False)
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            main = torch.cuda.current_stream(self.device)
            branches = self.streams + [g["stream"] for g in self.groups.values()]
            for st in branches:
                st.wait_stream(main)
            self._step(0)
            self._step(1)
            for st in branches:
                main.wait_stream(st)
        torch.cuda.synchronize(self.device)

    def steps(self, k: int):
        """k (even) merged steps by graph replay; CNN scenes are checked every check_every steps."""
        if k % 2:
            raise ValueError("the graph holds two steps: k must be even")
        for _ in range(k // 2):
            self.graph.replay()
            self.nstep += 2
            if self.groups and self.check_every > 0 and self.nstep % self.check_every == 0:
                self._check()

    def _check(self):
        """Energy of every CNN scene at the last step (synchronised time); reverts to plain PM
        the scenes whose monitor trips, then captures the graph again."""
        e = self.energy[:, 1].sum(-1).tolist()
        changed = False
        for i, s in enumerate(self.scenes):
            if s["cnn"] and not s["monitor"].observe(energy=e[i]):
                s["cnn"] = False
                changed = True
        if changed:
            # the reverted scenes continue plain: their plans are mid-run (a kick done, a grid due),
            # which is the state run_steps expects
            self._build_groups()
            self._capture()

    def end(self):
        """Closing half kick; writes every scene's positions and velocities back (scene order)."""
        torch.cuda.synchronize(self.device)
        if self.fused:
            for s in self.scenes:
                s["plan"].run_end(s["pos"], s["vel"])
            self._free_batch()
            torch.cuda.synchronize(self.device)
            return [(s["pos"], s["vel"]) for s in self.scenes]
        for s in self.scenes:
            p = s["plan"]
            if s["cnn"]:
                grp = self.groups[s["grid"]]
                p.run_grid(grp["rho"][s["slot"]], with_phi=True)
            else:
                p.run_grid(None, with_phi=False)
        for G, grp in self.groups.items():
            net = grp["net"]
            net.input(grp["rho"], grp["field"], out=grp["x"])
            net.forward(grp["x"], grp["B"], G, grp["field"].view(-1))
        for s in self.scenes:
            s["plan"].run_kick(0.5 * self.dt, False)
            s["plan"].run_unload(s["pos"], s["vel"])
            s["plan"].bind_force_grid(None)
        torch.cuda.synchronize(self.device)
        return [(s["pos"], s["vel"]) for s in self.scenes]

    def _free_batch(self):
        if self._batch is not None:
            self.graph = None
            _lib.load().augur_pm_batch_destroy(self._batch)
            self._batch = None

    def close(self):
        self.graph = None
        self._free_batch()
        for s in self.scenes:
            s["plan"].close()

    # ---- accuracy --------------------------------------------------------------------------
    def force_errors(self, ntarget: int = 1024, eps: float = 1.0 / 256, seed: int = 9300) -> list:
        """Per scene: relative RMS force error vs the FP64 Ewald-periodic direct sum at ntarget
        sampled bodies of the current state, plain PM and (where the scene has a net) CNN-corrected."""
        from .learned import errors
        out = []
        for i, s in enumerate(self.scenes):
            p, pos, mass = s["plan"], s["pos"], s["mass"]
            p.bind_force_grid(None)
            rng = np.random.default_rng(seed + i)
            idx = torch.from_numpy(rng.choice(s["n"], size=min(ntarget, s["n"]), replace=False)).to(self.device)
            tpos = pos[idx].contiguous()
            rho = p.deposit(pos, mass)
            F4 = p.poisson(rho)
            pm = p.gather(F4, tpos)[0]
            src = pos.double()
            truth = direct_sum_fp64(src[idx].contiguous(), src, mass.double(), eps=eps, box=1.0,
                                    target_index=idx.contiguous())
            row = {"kind": s["kind"], "n": s["n"], "grid": s["grid"], "plain_pm": errors(pm, truth)["rel_rms"]}
            net = self.nets.get(s["grid"])
            if net is not None:
                x = net.input(rho, F4)
                net.forward(x, 1, s["grid"], F4.view(-1))
                row["cnn"] = errors(p.gather(F4, tpos)[0], truth)["rel_rms"]
                row["cnn_active"] = bool(s["cnn"])
            out.append(row)
        return out
