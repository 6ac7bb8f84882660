"""Generates tests/golden/*.npz from the reference implementation itself.

Run where the reference (Faraday-dot-py/Augur) is checked out, with AUGUR_REF naming its root:
    AUGUR_REF=<path to the reference checkout> python tests/golden/make_golden.py
It imports the reference's own functions (ScatterField._corners / scatter / gather,
pm_baseline_force_error.sample / pm_acc, scatter_scaling_ops.exact_acc), runs them on
the CPU in float32/float64 exactly as the reference does, and stores inputs and outputs.
The published plain-PM medians are copied from the reference's
results/pm_baseline_force_error.json. Nothing at test time reads the reference.
"""
from __future__ import annotations

import json
import math
import os
import sys
from pathlib import Path

import numpy as np
import torch

if not os.environ.get("AUGUR_REF"):
    raise SystemExit("set AUGUR_REF to the root of the reference checkout (Faraday-dot-py/Augur)")
REF = Path(os.environ["AUGUR_REF"])
OUT = Path(__file__).resolve().parent
sys.dont_write_bytecode = True
sys.path.insert(0, str(REF))

from scripts import pm_baseline_force_error as pbe  # noqa: E402
from scripts import scatter_field as sf  # noqa: E402
from scripts import scatter_scaling_ops as ops  # noqa: E402


def cell_index_cases():
    rng = np.random.default_rng(4738)
    out = {}
    for G, E in ((96, 1.0), (256, 1.0), (64, 1.0), (128, 64.0)):
        D = 2 if E == 64.0 else 3
        n = 4096
        x = (rng.random((n, D)) - 0.5) * E
        # stress the rounding: points within a few ulps of cell centres and faces
        h = E / G
        k = rng.integers(0, G, size=(n // 2, D))
        near = (k + 0.5 * rng.integers(0, 2, size=(n // 2, D))) * h - E / 2
        near = near + rng.integers(-3, 4, size=near.shape) * np.spacing(np.float32(np.abs(near) + 1e-3))
        x[: n // 2] = near
        x = x.astype(np.float32)
        m = sf.ScatterField(grid=G, extent=E)
        i0, w = m._corners(torch.from_numpy(x)[None])
        out[f"G{G}_E{int(E)}_pos"] = x
        out[f"G{G}_E{int(E)}_i0"] = i0[0].numpy().astype(np.int32)
        out[f"G{G}_E{int(E)}_w"] = w[0].numpy()
    np.savez_compressed(OUT / "cell_index.npz", **out)


def scatter_gather_cases():
    torch.manual_seed(4738)
    m = sf.ScatterField(grid=32, extent=32.0)
    g = torch.Generator().manual_seed(4738)
    n = 400
    pos = ((torch.rand(1, n, 2, generator=g) - 0.5) * 36.0).float()  # some bodies off the grid
    vel = torch.randn(1, n, 2, generator=g).float()
    mass = (0.5 + torch.rand(1, n, generator=g)).float()
    mask = (torch.rand(1, n, generator=g) > 0.1).float()
    grid = m.scatter(pos, vel, mass, mask)
    field = torch.randn(1, 4, 32, 32, generator=g).float()
    gat = m.gather(field, pos)
    np.savez_compressed(OUT / "scatter_gather_2d.npz", pos=pos[0].numpy(), vel=vel[0].numpy(),
                        mass=mass[0].numpy(), mask=mask[0].numpy(), grid=grid[0].numpy(),
                        field=field[0].numpy(), gather=gat[0].numpy(), G=32, E=32.0)


def pm_acc_cases():
    """Scenes of scripts/pm_baseline_force_error.py main() with its seed and order, then the
    reference's pm_acc in float32 on the CPU (G=128, extent=64, EPS=0.5)."""
    model = sf.ScatterField(grid=128, extent=64.0, net="unet", recurrent=True, hidden_ch=0, dt=0.1, momfix=True,
                            in_scale=1.0, potential=True, kernel=True, pp=2.0, split=True, verlet=True).eval()
    rng = np.random.default_rng(4738)
    pub = json.load(open(REF / "results" / "pm_baseline_force_error.json"))
    out = {}
    keep = {("plummer", 300), ("plummer", 1000), ("two_clump", 300), ("exp_disk", 300)}
    for fam in pbe.FAMILIES:
        for n in (300, 1000, 10000, 100000):
            ns = pbe.NS[n]
            pos_np = np.stack([pbe.sample(fam, n, rng, 1.0) for _ in range(ns)])
            if (fam, n) not in keep:
                continue  # the generator stream is consumed in the reference's order regardless
            pos = torch.tensor(pos_np, dtype=torch.float32)
            vel = torch.zeros_like(pos)
            mass = torch.ones(ns, n)
            mask = torch.ones(ns, n)
            with torch.no_grad():
                acc = pbe.pm_acc(model, pos, vel, mass, mask)
            at = torch.stack([ops.exact_acc(p.double(), pbe.EPS) for p in pos])
            e, _ = pbe.errs(acc.double(), at, mask.double())
            key = f"{fam}_n{n}"
            out[key + "_pos"] = pos.numpy()
            out[key + "_acc"] = acc.numpy()
            out[key + "_median_here"] = np.float64(e.median())
            out[key + "_median_published"] = np.float64(pub[key]["plain_pm"]["norm_by_rms"]["median"])
            out[key + "_p90_published"] = np.float64(pub[key]["plain_pm"]["norm_by_rms"]["p90"])
    np.savez_compressed(OUT / "pm_acc_2d.npz", **out)


def exact_acc_cases():
    g = torch.Generator().manual_seed(9100)
    out = {}
    for D, n, eps in ((2, 300, 0.5), (3, 512, 1.0 / 64)):
        pos = (torch.randn(n, D, generator=g, dtype=torch.float64) * 0.1)
        out[f"d{D}_pos"] = pos.numpy()
        out[f"d{D}_acc"] = ops.exact_acc(pos, eps).numpy()
        out[f"d{D}_eps"] = np.float64(eps)
    np.savez_compressed(OUT / "exact_acc.npz", **out)


def kernel_acc_cases():
    """ScatterField.kernel_acc (learned radial kernel, scripts/scatter_field.py:263-289) with seeded
    kmlp weights: plain kernel with zero padding; split window with kpad = "ext"; cell-unit
    features with the prior, split and an eps feature."""
    cases = [
        dict(name="plain", grid=32, extent=64.0, cu=False, prior=False, split=False, pp=0.0, epsin=False, kpad="zero"),
        dict(name="split_ext", grid=32, extent=64.0, cu=False, prior=False, split=True, pp=3.0, epsin=False,
             kpad="ext"),
        dict(name="cu_prior", grid=64, extent=64.0, cu=True, prior=True, split=True, pp=2.0, epsin=True, kpad="ext"),
    ]
    out = {}
    for i, c in enumerate(cases):
        torch.manual_seed(4738 + i)
        m = sf.ScatterField(grid=c["grid"], extent=c["extent"], kernel=True, pp=c["pp"], split=c["split"],
                            prior=c["prior"], eps=0.5, cu=c["cu"], epsin=c["epsin"])
        m.kpad = c["kpad"]
        m.eps_cur = 0.8
        g = torch.Generator().manual_seed(9100 + i)
        with torch.no_grad():  # the output layer starts at zero: give it seeded values
            m.kmlp[-1].weight.copy_(torch.randn(m.kmlp[-1].weight.shape, generator=g) * 0.3)
            m.kmlp[-1].bias.copy_(torch.randn(1, generator=g) * 0.3)
        G = c["grid"]
        rho = (torch.rand(1, 1, G, G, generator=g) * (torch.rand(1, 1, G, G, generator=g) < 0.2)).float()
        with torch.no_grad():
            acc = m.kernel_acc(rho)
        params = torch.cat([t.detach().reshape(-1) for t in (m.kmlp[0].weight, m.kmlp[0].bias, m.kmlp[2].weight,
                                                             m.kmlp[2].bias, m.kmlp[4].weight, m.kmlp[4].bias)])
        extra = [math.log(m.eps_cur / sf.EPS0)] if c["epsin"] else []
        k = c["name"]
        out[f"{k}_params"] = params.numpy().astype(np.float32)
        out[f"{k}_extra"] = np.array(extra, np.float32)
        out[f"{k}_ncol"] = np.int32(m.kmlp[0].in_features)
        out[f"{k}_flags"] = np.int32((1 if c["cu"] else 0) | (2 if c["prior"] else 0) | (4 if c["split"] else 0) |
                                     (8 if c["kpad"] == "ext" else 0))
        out[f"{k}_split_radius"] = np.float64(m.ppe()) if c["split"] else np.float64(0.0)
        out[f"{k}_eps"] = np.float64(m.eps)
        out[f"{k}_grid"] = np.int32(G)
        out[f"{k}_extent"] = np.float64(c["extent"])
        out[f"{k}_rho"] = rho[0, 0].numpy()
        out[f"{k}_acc"] = acc[0].permute(1, 2, 0).numpy()  # (G, G, 2): (a_x, a_y)
    np.savez_compressed(OUT / "kernel_acc.npz", **out)


def pair_acc_cases():
    """ScatterField.pp_acc (pair term: k nearest neighbours, windowed learned weight and prior,
    scripts/scatter_field.py:291-300, 324-471, 500-521) with seeded ppmlp weights: dense mode
    (N <= 512), the cell-list mode (plain and cell-unit features) and the adaptive multilevel mode."""
    cases = [
        dict(name="dense", n=300, cu=False, cell=False, prior=True, epsin=False),
        dict(name="cell", n=3000, cu=False, cell=True, prior=True, epsin=False),
        dict(name="cell_cu", n=3000, cu=True, cell=True, prior=False, epsin=True),
        dict(name="adapt", n=3000, cu=False, cell=False, prior=True, epsin=False, adapt=True),
    ]
    out = {}
    for i, c in enumerate(cases):
        torch.manual_seed(4738 + i)
        m = sf.ScatterField(grid=64, extent=64.0, kernel=True, pp=2.0, split=True, prior=c["prior"], eps=0.5,
                            cu=c["cu"], epsin=c["epsin"])
        if c["cell"]:
            m.opt = {"cell"}
        if c.get("adapt"):
            m.opt = {"adapt"}  # the adaptive multilevel cell list (pp_acc_adapt, :366-471)
        m.eps_cur = 0.8
        g = torch.Generator().manual_seed(9200 + i)
        with torch.no_grad():  # the output layer starts at zero: give it seeded values
            m.ppmlp[-1].weight.copy_(torch.randn(m.ppmlp[-1].weight.shape, generator=g) * 0.3)
            m.ppmlp[-1].bias.copy_(torch.randn(1, generator=g) * 0.3)
        n = c["n"]
        # clustered bodies (many pairs inside ppe) plus a uniform background, a few off the grid
        cen = (torch.rand(8, 2, generator=g) - 0.5) * 50.0
        pos = cen[torch.randint(0, 8, (n,), generator=g)] + torch.randn(n, 2, generator=g) * 2.0
        pos[: n // 5] = (torch.rand(n // 5, 2, generator=g) - 0.5) * 66.0
        pos = pos.float()[None]
        mass = (0.5 + torch.rand(1, n, generator=g)).float()
        mask = (torch.rand(1, n, generator=g) > 0.05).float()
        with torch.no_grad():
            acc = m.pp_acc(pos, mass, mask)
        params = torch.cat([t.detach().reshape(-1) for t in (m.ppmlp[0].weight, m.ppmlp[0].bias, m.ppmlp[2].weight,
                                                             m.ppmlp[2].bias, m.ppmlp[4].weight, m.ppmlp[4].bias)])
        extra = [math.log(m.eps_cur / sf.EPS0)] if c["epsin"] else []
        k = c["name"]
        out[f"{k}_pos"] = pos[0].numpy()
        out[f"{k}_mass"] = mass[0].numpy()
        out[f"{k}_mask"] = mask[0].numpy()
        out[f"{k}_params"] = params.numpy().astype(np.float32)
        out[f"{k}_extra"] = np.array(extra, np.float32)
        out[f"{k}_ncol"] = np.int32(m.ppmlp[0].in_features)
        out[f"{k}_flags"] = np.int32((1 if c["cu"] else 0) | (2 if c["prior"] else 0))
        out[f"{k}_ppe"] = np.float64(m.ppe())
        out[f"{k}_eps"] = np.float64(m.eps)
        out[f"{k}_h"] = np.float64(m.h)
        out[f"{k}_extent"] = np.float64(64.0)
        out[f"{k}_knn"] = np.int32(16)
        out[f"{k}_acc"] = acc[0].numpy()
    np.savez_compressed(OUT / "pair_acc.npz", **out)


def field2d_cases():
    """The production 2D model of the reference's browser port (web/scatter/weights.json config:
    ScatterField(grid=128, extent=64, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
    potential=True, verlet=True), levels 5, width 32) in float64, as
    scripts/export_web_testvectors_scatter.py runs it, with seeded weights rounded to float16
    (so float32 holds them exactly; the zero-initialised output layers get seeded values):
    the U-Net alone on a seeded input, the three-channel scatter, and free Verlet rollouts of
    the exporter's scenes (30 and 100 bodies) with the recurrent potential."""
    torch.manual_seed(4738)
    m = sf.ScatterField(grid=128, extent=64.0, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
                        potential=True, verlet=True)
    g = torch.Generator().manual_seed(9300)
    with torch.no_grad():
        m.ppmlp[-1].weight.copy_(torch.randn(m.ppmlp[-1].weight.shape, generator=g) * 0.3)
        m.ppmlp[-1].bias.copy_(torch.randn(1, generator=g) * 0.3)
        m.kmlp[-1].weight.copy_(torch.randn(m.kmlp[-1].weight.shape, generator=g) * 0.3)
        m.kmlp[-1].bias.copy_(torch.randn(1, generator=g) * 0.3)
        m.net.out.weight.copy_(torch.randn(m.net.out.weight.shape, generator=g) * 1.0)
        m.net.out.bias.copy_(torch.randn(1, generator=g) * 0.05)
        for t in m.parameters():
            t.copy_(t.half().float())
    m32 = sf.ScatterField(grid=128, extent=64.0, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
                          potential=True, verlet=True).eval()  # the reference's own float32 path, same weights
    m32.load_state_dict(m.state_dict())
    m = m.double().eval()
    names = [k for k, _ in m.named_parameters()]
    out = {"names": np.array(names), "steps": np.int32(4)}
    for k, t in m.named_parameters():
        out["w_" + k] = t.detach().numpy().astype(np.float16)
    G = 128
    x = torch.randn(1, 6, G, G, generator=g, dtype=torch.float64)
    x[:, 0] = torch.rand(1, G, G, generator=g, dtype=torch.float64) * (torch.rand(1, G, G, generator=g) < 0.05)
    x = x.half().double()
    with torch.no_grad():
        out["unet_x"] = x[0].numpy().astype(np.float16)
        out["unet_y"] = m.net(x)[0].numpy().astype(np.float32)
    rng = np.random.default_rng(4738)
    for n in (30, 100):
        f, fv = (n / 8) ** 0.5, (n / 8) ** 0.25
        p0 = rng.uniform(-5.0 * f, 5.0 * f, (n, 2)).astype(np.float32)
        v0 = rng.normal(0.0, 0.5 * fv, (n, 2))
        v0 = (v0 - v0.mean(0)).astype(np.float32)
        pos, vel = torch.tensor(p0, dtype=torch.float64)[None], torch.tensor(v0, dtype=torch.float64)[None]
        mass, mask = torch.ones(1, n, dtype=torch.float64), torch.ones(1, n, dtype=torch.float64)
        k = f"n{n}"
        out[k + "_pos0"], out[k + "_vel0"] = p0, v0
        with torch.no_grad():
            out[k + "_scatter"] = m.scatter(pos, vel, mass, mask)[0].numpy().astype(np.float32)
            field = m.init_field(1, "cpu", torch.float64)
            a0, f1 = m.force(pos, vel, mass, mask, field[0])
            out[k + "_acc0"], out[k + "_field1"] = a0[0].numpy(), f1[0, 0].numpy().astype(np.float32)
            p32, v32, o32 = pos.float(), vel.float(), torch.ones(1, n)
            out[k + "_scatter32"] = m32.scatter(p32, v32, o32, o32)[0].numpy()
            out[k + "_acc0_32"] = m32.force(p32, v32, o32, o32, m32.init_field(1, "cpu")[0])[0][0].numpy()
            ps, vs = [], []
            for _ in range(4):
                pos, vel, field, _ = m.step(pos, vel, mass, mask, field)
                ps.append(pos[0].numpy())
                vs.append(vel[0].numpy())
            out[k + "_pos"], out[k + "_vel"] = np.stack(ps), np.stack(vs)
            out[k + "_field"] = field[0][0, 0].numpy().astype(np.float32)
    np.savez_compressed(OUT / "field2d.npz", **out)


def field2d_variant_cases():
    """The production 2D model's prior + cell-unit variant (ScatterField(..., prior=True, cu=True),
    the reference's ms_kp_pot_v_g128_prior / _cu family) with kpad = "ext" (the large-N driver's
    option) at grid 64 (U-Net levels 4, width 16), in float64 with seeded float16-exact weights:
    one force and two Verlet steps of 60 bodies."""
    torch.manual_seed(4739)
    m = sf.ScatterField(grid=64, extent=64.0, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
                        potential=True, verlet=True, prior=True, cu=True, width=16)
    m.kpad = "ext"
    g = torch.Generator().manual_seed(9400)
    with torch.no_grad():
        for mlp in (m.ppmlp, m.kmlp):
            mlp[-1].weight.copy_(torch.randn(mlp[-1].weight.shape, generator=g) * 0.3)
            mlp[-1].bias.copy_(torch.randn(1, generator=g) * 0.3)
        m.net.out.weight.copy_(torch.randn(m.net.out.weight.shape, generator=g) * 1.0)
        m.net.out.bias.copy_(torch.randn(1, generator=g) * 0.05)
        for t in m.parameters():
            t.copy_(t.half().float())
    m = m.double().eval()
    out = {"names": np.array([k for k, _ in m.named_parameters()]), "steps": np.int32(2),
           "levels": np.int32(m.net.levels), "width": np.int32(16), "grid": np.int32(64)}
    for k, t in m.named_parameters():
        out["w_" + k] = t.detach().numpy().astype(np.float16)
    rng = np.random.default_rng(4739)
    n = 60
    p0 = rng.uniform(-12.0, 12.0, (n, 2)).astype(np.float32)
    v0 = rng.normal(0.0, 0.5, (n, 2))
    v0 = (v0 - v0.mean(0)).astype(np.float32)
    pos, vel = torch.tensor(p0, dtype=torch.float64)[None], torch.tensor(v0, dtype=torch.float64)[None]
    mass, mask = torch.ones(1, n, dtype=torch.float64), torch.ones(1, n, dtype=torch.float64)
    out["pos0"], out["vel0"] = p0, v0
    with torch.no_grad():
        field = m.init_field(1, "cpu", torch.float64)
        a0, f1 = m.force(pos, vel, mass, mask, field[0])
        out["acc0"], out["field1"] = a0[0].numpy(), f1[0, 0].numpy().astype(np.float32)
        ps, vs = [], []
        for _ in range(2):
            pos, vel, field, _ = m.step(pos, vel, mass, mask, field)
            ps.append(pos[0].numpy())
            vs.append(vel[0].numpy())
        out["pos"], out["vel"] = np.stack(ps), np.stack(vs)
    np.savez_compressed(OUT / "field2d_variant.npz", **out)


def tick2d_cases():
    """The reference's chunked large-N tick (scripts/scatter_bh_1b.py: make_ic :66-104, Sim
    :107-146) on the CPU: the production 2D model without its pair term (ops.no_pp), relativistic
    speed (scripts/scatter_bh.py:22-23), state stored in float16 / float32, an 8000-body Gaussian
    scene in chunks of 3000; init_kick and two ticks. Weights: those of field2d.npz."""
    from types import SimpleNamespace

    from scripts import scatter_bh_1b as bh

    gw = np.load(OUT / "field2d.npz")
    m = sf.ScatterField(grid=128, extent=64.0, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
                        potential=True, verlet=True).eval()
    m.load_state_dict({k: torch.from_numpy(gw["w_" + k].astype(np.float32)) for k in gw["names"]}, strict=False)
    ops.no_pp(m)
    n, chunk, ticks = 8000, 3000, 2
    args = SimpleNamespace(sigma=8.0, vfac=0.3, c=10.0, seed=4738, ic="gaussian", ic_resample=False)
    out = {"n": np.int32(n), "c": np.float64(10.0), "dt": np.float64(0.1), "ticks": np.int32(ticks)}
    for name, pd, md in (("f16", torch.float16, torch.float16), ("f32", torch.float32, torch.float32)):
        with torch.no_grad():
            pos, mom = bh.make_ic(n, chunk, args, pd, md, 1.0, torch.device("cpu"))
            sim = bh.Sim(m, n, chunk, 10.0, 0.1, pd, md, 1.0, torch.device("cpu"))
            out[f"{name}_pos0"], out[f"{name}_mom0"] = pos.numpy().copy(), mom.numpy().copy()
            x = sim.scatter_pass(pos, mom, False)
            acc, abar = sim.grid_force(x)
            if name == "f32":
                out[f"{name}_x0"] = x[0].numpy()
            out[f"{name}_abar0"] = abar.numpy()
            sim.field = m.init_field(1, "cpu")[0]
            sim.init_kick(pos, mom)
            out[f"{name}_mom_ik"] = mom.numpy().copy()
            ps, ms_ = [], []
            for _ in range(ticks):
                sim.tick(pos, mom)
                ps.append(pos.numpy().copy())
                ms_.append(mom.numpy().copy())
            out[f"{name}_pos"], out[f"{name}_mom"] = np.stack(ps), np.stack(ms_)
            out[f"{name}_field"] = sim.field[0, 0].numpy().astype(np.float32)
    np.savez_compressed(OUT / "tick2d.npz", **out)


CASES = {"cell_index": cell_index_cases, "scatter_gather": scatter_gather_cases, "pm_acc": pm_acc_cases,
         "exact_acc": exact_acc_cases, "kernel_acc": kernel_acc_cases, "pair_acc": pair_acc_cases,
         "field2d": field2d_cases, "tick2d": tick2d_cases, "field2d_variant": field2d_variant_cases}

if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES)):
        CASES[name]()
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)
