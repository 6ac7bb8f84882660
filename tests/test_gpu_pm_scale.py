"""GPU parity of the PM path at the benchmarked sizes: 3M Plummer bodies on 256^3 (where heavy row
blocks are split into work items and the fixed-point sums need the 64-bit conversion), 1M bodies on
256^3 and 96^3 (a grid that is not a power of two), and the Poisson solve at 512^3 and 1024^3.

Bars: the deposit bit-exact against the oracle's fixed-point restatement for every tile shape; body
forces and potentials within 1e-5 relative RMS of the float64 oracle; the single-mode Poisson solve
within 1e-5 of the analytic field."""
import math

import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan, scenes
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
TOL = 1e-5


def t(x, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=DEV)


@pytest.fixture(scope="module")
def plummer3m():
    pos, vel, mass = scenes.make_scene("plummer", 3_000_000, seed=4738)
    return pos, vel, mass, O.deposit_fixed(pos, mass, np.ones(len(pos), np.float32), 256, 1.0, True)


TILES_256 = [
    None,  # the library defaults
    {"deposit_rows_y": 8, "deposit_rows_z": 2, "deposit_chunk": 1024, "green_tile_y": 8, "c2r_rows": 8,
     "fft_rows": 8, "deposit_aggregate": 1},
    {"deposit_rows_y": 32, "deposit_rows_z": 1, "deposit_chunk": 65536, "green_tile_y": 16, "c2r_rows": 16,
     "fft_rows": 16, "deposit_aggregate": 0},
]


@pytest.mark.parametrize("tiles", range(len(TILES_256)))
def test_deposit_bit_exact_3m_plummer_256(plummer3m, tiles):
    pos, _, mass, ref = plummer3m
    n = len(pos)
    plan = PMPlan(3, 256, n, "periodic", 1.0, device=DEV)
    if TILES_256[tiles] is not None:
        plan.set_tiles(TILES_256[tiles])
    rho = plan.deposit(t(pos), t(mass), torch.ones(n, device=DEV))
    plan.check()
    got = rho.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    plan.close()


def test_run_grid_density_bit_exact_3m_plummer_256(plummer3m):
    """The run loop's density (sorted state, fused x transform path) equals the oracle's deposit."""
    pos, vel, mass, ref = plummer3m
    n = len(pos)
    plan = PMPlan(3, 256, n, "periodic", 1.0, device=DEV)
    plan.run_load(t(pos), t(vel), t(mass), torch.ones(n, device=DEV), dt=5e-4)
    rho = torch.empty((256,) * 3, device=DEV)
    plan.run_grid(rho_out=rho)
    plan.check()
    assert np.array_equal(rho.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    plan.close()


@pytest.mark.parametrize("kind,n,G", [("plummer", 1_000_000, 256), ("clumpy", 1_000_000, 256),
                                      ("plummer", 1_000_000, 96), ("disk", 300_000, 96)])
def test_pm_force_periodic_at_scale_vs_oracle(kind, n, G):
    pos, _, mass = scenes.make_scene(kind, n, seed=9100)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    acc, phi = plan.force(t(pos), t(mass), torch.ones(n, device=DEV), with_phi=True)
    plan.check()
    ra, rp = O.pm_force_periodic(pos, mass, np.ones(n), G)
    assert O.rel_rms(acc.cpu().numpy(), ra) < TOL
    assert O.rel_rms(phi.cpu().numpy(), rp) < TOL
    plan.close()


@pytest.mark.parametrize("G", [512, 1024])
def test_poisson_single_mode_analytic_large(G):
    """rho = 1 + A cos(k.x) with k = 2 pi (3, 5, 7): a = -4 pi A k sin(k.x) / |k|^2, phi = -4 pi A cos(k.x) / |k|^2,
    checked slab by slab on the device."""
    A = 0.5
    m = torch.tensor([3.0, 5.0, 7.0], dtype=torch.float64, device=DEV)
    kv = 2 * math.pi * m
    k2 = float((kv * kv).sum())
    c = (torch.arange(G, dtype=torch.float64, device=DEV) + 0.5) / G - 0.5
    plan = PMPlan(3, G, 16, "periodic", 1.0, device=DEV)
    rho = torch.empty((G, G, G), dtype=torch.float32, device=DEV)
    yx = kv[1] * c[:, None] + kv[0] * c[None, :]
    for z in range(G):
        rho[z] = (1.0 + A * torch.cos(yx + kv[2] * c[z])).float()
    F = plan.poisson(rho)
    del rho
    amax = 4 * math.pi * A * float(kv.abs().max()) / k2
    pmax = 4 * math.pi * A / k2
    worst_a, worst_p = 0.0, 0.0
    for z in range(G):
        ph = yx + kv[2] * c[z]
        s, co = torch.sin(ph), torch.cos(ph)
        for comp in range(3):
            ref = -4 * math.pi * A * kv[comp] * s / k2
            worst_a = max(worst_a, float((F[z, :, :, comp].double() - ref).abs().max()))
        worst_p = max(worst_p, float((F[z, :, :, 3].double() + 4 * math.pi * A * co / k2).abs().max()))
    plan.close()
    assert worst_a < 1e-5 * amax
    assert worst_p < 1e-5 * pmax


def test_plummer_device_matches_host_sampler():
    """scenes.plummer_device (the 10^9-body generator) against scenes.plummer: radius and speed
    distributions agree within sampling error (two-sample Kolmogorov-Smirnov, 10^6 bodies each), and
    the enclosed-mass profile follows the truncated Plummer law."""
    n = 1_000_000
    host_p, host_v = scenes.plummer(n, np.random.default_rng(5))
    pos = torch.empty(n, 3, device=DEV)
    vel = torch.empty(n, 3, device=DEV)
    scenes.plummer_device(pos, vel, seed=5, chunk=1 << 18)
    dp, dv = pos.double().cpu().numpy(), vel.double().cpu().numpy()
    assert np.isfinite(dp).all() and np.isfinite(dv).all()
    assert (dp >= -0.5).all() and (dp < 0.5).all()

    def ks(a, b):
        a, b = np.sort(a), np.sort(b)
        grid = np.concatenate([a, b])
        return np.abs(np.searchsorted(a, grid, "right") / len(a) - np.searchsorted(b, grid, "right") / len(b)).max()

    r_h, r_d = np.linalg.norm(host_p, axis=1), np.linalg.norm(dp, axis=1)
    s_h, s_d = np.linalg.norm(host_v, axis=1), np.linalg.norm(dv, axis=1)
    crit = 2.0 * math.sqrt(2.0 / n)  # p ~ 1e-3 for two samples of n; deterministic seeds
    assert ks(r_h, r_d) < crit
    assert ks(s_h, s_d) < crit
    a, rmax = 0.05, 0.45
    menc = lambda r: r ** 3 / (r * r + a * a) ** 1.5
    for r in (0.02, 0.05, 0.1, 0.2, 0.4):
        frac = float((r_d < r).mean())
        assert abs(frac - menc(r) / menc(rmax)) < 4.0 * math.sqrt(0.25 / n), r
    # isotropy: mean position and mean velocity vanish within sampling error
    assert np.abs(dp.mean(0)).max() < 5.0 * r_d.std() / math.sqrt(n)
    assert np.abs(dv.mean(0)).max() < 5.0 * s_d.std() / math.sqrt(n)
