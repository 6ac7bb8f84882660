"""GPU parity of the FP64 truth: the softened direct sum (isolated and Ewald-periodic) and the
compensated energy / momentum reductions, against the reference's own exact_acc outputs and the
oracle's float64 restatements.

Bars:
  * isolated direct sum vs the reference's exact_acc (tests/golden/exact_acc.npz): 1e-12 of max|a|
    (same pair sums, different summation order);
  * periodic direct sum vs the oracle's tabulated restatement (same 65^3 Ewald table, same
    trilinear interpolation, in float64; the GPU interpolates the correction in fp32): 1e-6
    relative RMS;
  * periodic direct sum vs the exact Ewald sum (no table): 5e-6 relative RMS. The table's
    interpolation error, emulated in float64 on 2000-body scenes, is 1.5e-6 (uniform), 2e-7
    (clumpy) and 7e-9 (Plummer) relative RMS;
  * energy reductions vs float64 numpy sums: 1e-6 relative (fp32 products m*v, Kahan-compensated
    fp32 partials, FP64 folds).
"""
import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan, direct_sum_fp64, energy_fp64, scenes
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def t64(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=DEV)


@pytest.fixture(scope="module")
def ewald_tab():
    return O.ewald_table(64)


@pytest.mark.parametrize("d", [2, 3])
def test_direct_sum_matches_reference_exact_acc(golden, d):
    g = golden["exact_acc"]
    pos, ref, eps = g[f"d{d}_pos"], g[f"d{d}_acc"], float(g[f"d{d}_eps"])
    n = len(pos)
    out = direct_sum_fp64(t64(pos), t64(pos), eps=eps, target_index=torch.arange(n, device=DEV)).cpu().numpy()
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_direct_sum_masses_and_no_self_index():
    rng = np.random.default_rng(11)
    src = rng.normal(0.0, 0.1, (5000, 3))
    m = rng.uniform(0.5, 1.5, 5000)
    tg = rng.normal(0.0, 0.1, (300, 3))  # targets that are not sources
    out = direct_sum_fp64(t64(tg), t64(src), t64(m), eps=1e-3).cpu().numpy()
    ref = O.direct_sum(tg, src, 1e-3, mass=m)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def _periodic_targets(pos, k):
    """k bodies of the scene plus targets on the octant boundaries of the Ewald table and at +-box/2."""
    tg = pos[:k].astype(np.float64).copy()
    edge = np.array([[0.4999999, 0.0, 0.0], [-0.5, 0.1, 0.2], [0.0, 0.4999999, -0.4999999], [1e-7, -1e-7, 1e-7],
                     [0.25, 0.25, 0.25], [-0.5, -0.5, -0.5], [0.3, -0.49, 0.0], [0.0, 0.0, 0.0],
                     [0.125, -0.375, 0.4999], [-0.2500001, 0.2499999, 0.0]])
    tg[:len(edge)] = edge
    return tg


@pytest.mark.parametrize("kind", ["plummer", "uniform", "clumpy"])
def test_periodic_direct_sum_vs_oracle(kind, ewald_tab):
    pos, _, mass = scenes.make_scene(kind, 2048, seed=7)
    src = pos.astype(np.float64)
    m = mass.astype(np.float64)
    tg = _periodic_targets(pos, 256)
    eps = 1.0 / 256
    out = direct_sum_fp64(t64(tg), t64(src), t64(m), eps=eps, box=1.0).cpu().numpy()
    tab_ref = O.direct_sum_periodic_tabulated(tg, src, eps, 1.0, ewald_tab, mass=m)
    assert O.rel_rms(out, tab_ref) < 1e-6
    exact = O.direct_sum_periodic(tg, src, eps, 1.0, mass=m)
    assert O.rel_rms(out, exact) < 5e-6


def test_periodic_direct_sum_box_scaling_and_self_exclusion(ewald_tab):
    # a box of side 2: the correction scales as 1/box^2 on displacements / box
    pos, _, mass = scenes.make_scene("clumpy", 1024, seed=12)
    src = 2.0 * pos.astype(np.float64)
    idx = np.arange(0, 1024, 8)
    tg = src[idx]
    out = direct_sum_fp64(t64(tg), t64(src), t64(mass.astype(np.float64)), eps=0.01, box=2.0,
                          target_index=torch.as_tensor(idx, device=DEV)).cpu().numpy()
    ref = O.direct_sum_periodic_tabulated(tg, src, 0.01, 2.0, ewald_tab, mass=mass, target_index=idx)
    assert O.rel_rms(out, ref) < 1e-6


def test_energy_reductions_vs_float64():
    n = 1_000_003  # not a multiple of the block size
    pos, vel, mass = scenes.make_scene("plummer", n, seed=21)
    rng = np.random.default_rng(21)
    mask = (rng.random(n) > 0.1).astype(np.float32)
    phi = rng.normal(-1.0, 0.3, n).astype(np.float32)
    f = lambda x: torch.as_tensor(x, device=DEV)
    got = energy_fp64(f(vel), f(mass), f(mask), f(phi))
    ref = O.energy_sums(vel, mass, mask, phi)
    for k in ("ke", "mass", "pe"):
        assert abs(got[k] - ref[k]) <= 1e-6 * abs(ref[k]), k
    scale = float((np.abs(vel.astype(np.float64)) * (mass * mask)[:, None]).sum(0).max())
    assert np.abs(np.array(got["momentum"]) - np.array(ref["momentum"])).max() <= 1e-6 * scale
    # 2D and an empty input
    got2 = energy_fp64(f(vel[:777, :2].copy()), f(mass[:777]), f(mask[:777]))
    ref2 = O.energy_sums(vel[:777, :2], mass[:777], mask[:777])
    assert abs(got2["ke"] - ref2["ke"]) <= 1e-6 * ref2["ke"] and got2["pe"] == 0.0
    e = energy_fp64(torch.empty(0, 3, device=DEV), torch.empty(0, device=DEV), torch.empty(0, device=DEV))
    assert e["ke"] == 0.0 and e["mass"] == 0.0


def test_energy_tap_vs_float64():
    """The gather's energy tap (kinetic energy and PM potential energy written inside the step) against
    float64 sums of the same velocities and per-body potentials."""
    n, G = 50000, 32
    pos, vel, mass = scenes.make_scene("plummer", n, seed=8)
    plan = PMPlan(3, G, n, "periodic", 1.0, device=DEV)
    p, v, m = (torch.from_numpy(x).to(DEV) for x in (pos, vel, mass))
    ones = torch.ones(n, device=DEV)
    e = torch.zeros(2, dtype=torch.float64, device=DEV)
    plan.run_load(p, v, m, ones, dt=1e-3)
    plan.run_grid(with_phi=True)
    plan.run_kick(0.0, False, energy_out=e, esync=0.0)
    _, phi = plan.force(p, m, ones, with_phi=True)
    ref = O.energy_sums(vel, mass, np.ones(n, np.float32), phi.cpu().numpy())
    ke, pe = e.tolist()
    assert abs(ke - ref["ke"]) <= 1e-6 * abs(ref["ke"])
    assert abs(pe - ref["pe"]) <= 1e-6 * abs(ref["pe"])
    plan.close()
