"""GPU parity of the PM path against the oracle and the reference's golden vectors.

Bars: cell indices and the fixed-point deposit bit-exact; the fp32 gather bit-exact given
the same force grid; grid forces and body forces within 1e-5 relative RMS of the oracle."""
import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan, ScatterField, pm_acc, scenes
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
TOL = 1e-5  # relative RMS, fp32 forces vs the float64 oracle


def t(x, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=DEV)


# ---------------------------------------------------------------------------------------
# K1 cell index
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("tag", ["G96_E1", "G256_E1", "G64_E1", "G128_E64"])
def test_cell_index_bit_exact_vs_reference(golden, tag):
    g = golden["cell_index"]
    pos, i0, w = g[tag + "_pos"], g[tag + "_i0"], g[tag + "_w"]
    G = int(tag.split("_")[0][1:])
    E = float(tag.split("_")[1][1:])
    D = pos.shape[1]
    plan = PMPlan(D, G, len(pos), "periodic" if D == 3 else "isolated", E)
    gi, gw = plan.cell_index(t(pos))
    assert np.array_equal(gi.cpu().numpy(), i0)
    assert np.array_equal(gw.cpu().numpy().view(np.uint32), w.view(np.uint32))


# ---------------------------------------------------------------------------------------
# K2 deposit
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("kind,n,G", [("plummer", 20000, 32), ("uniform", 30000, 64), ("clumpy", 20000, 48),
                                      ("disk", 10000, 96)])
def test_deposit_periodic_bit_exact_vs_oracle(kind, n, G):
    pos, _, mass = scenes.make_scene(kind, n, seed=9100)
    rng = np.random.default_rng(0)
    mask = (rng.random(n) > 0.05).astype(np.float32)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    rho = plan.deposit(t(pos), t(mass), t(mask)).cpu().numpy()
    ref = O.deposit_fixed(pos, mass, mask, G, 1.0, True)
    assert np.array_equal(rho.view(np.uint32), ref.view(np.uint32))
    r64 = O.deposit_ref(pos, mass, mask, G, 1.0, True)
    assert np.abs(rho - r64).max() <= 2e-6 * np.abs(r64).max()


def test_deposit_isolated_2d_matches_reference_scatter(golden):
    g = golden["scatter_gather_2d"]
    G, E = int(g["G"]), float(g["E"])
    plan = PMPlan(2, G, len(g["pos"]), "isolated", E)
    rho = plan.deposit(t(g["pos"]), t(g["mass"]), t(g["mask"])).cpu().numpy()
    ref = O.deposit_fixed(g["pos"], g["mass"], g["mask"], G, E, False)
    assert np.array_equal(rho.view(np.uint32), ref.view(np.uint32))
    assert np.abs(rho - g["grid"][0]).max() <= 2e-6 * np.abs(g["grid"][0]).max()


def test_deposit_deterministic_under_shuffle_and_repeat():
    n, G = 200000, 64
    pos, _, mass = scenes.make_scene("plummer", n, seed=9200)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    ones = torch.ones(n, device=DEV)
    a = plan.deposit(t(pos), t(mass), ones)
    b = plan.deposit(t(pos), t(mass), ones)
    perm = np.random.default_rng(3).permutation(n)
    c = plan.deposit(t(pos[perm]), t(mass[perm]), ones)
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    assert torch.equal(a.view(torch.int32), c.view(torch.int32))


def test_deposit_edge_cases():
    G = 32
    plan = PMPlan(3, G, 5000, "periodic", 1.0)
    # empty input
    rho = plan.deposit(torch.empty((0, 3), device=DEV), torch.empty(0, device=DEV), torch.empty(0, device=DEV))
    assert float(rho.abs().sum()) == 0.0
    # every body in one cell (a heavy cell), on the box faces, and at exactly -E/2
    pos = np.zeros((5000, 3), np.float32)
    pos[:2000] = 0.013
    pos[2000:3000] = -0.5
    pos[3000:4000] = np.float32(0.5) - np.spacing(np.float32(0.5))
    pos[4000:] = np.random.default_rng(1).random((1000, 3)) - 0.5
    mass = np.random.default_rng(2).random(5000).astype(np.float32)
    mask = np.ones(5000, np.float32)
    rho = plan.deposit(t(pos), t(mass), t(mask)).cpu().numpy()
    ref = O.deposit_fixed(pos, mass, mask, G, 1.0, True)
    assert np.array_equal(rho.view(np.uint32), ref.view(np.uint32))
    assert abs(rho.sum() / G ** 3 - mass.sum()) < 1e-5 * mass.sum()


def test_nonfinite_positions_are_reported():
    plan = PMPlan(3, 32, 100, "periodic", 1.0)
    pos = np.zeros((100, 3), np.float32)
    pos[7, 1] = np.nan
    plan.deposit(t(pos), torch.ones(100, device=DEV), torch.ones(100, device=DEV))
    with pytest.raises(RuntimeError, match="non-finite"):
        plan.check()
    plan.check()  # the error word was cleared


# ---------------------------------------------------------------------------------------
# K3 FFT Poisson + gradient
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("G", [32, 64, 96, 128, 256])
def test_poisson_periodic_vs_oracle(G):
    pos, _, mass = scenes.make_scene("clumpy", 50000, seed=9300)
    rho = O.deposit_fixed(pos, mass, np.ones(len(pos)), G, 1.0, True)
    plan = PMPlan(3, G, 16, "periodic", 1.0)
    F = plan.poisson(t(rho)).cpu().numpy()
    ref = O.poisson_periodic(rho, 1.0)
    for c in range(4):
        assert O.rel_rms(F[..., c], ref[..., c]) < TOL, c


def test_poisson_single_mode_analytic():
    G = 64
    x = (np.arange(G) + 0.5) / G - 0.5
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    k = 2 * np.pi * 5
    rho = (1.0 + 0.5 * np.cos(k * y)).astype(np.float32)
    plan = PMPlan(3, G, 16, "periodic", 1.0)
    F = plan.poisson(t(rho)).cpu().numpy()
    ay = -4 * np.pi * 0.5 * np.sin(k * y) / k
    assert np.abs(F[..., 1] - ay).max() < 1e-5 * np.abs(ay).max()
    assert np.abs(F[..., 0]).max() < 1e-5 * np.abs(ay).max()


# ---------------------------------------------------------------------------------------
# K4 gather
# ---------------------------------------------------------------------------------------
def test_gather_bit_exact_periodic():
    G, n = 48, 30000
    rng = np.random.default_rng(5)
    F4 = rng.normal(size=(G, G, G, 4)).astype(np.float32)
    pos, _, _ = scenes.make_scene("uniform", n, seed=1)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    acc, phi = plan.gather(t(F4), t(pos))
    a, ph = O.gather_f32(F4, pos, G, 1.0, True)
    assert np.array_equal(acc.cpu().numpy(), a) and np.array_equal(phi.cpu().numpy(), ph)


def test_gather_2d_bit_exact_vs_reference(golden):
    g = golden["scatter_gather_2d"]
    G, E = int(g["G"]), float(g["E"])
    model = ScatterField(grid=G, extent=E, dim=2, mode="isolated")
    out = model.gather(t(g["field"][None]), t(g["pos"][None]))[0].cpu().numpy()
    assert np.array_equal(out[:, :3], g["gather"][:, :3])


# ---------------------------------------------------------------------------------------
# whole force: 3D periodic and the reference's 2D isolated pm_acc
# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("kind", scenes.SCENES)
def test_pm_force_periodic_vs_oracle(kind):
    n, G = 32768, 64
    pos, _, mass = scenes.make_scene(kind, n, seed=4738)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    acc, phi = plan.force(t(pos), t(mass), torch.ones(n, device=DEV), with_phi=True)
    plan.check()
    ra, rp = O.pm_force_periodic(pos, mass, np.ones(n), G)
    assert O.rel_rms(acc.cpu().numpy(), ra) < TOL
    assert O.rel_rms(phi.cpu().numpy(), rp) < TOL


@pytest.mark.parametrize("key", ["plummer_n300", "plummer_n1000", "two_clump_n300", "exp_disk_n300"])
def test_pm_acc_isolated_matches_reference(golden, key):
    g = golden["pm_acc_2d"]
    pos, ref = g[key + "_pos"], g[key + "_acc"]
    B, n = pos.shape[:2]
    model = ScatterField(grid=128, extent=64.0, dim=2, mode="isolated", eps=0.5)
    p = t(pos)
    ones = torch.ones(B, n, device=DEV)
    acc = pm_acc(model, p, torch.zeros_like(p), ones, ones).cpu().numpy()
    for s in range(B):
        assert O.rel_rms(acc[s], ref[s]) < TOL


@pytest.mark.parametrize("key", ["plummer_n300", "two_clump_n300", "exp_disk_n300"])
def test_pm_acc_isolated_reproduces_published_medians(golden, key):
    g = golden["pm_acc_2d"]
    pos = g[key + "_pos"]
    B, n = pos.shape[:2]
    model = ScatterField(grid=128, extent=64.0, dim=2, mode="isolated", eps=0.5)
    p = t(pos)
    ones = torch.ones(B, n, device=DEV)
    acc = pm_acc(model, p, torch.zeros_like(p), ones, ones).cpu().numpy()
    es = []
    for s in range(B):
        at = O.direct_sum(pos[s].astype(np.float64), pos[s].astype(np.float64), 0.5, target_index=np.arange(n))
        es.append(O.errs(acc[s], at)[0])
    med = O.median_lower(np.concatenate(es))
    assert abs(med - float(g[key + "_median_published"])) < 2e-5


def test_masked_bodies_get_zero_force_and_deposit_nothing():
    n, G = 5000, 32
    pos, _, mass = scenes.make_scene("plummer", n, seed=1)
    mask = np.ones(n, np.float32)
    mask[::3] = 0
    plan = PMPlan(3, G, n, "periodic", 1.0)
    acc = plan.force(t(pos), t(mass), t(mask)).cpu().numpy()
    assert np.all(acc[::3] == 0)
    keep = mask > 0
    acc2 = plan.force(t(pos[keep]), t(mass[keep]), torch.ones(int(keep.sum()), device=DEV)).cpu().numpy()
    assert np.array_equal(acc[keep], acc2)


def test_periodic_force_conserves_momentum_at_scale():
    n, G = 1_000_000, 128
    pos, _, mass = scenes.make_scene("plummer", n, seed=9100)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    acc = plan.force(t(pos), t(mass), torch.ones(n, device=DEV)).double()
    m = t(mass).double()[:, None]
    p = (m * acc).sum(0)
    scale = (m * acc.abs()).sum(0)
    assert float((p.abs() / scale).max()) < 1e-5


# ---------------------------------------------------------------------------------------
# integrators
# ---------------------------------------------------------------------------------------
def test_step_matches_reference_verlet_formula():
    n, G, dt = 8192, 32, 1e-3
    pos, vel, mass = scenes.make_scene("plummer", n, seed=2)
    model = ScatterField(grid=G, extent=1.0, dim=3, mode="periodic", dt=dt)
    p, v, m = t(pos)[None], t(vel)[None], t(mass)[None]
    ones = torch.ones(1, n, device=DEV)
    st = model.init_field(1, DEV)
    p1, v1, st1, dv = model.step(p, v, m, ones, st)
    # oracle: a0 = F(x0); x1 = x0 + dt v0 + dt^2/2 a0 (wrapped); a1 = F(x1); v1 = v0 + dt/2 (a0 + a1)
    a0, _ = O.pm_force_periodic(pos, mass, np.ones(n), G)
    a0 = a0.astype(np.float32)
    x1 = O.wrap_f32(pos + np.float32(dt) * vel + np.float32(0.5 * dt * dt) * a0, 1.0)
    assert np.abs(p1[0].cpu().numpy() - x1).max() < 1e-6
    a1, _ = O.pm_force_periodic(p1[0].cpu().numpy(), mass, np.ones(n), G)
    vr = vel + np.float32(0.5 * dt) * (a0 + a1)
    assert O.rel_rms(v1[0].cpu().numpy() - vel, vr - vel) < TOL
    assert O.rel_rms(st1[1][0].cpu().numpy(), a1) < TOL


@pytest.mark.parametrize("n", [1, 100_003])
def test_step_host_equals_device_step(n):
    """augur_pm_step_host on pinned host arrays (chunked copies overlapping the kernels) gives the
    same bits as augur_pm_step on device copies, over a first step and two more; n = 1 has fewer
    bodies than copy chunks."""
    G, dt = 32, 1e-3
    pos, vel, mass = scenes.make_scene("plummer", n, seed=5)
    plan_d = PMPlan(3, G, n, "periodic", 1.0)
    plan_h = PMPlan(3, G, n, "periodic", 1.0)
    m, ones = t(mass), torch.ones(n, device=DEV)
    dp, dv, da = t(pos), t(vel), torch.zeros(n, 3, device=DEV)
    hp, hv = torch.from_numpy(pos.copy()).pin_memory(), torch.from_numpy(vel.copy()).pin_memory()
    ha = torch.zeros(n, 3).pin_memory()
    for k in range(3):
        plan_d.step(dp, dv, da, m, ones, dt=dt, have_acc=k > 0)
        plan_h.step_host(hp, hv, ha, m, ones, dt=dt, have_acc=k > 0)
        torch.cuda.synchronize()
        assert torch.equal(hp, dp.cpu()) and torch.equal(hv, dv.cpu()) and torch.equal(ha, da.cpu())
    plan_h.check()


def test_run_matches_oracle_kdk():
    n, G, dt, steps = 4096, 32, 1e-3, 5
    pos, vel, mass = scenes.make_scene("plummer", n, seed=3)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    p, v = t(pos), t(vel)
    acc = plan.run(p, v, t(mass), torch.ones(n, device=DEV), dt=dt, nsteps=steps, want_acc=True)
    plan.check()

    def force(x):
        return O.pm_force_periodic(x, mass, np.ones(n), G)[0].astype(np.float32)

    x, vv, a = O.run_kdk(pos, vel, mass, np.ones(n), G, 1.0, dt, steps, force)
    assert np.abs(p.cpu().numpy() - x).max() < 1e-5
    assert O.rel_rms(v.cpu().numpy() - vel, vv - vel) < 1e-4
    assert O.rel_rms(acc.cpu().numpy(), a) < 1e-4


def test_run_split_equals_run():
    n, G, dt = 20000, 32, 5e-4
    pos, vel, mass = scenes.make_scene("flyby", n, seed=4)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    ones = torch.ones(n, device=DEV)
    p1, v1 = t(pos), t(vel)
    plan.run(p1, v1, t(mass), ones, dt=dt, nsteps=6)
    p2, v2 = t(pos), t(vel)
    plan.run_begin(p2, v2, t(mass), ones, dt=dt)
    plan.run_steps(2)
    plan.run_steps(3)
    plan.run_end(p2, v2)
    assert torch.equal(p1, p2) and torch.equal(v1, v2)
