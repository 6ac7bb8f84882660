"""The reference's production 2D model (ScatterField with the 5-level U-Net, recurrent potential,
learned kernel, pair term, momentum fix and velocity Verlet; scripts/scatter_field.py:28-67,
221-261, 551-688) on the GPU against the reference itself run in float64
(tests/golden/field2d.npz, seeded float16-exact weights): the U-Net alone, the three-channel
scatter, one force evaluation and four Verlet steps of two scenes."""
import numpy as np
import pytest
import torch

from augur_gb300 import UNetScatterField

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


@pytest.fixture(scope="module")
def model(golden):
    g = golden["field2d"]
    m = UNetScatterField(grid=128, extent=64.0, dt=0.1, width=32, levels=5, pp=2.0, device=DEV)
    m.load_state_dict({k: g["w_" + k].astype(np.float32) for k in g["names"]})
    return m


def _scene(g, n):
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=DEV)[None]
    return t(g[f"n{n}_pos0"]), t(g[f"n{n}_vel0"]), torch.ones(1, n, device=DEV), torch.ones(1, n, device=DEV)


def test_unet_matches_reference(golden, model):
    g = golden["field2d"]
    y = model.unet(torch.from_numpy(g["unet_x"].astype(np.float32))[None].to(DEV))
    assert rel(y[0].cpu().numpy(), g["unet_y"]) < 1e-5


@pytest.mark.parametrize("n", (30, 100))
def test_scatter_matches_reference(golden, model, n):
    g = golden["field2d"]
    pos, vel, mass, mask = _scene(g, n)
    x = model.scatter(pos, vel, mass, mask)[0].cpu().numpy()
    for c in range(3):
        # the reference's own float32 scatter, and its float64 one (fp32 cell weights: ~5e-6 apart)
        assert rel(x[c], g[f"n{n}_scatter32"][c]) < 1e-6, c
        assert rel(x[c], g[f"n{n}_scatter"][c]) < 2e-5, c


@pytest.mark.parametrize("n", (30, 100))
def test_force_matches_reference(golden, model, n):
    g = golden["field2d"]
    pos, vel, mass, mask = _scene(g, n)
    f0, _ = model.init_field(1)
    acc, field = model.force(pos, vel, mass, mask, f0)
    assert rel(field[0, 0].cpu().numpy(), g[f"n{n}_field1"]) < 1e-5
    # the reference's float32 force is 0.9-2.3e-5 from its float64 one on these scenes
    assert rel(acc[0].cpu().numpy(), g[f"n{n}_acc0_32"]) < 5e-5
    assert rel(acc[0].cpu().numpy(), g[f"n{n}_acc0"]) < 1e-4
    # deterministic: the same call again is bit-identical
    acc2, field2 = model.force(pos, vel, mass, mask, f0)
    assert torch.equal(acc, acc2) and torch.equal(field, field2)


@pytest.mark.parametrize("n", (30, 100))
def test_verlet_rollout_matches_reference(golden, model, n):
    g = golden["field2d"]
    pos, vel, mass, mask = _scene(g, n)
    field = model.init_field(1)
    for t in range(int(g["steps"])):
        pos, vel, field, _ = model.step(pos, vel, mass, mask, field)
        ep = np.abs(pos[0].cpu().numpy() - g[f"n{n}_pos"][t]).max()
        ev = np.abs(vel[0].cpu().numpy() - g[f"n{n}_vel"][t]).max()
        assert ep < 1e-4 and ev < 1e-4, (t, ep, ev)
    assert rel(field[0][0, 0].cpu().numpy(), g[f"n{n}_field"]) < 1e-5


def test_batch_equals_scenes(golden, model):
    """A (2, N, 2) batch is the two scenes run one by one, bit for bit; a masked body gets 0."""
    g = golden["field2d"]
    p, v, m, k = _scene(g, 30)
    p2 = p.flip(1).contiguous() * 0.9
    pos, vel = torch.cat([p, p2]), torch.cat([v, v.flip(1)])
    mass, mask = torch.cat([m, m * 1.5]), torch.cat([k, k]).contiguous()
    mask[1, 3] = 0.0
    f0 = torch.zeros(2, 1, 128, 128, device=DEV)
    acc, field = model.force(pos, vel, mass, mask, f0)
    for b in range(2):
        a1, f1 = model.force(pos[b:b + 1].contiguous(), vel[b:b + 1].contiguous(), mass[b:b + 1].contiguous(),
                             mask[b:b + 1].contiguous(), f0[b:b + 1])
        assert torch.equal(acc[b], a1[0]) and torch.equal(field[b], f1[0])
    assert torch.all(acc[1, 3] == 0)


def test_graphed_steps_equal_eager_steps(golden):
    """graph=True (the reference's "graph" option) captures the Verlet step once per shape and
    replays it: the trajectory is the eager one bit for bit."""
    g = golden["field2d"]
    sd = {k: g["w_" + k].astype(np.float32) for k in g["names"]}
    eager = UNetScatterField(device=DEV)
    eager.load_state_dict(sd)
    graphed = UNetScatterField(device=DEV, graph=True)
    graphed.load_state_dict(sd)
    p, v, m, k = _scene(g, 30)
    pos, vel = torch.cat([p, p * 0.8]).contiguous(), torch.cat([v, -v]).contiguous()
    mass, mask = torch.cat([m, m]).contiguous(), torch.cat([k, k]).contiguous()
    s1 = (pos, vel, eager.init_field(2))
    s2 = (pos.clone(), vel.clone(), graphed.init_field(2))
    for _ in range(4):
        a = eager.step(s1[0], s1[1], mass, mask, s1[2])
        b = graphed.step(s2[0], s2[1], mass, mask, s2[2])
        s1, s2 = (a[0], a[1], a[2]), (b[0], b[1], b[2])
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
        assert torch.equal(a[2][0], b[2][0]) and torch.equal(a[2][1], b[2][1])
    assert len(graphed._graphs) == 1


def test_prior_cell_unit_variant_matches_reference(golden):
    """ScatterField(..., prior=True, cu=True), kpad "ext", at grid 64 (U-Net levels 4, width 16): one force and
    two Verlet steps against the reference in float64 (tests/golden/field2d_variant.npz)."""
    g = golden["field2d_variant"]
    m = UNetScatterField(grid=64, extent=64.0, dt=0.1, width=int(g["width"]), levels=int(g["levels"]), pp=2.0,
                         prior=True, cu=True, kpad="ext", device=DEV)
    m.load_state_dict({k: g["w_" + k].astype(np.float32) for k in g["names"]})
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=DEV)[None]
    n = len(g["pos0"])
    pos, vel, one = t(g["pos0"]), t(g["vel0"]), torch.ones(1, n, device=DEV)
    acc, field = m.force(pos, vel, one, one, torch.zeros(1, 1, 64, 64, device=DEV))
    assert rel(acc[0].cpu().numpy(), g["acc0"]) < 1e-4
    assert rel(field[0, 0].cpu().numpy(), g["field1"]) < 1e-5
    state = m.init_field(1)
    for s in range(int(g["steps"])):
        pos, vel, state, _ = m.step(pos, vel, one, one, state)
        assert np.abs(pos[0].cpu().numpy() - g["pos"][s]).max() < 1e-4
        assert np.abs(vel[0].cpu().numpy() - g["vel"][s]).max() < 1e-4
