"""The chunked large-N tick (Sim, scripts/scatter_bh_1b.py:107-146) on the GPU against the
reference's own Sim run on the CPU (tests/golden/tick2d.npz: an 8000-body Gaussian scene from its
make_ic, fp32 and fp16 state, init_kick then two ticks; the production 2D model's weights of
field2d.npz with the pair term removed, as the reference's driver removes it)."""
import numpy as np
import pytest
import torch

from augur_gb300 import ChunkedTick2D, UNetScatterField

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


@pytest.fixture(scope="module")
def model(golden):
    g = golden["field2d"]
    m = UNetScatterField(grid=128, extent=64.0, dt=0.1, device=DEV)
    m.load_state_dict({k: g["w_" + k].astype(np.float32) for k in g["names"]})
    return m


def _state(g, name):
    return (torch.from_numpy(g[f"{name}_pos0"]).to(DEV).contiguous(),
            torch.from_numpy(g[f"{name}_mom0"]).to(DEV).contiguous())


def test_scatter_and_mean_acceleration_match_reference(golden, model):
    g = golden["tick2d"]
    pos, mom = _state(g, "f32")
    sim = ChunkedTick2D(model, int(g["n"]), c=float(g["c"]), dt=float(g["dt"]), pos_dtype=torch.float32,
                        mom_dtype=torch.float32)
    x = sim.scatter_pass(pos, mom, False).cpu().numpy()
    for c in range(3):
        assert rel(x[c], g["f32_x0"][c]) < 1e-6, c
    _, abar = sim.grid_force()
    ref = g["f32_abar0"].astype(np.float64)
    assert np.abs(abar.cpu().numpy() - ref).max() < 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize("name,dtype,tol", (("f32", torch.float32, 5e-5), ("f16", torch.float16, 5e-4)))
def test_ticks_match_reference(golden, model, name, dtype, tol):
    g = golden["tick2d"]
    pos, mom = _state(g, name)
    sim = ChunkedTick2D(model, int(g["n"]), c=float(g["c"]), dt=float(g["dt"]), pos_dtype=dtype, mom_dtype=dtype)
    sim.init_kick(pos, mom)
    got = [("mom_ik", mom.float().cpu().numpy(), g[f"{name}_mom_ik"])]
    for t in range(int(g["ticks"])):
        sim.tick(pos, mom)
        got += [(f"pos{t}", pos.float().cpu().numpy(), g[f"{name}_pos"][t]),
                (f"mom{t}", mom.float().cpu().numpy(), g[f"{name}_mom"][t])]
    for tag, a, b in got:
        assert rel(a, b) < tol, (tag, rel(a, b))
        if dtype == torch.float16:  # stored values: mostly the same float16 as the reference's
            assert np.mean(a == b.astype(np.float32)) > 0.85, tag
            sp = np.spacing(np.abs(b).astype(np.float16)).astype(np.float64)
            assert np.mean(np.abs(a - b) <= 2 * sp) > 0.98, tag
    assert rel(sim.field[0].cpu().numpy(), g[f"{name}_field"]) < 1e-4


def test_tick_is_deterministic(golden, model):
    g = golden["tick2d"]
    out = []
    for _ in range(2):
        pos, mom = _state(g, "f16")
        sim = ChunkedTick2D(model, int(g["n"]), pos_dtype=torch.float16, mom_dtype=torch.float16)
        sim.init_kick(pos, mom)
        sim.tick(pos, mom)
        out.append((pos.clone(), mom.clone(), sim.field.clone()))
    assert all(torch.equal(a, b) for a, b in zip(out[0], out[1]))


def test_bf16_momentum_state_runs(golden, model):
    g = golden["tick2d"]
    pos = torch.from_numpy(g["f16_pos0"]).to(DEV).contiguous()
    mom = torch.from_numpy(g["f32_mom0"]).to(DEV).to(torch.bfloat16).contiguous()
    sim = ChunkedTick2D(model, int(g["n"]), pos_dtype=torch.float16, mom_dtype=torch.bfloat16)
    sim.init_kick(pos, mom)
    sim.tick(pos, mom)
    ref = g["f16_mom"][0].astype(np.float64)
    assert torch.isfinite(mom.float()).all()
    assert rel(mom.float().cpu().numpy(), ref) < 2e-2  # bf16 holds 8 bits: a few ulps from the fp16 run
