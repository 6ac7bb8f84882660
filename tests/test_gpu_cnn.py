"""GPU CNN kernels (tcgen05 forward and data gradient, CUDA-core input layer and weight
gradients) against a plain PyTorch fp32 CPU reference of the same network.

Tolerances: forward 5e-3 relative RMS (the reference rounds activations to BF16 at the same
points as the kernels; what remains is FP32 accumulation order); gradients 3e-2 relative RMS
and cosine > 0.999 against fp32 autograd (the kernels keep activations and dz in BF16)."""
import math

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from augur_gb300.cnn import GridCNN

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def bf(t):
    return t.to(torch.bfloat16).float()


def rel_rms(a, b):
    return float(((a - b) ** 2).sum().sqrt() / (b ** 2).sum().sqrt().clamp_min(1e-30))


def torch_weights(net: GridCNN):
    """(n, c, 3, 3, 3) torch-layout weights from the flat parameters (fp32, CPU)."""
    out = {}
    for name in ["in", "mid0", "mid1", "mid2", "out"]:
        w = net.view[f"w_{name}"].detach().cpu()
        out[name] = (w.view(w.shape[0], 3, 3, 3, w.shape[2]).permute(0, 4, 1, 2, 3).contiguous(),
                     net.view[f"b_{name}"].detach().cpu().clone())
    return out


def ref_forward(x, tw, out_scale, round_bf16=True):
    r = bf if round_bf16 else (lambda t: t)
    win = bf(tw["in"][0]) if round_bf16 else tw["in"][0]
    z0 = F.conv3d(x, win, tw["in"][1], padding=1)
    h = r(F.gelu(z0))
    for i in range(3):
        wmid = bf(tw[f"mid{i}"][0]) if round_bf16 else tw[f"mid{i}"][0]
        z = F.conv3d(h, wmid, tw[f"mid{i}"][1], padding=1)
        h = r(h + F.gelu(z))
    wout = bf(tw["out"][0]) if round_bf16 else tw["out"][0]
    return out_scale * F.conv3d(h, wout, tw["out"][1], padding=1)


def make_net(seed=1, out_nonzero=True):
    net = GridCNN(DEV, seed=seed, out_scale=0.7)
    if out_nonzero:
        g = torch.Generator().manual_seed(seed + 100)
        net.view["w_out"].copy_((torch.rand(3, 27, 32, generator=g) * 2 - 1) / math.sqrt(27 * 32))
        net.view["b_out"].copy_(torch.rand(3, generator=g) - 0.5)
        for i in range(3):
            net.view[f"b_mid{i}"].copy_((torch.rand(32, generator=g) - 0.5) * 0.2)
        net.prepare()
    return net


def inputs(B, G, seed=0):
    g = torch.Generator().manual_seed(seed)
    x = bf(torch.randn(B, 2, G, G, G, generator=g))
    xd = x.permute(0, 2, 3, 4, 1).contiguous().to(DEV).to(torch.bfloat16).view(-1)
    return x, xd


@pytest.mark.parametrize("B,G", [(1, 16), (2, 24), (1, 130)])
def test_forward_matches_torch(B, G):
    net = make_net()
    x, xd = inputs(B, G)
    field = torch.zeros(B * G ** 3 * 4, device=DEV)
    net.forward(xd, B, G, field)
    net.check()
    ours = field.view(B, G, G, G, 4)[..., :3].permute(0, 4, 1, 2, 3).cpu()
    ref = ref_forward(x, torch_weights(net), net.out_scale)
    assert rel_rms(ours, ref) < 5e-3
    assert float(field.view(-1, 4)[:, 3].abs().max()) == 0.0


def test_forward_adds_into_the_force_grid():
    net = make_net(seed=3)
    B, G = 1, 16
    x, xd = inputs(B, G, seed=5)
    base = torch.randn(B * G ** 3 * 4, device=DEV)
    field = base.clone()
    net.forward(xd, B, G, field)
    field0 = torch.zeros_like(base)
    net.forward(xd, B, G, field0)
    assert torch.allclose(field, base + field0, atol=1e-5)


def test_zero_initialised_output_layer_gives_zero_correction():
    net = GridCNN(DEV, seed=7)
    B, G = 1, 16
    _, xd = inputs(B, G)
    field = torch.zeros(B * G ** 3 * 4, device=DEV)
    net.forward(xd, B, G, field)
    assert float(field.abs().max()) == 0.0


@pytest.mark.parametrize("B,G", [(1, 16), (2, 20)])
def test_backward_matches_torch_autograd(B, G):
    net = make_net(seed=11)
    x, xd = inputs(B, G, seed=2)
    gfield = torch.randn(B, G, G, G, 3, generator=torch.Generator().manual_seed(9))
    field = torch.zeros(B * G ** 3 * 4, device=DEV)
    net.forward(xd, B, G, field, train=True)
    d4 = torch.zeros(B, G, G, G, 4)
    d4[..., :3] = gfield
    net.backward(d4.view(-1).to(DEV), B, G)
    net.check()
    # reference: fp32 autograd with the same (bf16-rounded where the kernels round) weights
    tw = torch_weights(net)
    params = {k: (v[0].clone().requires_grad_(True), v[1].clone().requires_grad_(True)) for k, v in tw.items()}
    for k in ["mid0", "mid1", "mid2", "out"]:
        params[k] = (bf(params[k][0].detach()).requires_grad_(True), params[k][1])
    y = ref_forward(x, params, net.out_scale, round_bf16=False)
    (y * gfield.permute(0, 4, 1, 2, 3)).sum().backward()
    for name in ["in", "mid0", "mid1", "mid2", "out"]:
        gw = net.gview[f"w_{name}"].detach().cpu()
        gw = gw.view(gw.shape[0], 3, 3, 3, gw.shape[2]).permute(0, 4, 1, 2, 3)
        rw = params[name][0].grad
        cos = float((gw * rw).sum() / (gw.norm() * rw.norm()))
        assert rel_rms(gw, rw) < 3e-2, name
        assert cos > 0.999, name
        gb = net.gview[f"b_{name}"].detach().cpu()
        assert rel_rms(gb, params[name][1].grad) < 3e-2, name


def test_gather_transpose_is_the_adjoint_of_the_gather():
    from augur_gb300 import PMPlan, scenes

    G, n = 16, 2000
    pos, _, _ = scenes.make_scene("uniform", n, seed=3)
    plan = PMPlan(3, G, n, "periodic", 1.0)
    p = torch.from_numpy(pos).to(DEV)
    Fg = torch.randn(G, G, G, 4, device=DEV)
    Fg[..., 3] = 0
    a, _ = plan.gather(Fg.contiguous(), p)
    v = torch.randn(n, 3, device=DEV)
    out = torch.zeros(G ** 3 * 4, device=DEV)
    net = GridCNN(DEV)
    net._call("augur_cnn_gather_transpose", p.data_ptr(), v.data_ptr(), n, G, 1.0, out.data_ptr())
    lhs = float((a.double() * v.double()).sum())
    rhs = float((Fg.view(-1).double() * out.double()).sum())
    assert abs(lhs - rhs) < 1e-4 * abs(lhs)


@pytest.mark.parametrize("B,G", [(1, 20), (2, 130)])
def test_tensor_core_input_layer_matches_cuda_core_layer(B, G):
    """The tcgen05 input layer (bf16 weights, K padded to 64) against the CUDA-core one
    (fp32 weights) and against torch with bf16-rounded weights."""
    net = make_net(seed=3)
    x, xd = inputs(B, G, seed=4)
    nv = B * G ** 3
    bf16 = dict(dtype=torch.bfloat16, device=DEV)
    z_tc, h_tc = torch.empty(nv * 32, **bf16), torch.empty(nv * 32, **bf16)
    z_cc, h_cc = torch.empty(nv * 32, **bf16), torch.empty(nv * 32, **bf16)
    net._call("augur_cnn_conv_in_tc", xd.data_ptr(), net.op_in.data_ptr(), net.view["b_in"].data_ptr(), B, G,
              z_tc.data_ptr(), h_tc.data_ptr(), net.err.data_ptr())
    net._call("augur_cnn_conv_in", xd.data_ptr(), net.view["w_in"].data_ptr(), net.view["b_in"].data_ptr(), B, G,
              z_cc.data_ptr(), h_cc.data_ptr())
    net.check()
    tw = torch_weights(net)
    ref = F.conv3d(x, bf(tw["in"][0]), tw["in"][1], padding=1).permute(0, 2, 3, 4, 1).reshape(-1)
    assert rel_rms(z_tc.float().cpu(), ref) < 5e-3
    assert rel_rms(z_tc.float(), z_cc.float()) < 1e-2
    assert rel_rms(h_tc.float(), h_cc.float()) < 1e-2
    # without z0 the layer writes h0 only
    h2 = torch.empty_like(h_tc)
    net._call("augur_cnn_conv_in_tc", xd.data_ptr(), net.op_in.data_ptr(), net.view["b_in"].data_ptr(), B, G,
              None, h2.data_ptr(), net.err.data_ptr())
    assert torch.equal(h2, h_tc)


def _wgrad(net, kind, h, dz, B, G, nout):
    parts = 4 * 152
    partial = torch.empty(parts * (nout * 27 * 32 + nout), dtype=torch.float32, device=DEV)
    out = torch.empty(nout * 27 * 32 + nout, dtype=torch.float32, device=DEV)
    net._call("augur_cnn_wgrad", kind, h.data_ptr(), dz.data_ptr(), B, G, partial.data_ptr(), parts, out.data_ptr(),
              net.err.data_ptr())
    net.check()
    return out


@pytest.mark.parametrize("B,G", [(1, 16), (2, 20), (1, 130)])
def test_wgrad_tensor_cores_match_cuda_cores_and_float64(B, G):
    """Weight and bias gradients of a 32 -> 32 layer on tcgen05 (kind 0) against the CUDA-core kernel
    (kind 4, the same fp32 sums of exact bf16 products in another order) and, at the small grid,
    against a float64 restatement dW[n][tap][c] = sum_v dz[v][n] h[v + tap][c]."""
    net = make_net(seed=21)
    g = torch.Generator().manual_seed(B * 100 + G)
    nv = B * G ** 3
    h = torch.randn(nv * 32, generator=g).to(torch.bfloat16).to(DEV)
    dz = (torch.randn(nv * 32, generator=g) * 0.1).to(torch.bfloat16).to(DEV)
    tc = _wgrad(net, 0, h, dz, B, G, 32).cpu().double()
    cc = _wgrad(net, 4, h, dz, B, G, 32).cpu().double()
    assert rel_rms(tc, cc) < 1e-4  # fp32 sums over up to 2.2M voxels in two orders
    if G <= 20:
        hh = h.cpu().double().view(B, G, G, G, 32)
        dd = dz.cpu().double().view(B, G, G, G, 32)
        hp = F.pad(hh.permute(0, 4, 1, 2, 3), (1, 1, 1, 1, 1, 1)).permute(0, 2, 3, 4, 1)
        ref = torch.empty(32, 27, 32, dtype=torch.float64)
        for tap in range(27):
            oz, oy, ox = tap // 9, (tap // 3) % 3, tap % 3
            sh = hp[:, oz:oz + G, oy:oy + G, ox:ox + G, :]
            ref[:, tap, :] = torch.einsum("bzyxn,bzyxc->nc", dd, sh)
        ref = torch.cat([ref.reshape(-1), dd.sum((0, 1, 2, 3))])
        assert rel_rms(tc, ref) < 1e-5


@pytest.mark.parametrize("B,G", [(1, 16), (1, 130)])
def test_wgrad_output_layer_tensor_cores(B, G):
    """Output-layer gradients on tcgen05 from the packed 16-channel bf16 gradient (kind 3) against the
    CUDA-core kernel on the same bf16-rounded values as an fp32 float4 grid (kind 1)."""
    net = make_net(seed=22)
    g = torch.Generator().manual_seed(G)
    nv = B * G ** 3
    h = torch.randn(nv * 32, generator=g).to(torch.bfloat16).to(DEV)
    d4 = torch.zeros(nv, 4)
    d4[:, :3] = torch.randn(nv, 3, generator=g)
    d4 = d4.to(DEV)
    d16 = torch.empty(nv * 16, dtype=torch.bfloat16, device=DEV)
    net._call("augur_cnn_pack_dout", d4.data_ptr(), nv, 1.0, d16.data_ptr())
    d4r = torch.zeros(nv, 4, device=DEV)
    d4r[:, :3] = d16.view(nv, 16)[:, :3].float()
    tc = _wgrad(net, 3, h, d16, B, G, 4).cpu().double()
    cc = _wgrad(net, 1, h, d4r, B, G, 4).cpu().double()
    assert rel_rms(tc, cc) < 1e-4  # fp32 sums over up to 2.2M voxels in two orders
    assert float(tc[3 * 27 * 32:4 * 27 * 32].abs().max()) == 0.0 and float(tc[-1]) == 0.0


def test_wait_budget_expiry_is_reported_and_recovers():
    """With a wait budget of zero every pipeline wait of the tensor-core kernels gives up at once: the
    kernels leave their loops, drain their own copies and MMAs, free TMEM and raise the timeout bit,
    which GridCNN.check() reports. The next launches with the default budget are unaffected."""
    net = make_net(seed=23)
    B, G = 1, 24
    x, xd = inputs(B, G, seed=6)
    good = torch.zeros(B * G ** 3 * 4, device=DEV)
    net.forward(xd, B, G, good)
    net.check()
    prev = net.lib.augur_cnn_set_wait_budget(0)
    try:
        field = torch.zeros_like(good)
        net.forward(xd, B, G, field)
        with pytest.raises(RuntimeError, match="ran out of its budget"):
            net.check()
    finally:
        net.lib.augur_cnn_set_wait_budget(prev)
    again = torch.zeros_like(good)
    net.forward(xd, B, G, again)
    net.check()
    assert torch.equal(again, good)
