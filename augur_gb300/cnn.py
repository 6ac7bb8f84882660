"""The scatter-field grid CNN on the GB300 tensor cores.

LocalNet (Faraday-dot-py/Augur, scripts/scatter_field.py:15-26) in 3D: Conv3d 3x3x3 with
zero padding, widths 2 -> 32 -> 32 -> 32 -> 32 -> 3, GELU, residual middle layers, output
layer zero-initialised (:135-136). Its input is [density, potential] cast to BF16
(ScatterField._grid_force feeds the net the scattered grid and potential, :620-657); its
3-channel output is a force-correction field added to the PM force grid before the gather.

Forward and data-gradient convolutions of the 32-channel layers run on tcgen05 (C ABI
include/augur_cnn.h); the input layer and the weight gradients run on the CUDA cores.
Parameters are one flat fp32 vector with AdamW state beside it.
"""
from __future__ import annotations

import math

import torch

from . import _lib

W = 32  # width


def _p(t):
    return None if t is None else t.data_ptr()


class GridCNN:
    # flat parameter layout: name -> (shape) in w[n][tap][c] order
    SHAPES = [("w_in", (W, 27, 2)), ("b_in", (W,))] + \
             [(f"w_mid{i}", (W, 27, W)) for i in range(3)] + [(f"b_mid{i}", (W,)) for i in range(3)] + \
             [("w_out", (3, 27, W)), ("b_out", (3,))]

    def __init__(self, device=None, seed: int = 4738, rho_scale: float = 1.0, phi_scale: float = 1.0,
                 out_scale: float = 1.0):
        self.lib = _lib.load()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.rho_scale, self.phi_scale, self.out_scale = float(rho_scale), float(phi_scale), float(out_scale)
        sizes = [math.prod(s) for _, s in self.SHAPES]
        self.n_params = sum(sizes)
        self.params = torch.zeros(self.n_params, dtype=torch.float32, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.view, self.gview, off = {}, {}, 0
        for (name, shape), sz in zip(self.SHAPES, sizes):
            self.view[name] = self.params[off:off + sz].view(shape)
            self.gview[name] = self.grads[off:off + sz].view(shape)
            off += sz
        self.reset_parameters(seed)
        bf = dict(dtype=torch.bfloat16, device=self.device)
        self.op_fwd_mid = [torch.empty(27 * W * W, **bf) for _ in range(3)]
        self.op_bwd_mid = [torch.empty(27 * W * W, **bf) for _ in range(3)]
        self.op_fwd_out = torch.empty(27 * W * 16, **bf)
        self.op_in = torch.zeros(64 * W, **bf)  # input layer: K = 27 x 2 padded to 64
        self.op_bwd_out = torch.empty(27 * 16 * W, **bf)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.adam_step = 0
        self._ws: dict = {}
        self.keep_workspaces = True  # one workspace per (batch, grid, train); False keeps only the last
        self._partial = None
        self.prepare()

    # ---- parameters ------------------------------------------------------------------------
    def reset_parameters(self, seed: int) -> None:
        """torch.nn.Conv3d's default init (uniform +-1/sqrt(fan_in)); output layer zero."""
        g = torch.Generator().manual_seed(seed)
        for name, shape in self.SHAPES:
            if name.endswith("out"):
                self.view[name].zero_()
                continue
            cin = 2 if name.endswith("_in") else W
            bound = 1.0 / math.sqrt(cin * 27)
            self.view[name].copy_((torch.rand(shape, generator=g) * 2 - 1) * bound)

    def load_torch_weights(self, convs) -> None:
        """Copy weights from torch Conv3d modules [in, mid0, mid1, mid2, out]."""
        names = ["in", "mid0", "mid1", "mid2", "out"]
        for nm, c in zip(names, convs):
            w = c.weight.detach().float()  # (n, c, 3, 3, 3)
            self.view[f"w_{nm}"].copy_(w.permute(0, 2, 3, 4, 1).reshape(w.shape[0], 27, w.shape[1]))
            self.view[f"b_{nm}"].copy_(c.bias.detach().float())
        self.prepare()

    def state_dict(self) -> dict:
        return {"params": self.params.detach().cpu().clone(), "m": self.m.cpu().clone(), "v": self.v.cpu().clone(),
                "step": self.adam_step, "scales": (self.rho_scale, self.phi_scale, self.out_scale)}

    def load_state_dict(self, d: dict) -> None:
        """Loads parameters and scales; AdamW moments when present (inference weights omit them)."""
        self.params.copy_(d["params"].to(self.device))
        if "m" in d:
            self.m.copy_(d["m"].to(self.device))
            self.v.copy_(d["v"].to(self.device))
        self.adam_step = int(d["step"])
        self.rho_scale, self.phi_scale, self.out_scale = d["scales"]
        self.prepare()

    def _call(self, name, *args):
        with torch.cuda.device(self.device):
            rc = getattr(self.lib, name)(*args, torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(rc, name)

    def prepare(self) -> None:
        """Rebuild the bf16 tensor-core operands from the fp32 master weights."""
        for i in range(3):
            w = self.view[f"w_mid{i}"]
            self._call("augur_cnn_prep_weights", w.data_ptr(), W, W, W, W, 0, self.op_fwd_mid[i].data_ptr())
            self._call("augur_cnn_prep_weights", w.data_ptr(), W, W, W, W, 1, self.op_bwd_mid[i].data_ptr())
        self._call("augur_cnn_prep_weights", self.view["w_in"].data_ptr(), W, 2, 2, W, 0, self.op_in.data_ptr())
        wo = self.view["w_out"]
        self._call("augur_cnn_prep_weights", wo.data_ptr(), 3, W, W, 16, 0, self.op_fwd_out.data_ptr())
        self._call("augur_cnn_prep_weights", wo.data_ptr(), 3, W, 16, W, 1, self.op_bwd_out.data_ptr())

    # ---- workspace ---------------------------------------------------------------------------
    def _workspace(self, B: int, G: int, train: bool) -> dict:
        key = (B, G, train)
        ws = self._ws.get(key)
        if ws is None:
            nv = B * G ** 3
            bf = dict(dtype=torch.bfloat16, device=self.device)
            if train:
                ws = {"h": [torch.empty(nv * W, **bf) for _ in range(4)]}
                ws["z"] = [torch.empty(nv * W, **bf) for _ in range(4)]
                ws["dh"] = [torch.empty(nv * W, dtype=torch.float32, device=self.device) for _ in range(2)]
                ws["dz"] = [torch.empty(nv * W, **bf) for _ in range(2)]
                ws["dout16"] = torch.empty(nv * 16, **bf)
            else:
                # inference keeps no activations for a backward pass: two buffers in turn
                a, b = (torch.empty(nv * W, **bf) for _ in range(2))
                ws = {"h": [a, b, a, b]}
            if not self.keep_workspaces:
                self._ws = {}
            self._ws[key] = ws
        return ws

    def release_workspaces(self) -> None:
        self._ws = {}

    def input(self, rho: torch.Tensor, force4: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """x (nvox, 2) bf16 = (log(1 + rho_scale * rho), phi_scale * phi) from the density grid and
        the potential lane of the PM force grid; written to out (nvox * 2 bf16) when given."""
        nv = rho.numel()
        x = torch.empty(nv * 2, dtype=torch.bfloat16, device=self.device) if out is None else out
        if x.numel() != nv * 2 or x.dtype != torch.bfloat16:
            raise ValueError("out must hold nvox * 2 bf16 values")
        self._call("augur_cnn_input", rho.data_ptr(), force4.data_ptr(), nv, self.rho_scale, self.phi_scale,
                   x.data_ptr())
        return x

    # ---- forward / backward -------------------------------------------------------------------
    def forward(self, x: torch.Tensor, B: int, G: int, field4: torch.Tensor, train: bool = False,
                stats: torch.Tensor | None = None) -> None:
        """field4 (B*G^3*4 floats) lanes 0..2 += out_scale * net(x). stats (float64 (2,), device):
        += (sum |correction|^2, sum |field4 lanes 0..2 before the correction|^2)."""
        ws = self._workspace(B, G, train)
        h, z = ws["h"], ws.get("z")
        self._call("augur_cnn_conv_in_tc", x.data_ptr(), self.op_in.data_ptr(), self.view["b_in"].data_ptr(),
                   B, G, _p(z[0]) if train else None, h[0].data_ptr(), self.err.data_ptr())
        for i in range(3):
            self._call("augur_cnn_conv_tc", 0, h[i].data_ptr(), self.op_fwd_mid[i].data_ptr(),
                       self.view[f"b_mid{i}"].data_ptr(), h[i].data_ptr(), None, h[i + 1].data_ptr(),
                       _p(z[i + 1]) if train else None, B, G, 1.0, self.err.data_ptr(), None)
        self._call("augur_cnn_conv_tc", 1, h[3].data_ptr(), self.op_fwd_out.data_ptr(),
                   self.view["b_out"].data_ptr(), None, None, field4.data_ptr(), None, B, G, self.out_scale,
                   self.err.data_ptr(), _p(stats))
        self._x = x

    def backward(self, dfield4: torch.Tensor, B: int, G: int) -> None:
        """Gradients of all parameters given dL/d(field4 lanes 0..2) (lane 3 must be zero).
        Requires the preceding forward(train=True)."""
        ws = self._workspace(B, G, True)
        h, z, dh, dz = ws["h"], ws["z"], ws["dh"], ws["dz"]
        nv = B * G ** 3
        if self._partial is None:
            self._partial = torch.empty(4 * 152 * (W * 27 * W + W), dtype=torch.float32, device=self.device)
        parts = 4 * 152
        s = self.out_scale
        # output layer: y = s (conv(h3) + b); dout16 = s dL/dy as bf16 feeds both of its gradients
        self._call("augur_cnn_pack_dout", dfield4.data_ptr(), nv, s, ws["dout16"].data_ptr())
        gw = torch.empty(4 * 27 * W + 4, dtype=torch.float32, device=self.device)
        self._call("augur_cnn_wgrad", 3, h[3].data_ptr(), ws["dout16"].data_ptr(), B, G, self._partial.data_ptr(),
                   parts, gw.data_ptr(), self.err.data_ptr())
        self.gview["w_out"].copy_(gw[:3 * 27 * W].view(3, 27, W))
        self.gview["b_out"].copy_(gw[4 * 27 * W:4 * 27 * W + 3])
        self._call("augur_cnn_conv_tc", 3, ws["dout16"].data_ptr(), self.op_bwd_out.data_ptr(), None, None,
                   z[3].data_ptr(), dh[1].data_ptr(), dz[1].data_ptr(), B, G, 1.0, self.err.data_ptr(), None)
        cur = 1
        for i in (2, 1, 0):  # middle layer i maps h[i] -> h[i+1]
            gm = torch.empty(W * 27 * W + W, dtype=torch.float32, device=self.device)
            self._call("augur_cnn_wgrad", 0, h[i].data_ptr(), dz[cur].data_ptr(), B, G, self._partial.data_ptr(),
                       parts, gm.data_ptr(), self.err.data_ptr())
            self.gview[f"w_mid{i}"].copy_(gm[:W * 27 * W].view(W, 27, W))
            self.gview[f"b_mid{i}"].copy_(gm[W * 27 * W:])
            nxt = 1 - cur
            self._call("augur_cnn_conv_tc", 2, dz[cur].data_ptr(), self.op_bwd_mid[i].data_ptr(), None,
                       dh[cur].data_ptr(), z[i].data_ptr(), dh[nxt].data_ptr(), dz[nxt].data_ptr(), B, G, 1.0,
                       self.err.data_ptr(), None)
            cur = nxt
        gi = torch.empty(W * 27 * 2 + W, dtype=torch.float32, device=self.device)
        self._call("augur_cnn_wgrad", 2, self._x.data_ptr(), dz[cur].data_ptr(), B, G, self._partial.data_ptr(),
                   parts, gi.data_ptr(), None)
        self.gview["w_in"].copy_(gi[:W * 27 * 2].view(W, 27, 2))
        self.gview["b_in"].copy_(gi[W * 27 * 2:])

    def clip_grad_norm(self, max_norm: float = 1.0) -> float:
        """Scale the gradients to norm <= max_norm (the reference clips at 1.0,
        scripts/train_scatter_field.py:228); returns the norm before clipping."""
        gn = float(self.grads.norm())
        if gn > max_norm and math.isfinite(gn):
            self.grads.mul_(max_norm / gn)
        return gn

    def adamw(self, lr: float = 3e-4, betas=(0.9, 0.999), eps: float = 1e-8, weight_decay: float = 0.01) -> None:
        self.adam_step += 1
        self._call("augur_cnn_adamw", self.params.data_ptr(), self.grads.data_ptr(), self.m.data_ptr(),
                   self.v.data_ptr(), self.n_params, lr, betas[0], betas[1], eps, weight_decay, self.adam_step)
        self.prepare()

    def check(self) -> None:
        torch.cuda.synchronize(self.device)
        e = int(self.err.item())
        if e:
            self.err.zero_()
            raise RuntimeError(f"GridCNN: a tensor-core wait ran out of its budget (error bits {e:#x})")
