"""CPU oracle for the reference's production 2D model and its large-N tick — TEST INFRASTRUCTURE ONLY.

A float64 numpy restatement of ScatterField with net="unet", potential=True, kernel=True, pp > 0,
verlet=True (Faraday-dot-py/Augur, scripts/scatter_field.py) and of the chunked tick of
scripts/scatter_bh_1b.py, built on oracle/pm_oracle.py's kernel term and pair term. Only tests/
may import it. Parity pin: tests/golden/field2d.npz and tick2d.npz, produced by
tests/golden/make_golden.py from the reference's own ScatterField and Sim.

Weights are a dict of the reference's parameter names (ppmlp.*, kmlp.*, net.*) to arrays.
Grids are channels-first (C, G, G), x the last axis, covering [-E/2, E/2)^2.
"""
from __future__ import annotations

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover - scipy is in both images
    from math import erf as _e

    _erf = np.vectorize(_e)

from . import pm_oracle as O


def gelu(x):
    """Exact GELU, 0.5 x (1 + erf(x / sqrt 2)) (torch.nn.GELU / F.gelu default)."""
    return 0.5 * x * (1.0 + _erf(x / np.sqrt(2.0)))


# ----------------------------------------------------------------------------------
# U-Net (scripts/scatter_field.py:28-67)
# ----------------------------------------------------------------------------------
def conv3x3(x, W, b):
    """nn.Conv2d(cin, cout, 3, padding=1): x (cin, H, W), W (cout, cin, 3, 3), b (cout,)."""
    C, H, Wd = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1)))
    out = np.broadcast_to(np.asarray(b, np.float64)[:, None, None], (W.shape[0], H, Wd)).copy()
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("oc,chw->ohw", W[:, :, ky, kx], xp[:, ky:ky + H, kx:kx + Wd], optimize=True)
    return out


def _block(sd, pre, x):
    """_block (:30-31): Conv, GELU, Conv, GELU."""
    h = gelu(conv3x3(x, sd[pre + ".0.weight"], sd[pre + ".0.bias"]))
    return gelu(conv3x3(h, sd[pre + ".2.weight"], sd[pre + ".2.bias"]))


def unet(sd, x, levels: int = 5):
    """UNet.forward (:57-66) without its instrumentation hooks: x (cin, G, G) -> (cout, G, G)."""
    x = np.asarray(x, np.float64)
    h = _block(sd, "net.enc.0", gelu(conv3x3(x, sd["net.inp.weight"], sd["net.inp.bias"])))
    skips = [h]
    for lvl in range(1, levels + 1):
        C, H, W = h.shape
        h = _block(sd, f"net.enc.{lvl}", h.reshape(C, H // 2, 2, W // 2, 2).mean((2, 4)))  # avg_pool2d(2)
        skips.append(h)
    for lvl in reversed(range(levels)):
        h = np.repeat(np.repeat(h, 2, 1), 2, 2)  # interpolate(scale 2, nearest)
        h = _block(sd, f"net.dec.{lvl}", np.concatenate([h, skips[lvl]], 0))
    return conv3x3(h, sd["net.out.weight"], sd["net.out.bias"])


# ----------------------------------------------------------------------------------
# scatter / gather / gradient (:179-261, 551-555), float64
# ----------------------------------------------------------------------------------
def _corners64(pos, G, E):
    h = E / G
    u = (np.asarray(pos, np.float64) + E / 2) / h - 0.5
    i0 = np.floor(u)
    return i0.astype(np.int64), u - i0


def scatter3(pos, vel, mass, mask, G: int, E: float, in_scale: float = 1.0):
    """ScatterField.scatter (:237-250): (3, G, G) of [m mask, m mask vx, m mask vy] * in_scale / h^2."""
    h = E / G
    mm = np.asarray(mass, np.float64) * np.asarray(mask, np.float64)
    vel = np.asarray(vel, np.float64)
    val = np.stack([mm, mm * vel[:, 0], mm * vel[:, 1]], -1) * (in_scale / h ** 2)
    i0, w = _corners64(pos, G, E)
    out = np.zeros((3, G * G))
    for ox in (0, 1):
        for oy in (0, 1):
            ix, iy = i0[:, 0] + ox, i0[:, 1] + oy
            wt = (w[:, 0] if ox else 1 - w[:, 0]) * (w[:, 1] if oy else 1 - w[:, 1])
            ok = (ix >= 0) & (ix < G) & (iy >= 0) & (iy < G)
            flat = np.clip(iy, 0, G - 1) * G + np.clip(ix, 0, G - 1)
            for c in range(3):
                np.add.at(out[c], flat, val[:, c] * wt * ok)
    return out.reshape(3, G, G)


def gather(field, pos, E: float):
    """ScatterField.gather (:252-261): field (C, G, G) at pos -> (N, C)."""
    C, G, _ = field.shape
    fl = np.asarray(field, np.float64).reshape(C, G * G)
    i0, w = _corners64(pos, G, E)
    out = np.zeros((len(pos), C))
    for ox in (0, 1):
        for oy in (0, 1):
            ix, iy = i0[:, 0] + ox, i0[:, 1] + oy
            wt = (w[:, 0] if ox else 1 - w[:, 0]) * (w[:, 1] if oy else 1 - w[:, 1])
            ok = (ix >= 0) & (ix < G) & (iy >= 0) & (iy < G)
            flat = np.clip(iy, 0, G - 1) * G + np.clip(ix, 0, G - 1)
            out += (fl[:, flat] * (wt * ok)).T
    return out


def neg_grad(phi, h: float):
    """ScatterField.neg_grad (:551-555), zero padding: (G, G) -> (2, G, G)."""
    p = np.pad(np.asarray(phi, np.float64), 1)
    gx = (p[1:-1, 2:] - p[1:-1, :-2]) / (2 * h)
    gy = (p[2:, 1:-1] - p[:-2, 1:-1]) / (2 * h)
    return -np.stack([gx, gy])


def _mlp_params(sd, pre):
    return np.concatenate([np.asarray(sd[f"{pre}.{i}.{w}"], np.float64).reshape(-1)
                           for i in (0, 2, 4) for w in ("weight", "bias")])


class Model2D:
    """The production configuration: grid 128, extent 64, dt 0.1, U-Net 5 levels, learned kernel with
    the split window at ppe = pp, zero kpad, pair term (dense top-knn), momentum fix, Verlet."""

    def __init__(self, sd, grid=128, extent=64.0, dt=0.1, pp=2.0, knn=16, eps=0.5, in_scale=1.0, levels=5,
                 pair=True, prior=False, cu=False, kpad="zero"):
        self.sd = {k: np.asarray(v, np.float64) for k, v in sd.items()}
        self.G, self.E, self.h, self.dt, self.pp, self.knn, self.eps = grid, extent, extent / grid, dt, pp, knn, eps
        self.in_scale, self.levels, self.pair, self.prior, self.cu = in_scale, levels, pair, prior, cu
        self.ncol = 3 if cu else 2
        self.kpad = kpad
        self.ppe = pp * self.h / 0.5 if cu else pp  # ScatterField.ppe (:138-139)
        self.kparams, self.pparams = _mlp_params(sd, "kmlp"), _mlp_params(sd, "ppmlp")

    def kernel_acc(self, rho):
        """kernel_acc (:274-289): (2, G, G); split window at ppe, optional prior and cell units."""
        flags = 4 | (1 if self.cu else 0) | (2 if self.prior else 0) | (8 if self.kpad == "ext" else 0)
        a = O.kernel_acc_2d(rho, self.kparams, self.ncol, [], flags, self.ppe, self.eps, self.E)
        return np.moveaxis(a, -1, 0)

    def grid_force(self, x, field):
        """_grid_force (:620-666) on a scatter x (3, G, G): (acceleration grid (2, G, G), new field)."""
        ak = self.kernel_acc(x[0])
        phi = unet(self.sd, np.concatenate([x, ak, field], 0), self.levels)
        return neg_grad(phi[0], self.h) + ak, phi

    def force(self, pos, vel, mass, mask, field):
        """ScatterField.force (:561-615) for one scene: (acc (N, 2), field (1, G, G))."""
        x = scatter3(pos, vel, mass, mask, self.G, self.E, self.in_scale)
        acc, field = self.grid_force(x, field)
        a = gather(acc, pos, self.E)
        if self.pair:
            flags = (1 if self.cu else 0) | (2 if self.prior else 0)
            a = a + O.pair_acc_2d(pos, mass, mask, self.pparams, self.ncol, [], flags, self.ppe, self.eps, self.h,
                                  self.knn)
        mm = (np.asarray(mass, np.float64) * np.asarray(mask, np.float64))[:, None]
        a = a - (mm * a).sum(0, keepdims=True) / max(mm.sum(), 1e-9)
        return a * np.asarray(mask, np.float64)[:, None], field

    def step(self, pos, vel, mass, mask, state):
        """_step with verlet (:677-688); state = (field, a_prev or None)."""
        field, a_prev = state
        if a_prev is None:
            a_prev, field = self.force(pos, vel, mass, mask, field)
        dt = self.dt
        pos_new = pos + dt * vel + 0.5 * dt ** 2 * a_prev
        a_new, field = self.force(pos_new, vel + dt * a_prev, mass, mask, field)
        dv = 0.5 * dt * (a_prev + a_new)
        return pos_new, vel + dv, (field, a_new), dv


# ----------------------------------------------------------------------------------
# chunked large-N tick (scripts/scatter_bh_1b.py:107-146; speed: scripts/scatter_bh.py:22-23)
# ----------------------------------------------------------------------------------
def speed(p, c: float):
    return p / np.sqrt(1.0 + (p ** 2).sum(-1, keepdims=True) / c ** 2)


class Tick2D:
    """Sim with unit masses; state arrays are float64 here, rounded to `state_dtype` where the
    reference stores them (pos after the drift, mom after the kick)."""

    def __init__(self, model: Model2D, n: int, c: float = 10.0, dt: float = 0.1, ms: float = 1.0,
                 state_dtype=np.float32):
        self.m, self.n, self.c, self.dt, self.ms, self.sd = model, n, c, dt, ms, state_dtype
        self.field = np.zeros((1, model.G, model.G))

    def scatter_pass(self, pos, mom, drift: bool):
        v = speed(mom.astype(np.float64) * self.ms, self.c)
        if drift:
            pos = (pos.astype(np.float64) + self.dt * v).astype(self.sd)
        ones = np.ones(self.n)
        return pos, scatter3(pos, v, ones, ones, self.m.G, self.m.E, self.m.in_scale)

    def grid_force(self, x):
        acc, self.field = self.m.grid_force(x, self.field)
        w = x[0] * (self.m.h ** 2 / self.m.in_scale)
        return acc, (acc * w).sum((1, 2)) / self.n

    def _kick(self, pos, mom, acc, abar, kick):
        a = gather(acc, pos, self.m.E)
        return (mom.astype(np.float64) + kick * (a - abar) / self.ms).astype(self.sd)

    def tick(self, pos, mom):
        pos, x = self.scatter_pass(pos, mom, True)
        acc, abar = self.grid_force(x)
        return pos, self._kick(pos, mom, acc, abar, self.dt)

    def init_kick(self, pos, mom):
        _, x = self.scatter_pass(pos, mom, False)
        acc, abar = self.grid_force(x)
        return pos, self._kick(pos, mom, acc, abar, 0.5 * self.dt)
