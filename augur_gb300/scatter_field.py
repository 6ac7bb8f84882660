"""Drop-in for the reference's PM path behind ScatterField's call signature.

Reference interface (Faraday-dot-py/Augur, scripts/scatter_field.py):
    ScatterField.force(pos, vel, mass, mask, field) -> (acc, field)          :561-565
    ScatterField.step(pos, vel, mass, mask, field)  -> (pos, vel, field, dv) :668-688
    ScatterField.scatter / gather / init_field                               :237-261, :557-559
    pm_acc(model, pos, vel, mass, mask) -> acc      scripts/pm_baseline_force_error.py:68-76
Layouts are the reference's: pos/vel (B, N, D) float32, mass/mask (B, N); grids
(B, C, G, G[, G]). Each scene is one call into the native plan on the current stream.

Two modes:
  mode="isolated", dim=2: the reference's plain PM (2G zero-padded softened kernel,
      central-difference gradient), bit-exact cell indices, forces within 1e-5 rel RMS.
  mode="periodic", dim=3: the periodic box (-4 pi G / k^2, spectral gradient).
An optional learned correction (`net`) adds a CNN force-correction field; see cnn.py.
"""
from __future__ import annotations

import torch

from .pm import PMPlan


class ScatterField:
    def __init__(self, grid: int = 64, extent: float = 1.0, dim: int = 3, mode: str = "periodic",
                 eps: float = 0.5, g_newton: float = 1.0, dt: float = 1e-3, verlet: bool = True,
                 momfix: bool = False, net=None, device=None):
        if mode == "periodic" and dim != 3:
            raise ValueError("the periodic mode is 3D")
        if mode != "periodic" and dim != 2:
            raise ValueError("the isolated (reference) mode is 2D")
        self.grid, self.extent, self.h, self.dim, self.mode = grid, float(extent), float(extent) / grid, dim, mode
        self.eps, self.g_newton, self.dt, self.verlet, self.momfix = eps, g_newton, dt, verlet, momfix
        self.net = net
        self.device = torch.device(device) if device is not None else None
        self._plans: dict = {}

    # ---- plan cache --------------------------------------------------------------------
    def plan(self, n: int, device) -> PMPlan:
        device = torch.device(device)
        p = self._plans.get(device)
        if p is None or p.max_bodies < n:
            if p is not None:
                p.close()
            cap = max(int(n), 1)
            p = PMPlan(self.dim, self.grid, cap, self.mode, self.extent, self.eps, self.g_newton, device=device)
            self._plans[device] = p
        return p

    def close(self):
        for p in self._plans.values():
            p.close()
        self._plans.clear()

    # ---- reference sub-ops ---------------------------------------------------------------
    def init_field(self, B, device, dtype=torch.float32):
        f = torch.zeros((B, 1) + (self.grid,) * self.dim, device=device, dtype=dtype)
        return (f, None) if self.verlet else f

    def scatter(self, pos, vel, mass, mask):
        """Mass channel of ScatterField.scatter: (B, 1, G^D) density m*mask*w/h^D."""
        B, N = pos.shape[:2]
        p = self.plan(N, pos.device)
        out = torch.empty((B, 1) + (self.grid,) * self.dim, device=pos.device, dtype=torch.float32)
        for b in range(B):
            out[b, 0] = p.deposit(pos[b].contiguous(), mass[b].contiguous(), mask[b].contiguous())
        return out

    def gather(self, field, pos):
        """(B, C, G^D) field at the bodies -> (B, N, C), CIC weights, out-of-grid corners dropped."""
        B, Cc = field.shape[:2]
        N = pos.shape[1]
        p = self.plan(N, pos.device)
        out = torch.empty((B, N, Cc), device=pos.device, dtype=torch.float32)
        ones = torch.ones(N, device=pos.device)
        # the native gather returns lanes 0..D-1 of a 4-lane grid as acc and lane 3 as phi
        lanes = [0, 1, 2, 3] if self.dim == 3 else [0, 1, 3]
        for b in range(B):
            for c0 in range(0, Cc, len(lanes)):
                k = min(len(lanes), Cc - c0)
                f4 = torch.zeros((self.grid,) * self.dim + (4,), device=pos.device, dtype=torch.float32)
                for j in range(k):
                    f4[..., lanes[j]] = field[b, c0 + j]
                acc, phi = p.gather(f4, pos[b].contiguous(), ones)
                vals = torch.cat([acc, phi[:, None]], 1)
                out[b, :, c0:c0 + k] = vals[:, :k]
        return out

    def potential_force(self, rho):
        """Grid force (..., 4) = (a_x, a_y, a_z, phi) of one density grid (the FFT solve + gradient)."""
        p = self.plan(1, rho.device)
        return p.poisson(rho.contiguous())

    # ---- force / step ----------------------------------------------------------------------
    def force(self, pos, vel, mass, mask, field):
        B, N, D = pos.shape
        p = self.plan(N, pos.device)
        acc = torch.empty_like(pos)
        for b in range(B):
            acc[b] = p.force(pos[b].contiguous(), mass[b].contiguous(), mask[b].contiguous())
        if self.net is not None:
            acc = acc + self.net.correction(self, pos, mass, mask)
        if self.momfix:
            mm = (mass * mask)[..., None]
            acc = (acc - (mm * acc).sum(1, keepdim=True) / mm.sum(1, keepdim=True).clamp_min(1e-9)) * mask[..., None]
        return acc, field

    def step(self, pos, vel, mass, mask, field, dt=None):
        """Velocity Verlet (scripts/scatter_field.py:677-688); periodic mode wraps positions."""
        dt = self.dt if dt is None else dt
        if not self.verlet:
            a, field = self.force(pos, vel, mass, mask, field)
            dv = a * dt
            return pos + dt * (vel + 0.5 * dv), vel + dv, field, dv
        field, a_prev = field
        if self.net is not None:
            if a_prev is None:
                a_prev, field = self.force(pos, vel, mass, mask, field)
            pos_new = pos + dt * vel + 0.5 * dt ** 2 * a_prev
            if self.mode == "periodic":
                half = self.extent / 2
                pos_new = torch.where(pos_new >= half, pos_new - self.extent, pos_new)
                pos_new = torch.where(pos_new < -half, pos_new + self.extent, pos_new)
            a_new, field = self.force(pos_new, vel + dt * a_prev, mass, mask, field)
            dv = 0.5 * dt * (a_prev + a_new)
            return pos_new, vel + dv, (field, a_new), dv
        B, N, D = pos.shape
        p = self.plan(N, pos.device)
        pos_n, vel_n = pos.clone().contiguous(), vel.clone().contiguous()
        have = a_prev is not None
        a = a_prev.clone().contiguous() if have else torch.empty_like(pos)
        for b in range(B):
            p.step(pos_n[b], vel_n[b], a[b], mass[b].contiguous(), mask[b].contiguous(), dt=dt, have_acc=have)
        dv = vel_n - vel
        return pos_n, vel_n, (field, a), dv

    def run(self, pos, vel, mass, mask, nsteps: int, dt=None):
        """nsteps leapfrog steps on the device-resident sorted state (periodic mode)."""
        dt = self.dt if dt is None else dt
        B, N, D = pos.shape
        p = self.plan(N, pos.device)
        pos_n, vel_n = pos.clone().contiguous(), vel.clone().contiguous()
        for b in range(B):
            p.run(pos_n[b], vel_n[b], mass[b].contiguous(), mask[b].contiguous(), dt=dt, nsteps=nsteps)
        return pos_n, vel_n


def pm_acc(model: ScatterField, pos, vel, mass, mask):
    """Plain PM acceleration (scripts/pm_baseline_force_error.py:68-76)."""
    B, N, D = pos.shape
    p = model.plan(N, pos.device)
    out = torch.empty_like(pos)
    for b in range(B):
        out[b] = p.force(pos[b].contiguous(), mass[b].contiguous(), mask[b].contiguous())
    return out
