"""The 3D periodic PM step written the way the reference writes its PM path, on the CPU —
TEST / BASELINE INFRASTRUCTURE ONLY (bench.py's CPU-baseline and reference legs).

The reference's PM (scripts/pm_baseline_force_error.py:68-76 with ScatterField.scatter /
gather, scripts/scatter_field.py:237-261) is PyTorch: a CIC deposit by `index_add_` over the
corners, `torch.fft` for the solve, and a gather by indexing. This module applies that
idiom to the 3D periodic step the GPU path computes (Green's function -4 pi G / k^2,
spectral gradient, merged kick-drift-kick), in float32 with every host thread torch uses.
"""
from __future__ import annotations

import math

import torch


class TorchCPUPM:
    def __init__(self, G: int, E: float = 1.0, g_newton: float = 1.0):
        self.G, self.E, self.h = G, E, E / G
        m = torch.fft.fftfreq(G, 1.0 / G)
        mx = torch.arange(G // 2 + 1, dtype=torch.float64)
        kf = 2 * math.pi / E
        k2 = kf * kf * (mx[None, None, :] ** 2 + m[None, :, None] ** 2 + m[:, None, None] ** 2)
        green = torch.where(k2 > 0, -4 * math.pi * g_newton / k2, torch.zeros_like(k2))
        nyq = G // 2

        def d(v):
            return torch.where(v.abs() == nyq, torch.zeros_like(v), v) * kf

        self.green = green.to(torch.complex64)
        self.kx = d(mx)[None, None, :].to(torch.complex64)
        self.ky = d(m)[None, :, None].to(torch.complex64)
        self.kz = d(m)[:, None, None].to(torch.complex64)

    def _corners(self, pos):
        u = (pos + self.E / 2) / self.h - 0.5
        i0 = torch.floor(u)
        return i0.long(), u - i0

    def force(self, pos, mass):
        G = self.G
        i0, w = self._corners(pos)
        val = mass / self.h ** 3
        rho = torch.zeros(G * G * G, dtype=torch.float32)
        flats, wts = [], []
        for ox in (0, 1):
            for oy in (0, 1):
                for oz in (0, 1):
                    ix = (i0[:, 0] + ox) % G
                    iy = (i0[:, 1] + oy) % G
                    iz = (i0[:, 2] + oz) % G
                    wt = (w[:, 0] if ox else 1 - w[:, 0]) * (w[:, 1] if oy else 1 - w[:, 1]) * \
                         (w[:, 2] if oz else 1 - w[:, 2])
                    flat = (iz * G + iy) * G + ix
                    rho.index_add_(0, flat, val * wt)
                    flats.append(flat)
                    wts.append(wt)
        phik = torch.fft.rfftn(rho.view(G, G, G)) * self.green
        F = torch.stack([torch.fft.irfftn(-1j * k * phik, s=(G, G, G)) for k in (self.kx, self.ky, self.kz)], -1)
        F = F.reshape(-1, 3)
        acc = torch.zeros_like(pos)
        for flat, wt in zip(flats, wts):
            acc += F[flat] * wt[:, None]
        return acc

    def wrap(self, x):
        half = self.E / 2
        x = torch.where(x >= half, x - self.E, x)
        return torch.where(x < -half, x + self.E, x)

    def begin(self, pos, vel, mass, dt):
        """Opening half kick: v += dt/2 F(x)."""
        vel += 0.5 * dt * self.force(pos, mass)

    def step(self, pos, vel, mass, dt):
        """One merged step: x += dt v (wrapped) ; v += dt F(x)."""
        pos.copy_(self.wrap(pos + dt * vel))
        vel += dt * self.force(pos, mass)
