"""Seeded 3D initial conditions in a unit periodic box [-E/2, E/2)^3 (total mass 1, G = 1).

Synthetic stand-ins for the workloads the PM step is measured on; all scenes are
generated on the host with numpy from an explicit seed:
  plummer  — Plummer sphere, scale radius a; positions by inverting M(r), velocities
             from the isotropic distribution function by rejection sampling
             (Aarseth, Henon & Wielen 1974, A&A 37, 183); radius truncated at rmax.
  uniform  — uniform in the box, zero velocity.
  clumpy   — 64 Gaussian clumps of width sigma, centres uniform, counts multinomial,
             zero velocity.
  disk     — exponential disk: cylindrical radius ~ Gamma(2, R_d), height ~ Laplace(z_d),
             circular velocity sqrt(M(<r)/r) from the enclosed mass of the sample.
  flyby    — two Plummer spheres (a = 0.03) 0.3 apart along x moving past each other along y
             with relative speed 0.5.
The seeds the reference uses are 4738 (training) and 9100/9200/9300 (evaluation).
"""
from __future__ import annotations

import numpy as np

SCENES = ("plummer", "uniform", "clumpy", "disk", "flyby")


def _iso(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def plummer(n, rng, a=0.05, rmax=0.45, mass=1.0, g=1.0):
    r = np.empty(0)
    while r.size < n:
        x1 = rng.random(2 * n + 16)
        x1 = x1[(x1 > 0) & (x1 < 1)]
        rr = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr < rmax]])
    r = r[:n]
    pos = r[:, None] * _iso(rng, n)
    q = np.empty(0)
    while q.size < n:
        x4 = rng.random(2 * n + 16)
        x5 = rng.random(2 * n + 16) * 0.1
        q = np.concatenate([q, x4[x5 < x4 ** 2 * (1 - x4 ** 2) ** 3.5]])
    q = q[:n]
    vesc = np.sqrt(2.0 * g * mass / a) * (1.0 + (r / a) ** 2) ** -0.25
    vel = (q * vesc)[:, None] * _iso(rng, n)
    return pos, vel


def uniform(n, rng, box=1.0):
    return (rng.random((n, 3)) - 0.5) * box, np.zeros((n, 3))


def clumpy(n, rng, nclump=64, sigma=0.02, box=1.0):
    cen = (rng.random((nclump, 3)) - 0.5) * box
    counts = rng.multinomial(n, np.full(nclump, 1.0 / nclump))
    idx = np.repeat(np.arange(nclump), counts)
    pos = cen[idx] + rng.normal(scale=sigma, size=(n, 3))
    return pos, np.zeros((n, 3))


def disk(n, rng, rd=0.08, zd=0.005, rmax=0.45, g=1.0):
    R = np.empty(0)
    while R.size < n:
        rr = rng.gamma(2.0, rd, size=2 * n + 16)
        R = np.concatenate([R, rr[rr < rmax]])
    R = R[:n]
    th = rng.random(n) * 2 * np.pi
    z = rng.laplace(0.0, zd, size=n)
    pos = np.stack([R * np.cos(th), R * np.sin(th), z], 1)
    r = np.sqrt(R ** 2 + z ** 2)
    order = np.argsort(r)
    menc = np.empty(n)
    menc[order] = np.arange(1, n + 1) / n
    vc = np.sqrt(g * menc / np.maximum(r, 1e-6))
    vel = np.stack([-vc * np.sin(th), vc * np.cos(th), np.zeros(n)], 1)
    return pos, vel


def flyby(n, rng, a=0.03, sep=0.3, vrel=0.5, rmax=0.12):
    n1 = n // 2
    p1, v1 = plummer(n1, rng, a=a, rmax=rmax, mass=0.5)
    p2, v2 = plummer(n - n1, rng, a=a, rmax=rmax, mass=0.5)
    p1[:, 0] -= sep / 2
    p2[:, 0] += sep / 2
    v1[:, 1] += vrel / 2
    v2[:, 1] -= vrel / 2
    return np.concatenate([p1, p2]), np.concatenate([v1, v2])


def wrap(pos, box=1.0):
    """Wrap into [-box/2, box/2) in float32 with the integrator's rule."""
    p = np.asarray(pos, np.float32)
    h, b = np.float32(box / 2), np.float32(box)
    p = np.where(p >= h, p - b, p)
    p = np.where(p < -h, p + b, p)
    p = np.mod(p + h, b) - h  # anything farther than one box away
    p = np.where(p >= h, p - b, p)
    return p.astype(np.float32)


def plummer_device(pos_out, vel_out, seed: int, a: float = 0.05, rmax: float = 0.45, chunk: int = 1 << 25) -> None:
    """The plummer() distribution sampled on the GPU into (n, 3) float32 CUDA tensors, chunk by
    chunk, for scenes too large to build on the host (10^9 bodies). The truncation at rmax is
    applied by drawing the enclosed-mass fraction from [0, M(rmax)) instead of by rejection, which
    gives the same truncated distribution; speeds use the same rejection sampler. Seeded with
    torch's device generator, so the bodies differ from plummer()'s for the same seed. Positions are
    wrapped into the unit box like wrap()."""
    import torch

    n, dev = pos_out.shape[0], pos_out.device
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    f64 = dict(dtype=torch.float64, device=dev)
    fmax = rmax ** 3 / (rmax ** 2 + a * a) ** 1.5
    vfac = (2.0 / a) ** 0.5

    def iso(m):
        v = torch.randn(m, 3, generator=gen, **f64)
        return v / v.norm(dim=1, keepdim=True)

    for s0 in range(0, n, chunk):
        m = min(chunk, n - s0)
        u = torch.rand(m, generator=gen, **f64).clamp_(min=1e-300) * fmax
        r = a / torch.sqrt(u.pow(-2.0 / 3.0) - 1.0)
        q = torch.empty(m, **f64)
        todo = torch.arange(m, device=dev)
        while todo.numel():
            k = todo.numel()
            x4 = torch.rand(k, generator=gen, **f64)
            x5 = torch.rand(k, generator=gen, **f64) * 0.1
            ok = x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
            q[todo[ok]] = x4[ok]
            todo = todo[~ok]
        p = (r[:, None] * iso(m)).float()
        p = torch.where(p >= 0.5, p - 1.0, p)
        p = torch.where(p < -0.5, p + 1.0, p)
        pos_out[s0:s0 + m] = p
        vel_out[s0:s0 + m] = ((q * vfac * (1.0 + (r / a) ** 2) ** -0.25)[:, None] * iso(m)).float()


def make_scene(kind: str, n: int, seed: int, box: float = 1.0):
    """(pos, vel, mass) float32 arrays of n bodies, centred in the periodic box."""
    rng = np.random.default_rng(seed)
    if kind == "plummer":
        pos, vel = plummer(n, rng)
    elif kind == "uniform":
        pos, vel = uniform(n, rng, box)
    elif kind == "clumpy":
        pos, vel = clumpy(n, rng, box=box)
    elif kind == "disk":
        pos, vel = disk(n, rng)
    elif kind == "flyby":
        pos, vel = flyby(n, rng)
    else:
        raise ValueError(f"unknown scene {kind!r}; expected one of {SCENES}")
    mass = np.full(n, 1.0 / n, np.float32)
    return wrap(pos, box), vel.astype(np.float32), mass
