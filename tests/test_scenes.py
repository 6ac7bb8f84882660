"""Distribution properties of the seeded scene generators (augur_gb300/scenes.py), on the CPU.

Each scene is checked against a property of the distribution it samples, within sampling error:
the Plummer sphere's enclosed-mass law, velocity bound and virial ratio; the exponential disk's
radial and vertical scale lengths and circular velocities; the clumps' widths; the flyby's two
spheres; the uniform scene's moments."""
import math

import numpy as np
import pytest

from augur_gb300 import scenes


def test_plummer_enclosed_mass_and_escape_bound():
    n, a, rmax = 200_000, 0.05, 0.45
    pos, vel = scenes.plummer(n, np.random.default_rng(1), a=a, rmax=rmax)
    r = np.linalg.norm(pos, axis=1)
    assert r.max() < rmax
    menc = lambda x: x ** 3 / (x * x + a * a) ** 1.5
    for x in (0.01, 0.03, 0.05, 0.1, 0.2, 0.3):
        assert abs((r < x).mean() - menc(x) / menc(rmax)) < 4 * math.sqrt(0.25 / n), x
    vesc = np.sqrt(2.0 / a) * (1 + (r / a) ** 2) ** -0.25
    assert (np.linalg.norm(vel, axis=1) < vesc).all()
    # isotropy of the directions
    assert np.abs((pos / r[:, None]).mean(0)).max() < 5 / math.sqrt(3 * n)


def test_plummer_virial_ratio():
    """2K / |W| = 1 for a Plummer sphere in equilibrium (the truncation at 9a moves it by ~1 %)."""
    n = 6000
    pos, vel = scenes.plummer(n, np.random.default_rng(2))
    m = 1.0 / n
    ke = 0.5 * m * (vel ** 2).sum()
    w = 0.0
    for s in range(0, n, 1000):
        d = np.linalg.norm(pos[s:s + 1000, None, :] - pos[None, :, :], axis=-1)
        idx = np.arange(s, min(n, s + 1000))
        d[idx - s, idx] = np.inf
        w -= 0.5 * m * m * (1.0 / d).sum()
    assert abs(2 * ke / abs(w) - 1.0) < 0.06


def test_disk_scale_lengths_and_circular_speed():
    n, rd, zd = 200_000, 0.08, 0.005
    pos, vel = scenes.disk(n, np.random.default_rng(3), rd=rd, zd=zd)
    sp = pytest.importorskip("scipy.special")
    R = np.hypot(pos[:, 0], pos[:, 1])
    # R ~ Gamma(2, rd) truncated at 0.45: E[R | R < c] = 2 rd P(3, c/rd) / P(2, c/rd)
    x = 0.45 / rd
    mean = 2 * rd * sp.gammainc(3, x) / sp.gammainc(2, x)
    assert abs(R.mean() / mean - 1.0) < 0.01
    assert abs(np.abs(pos[:, 2]).mean() / zd - 1.0) < 0.02
    # circular orbits: v perpendicular to R, v^2 r = M(<r)
    vr = (vel[:, 0] * pos[:, 0] + vel[:, 1] * pos[:, 1]) / np.maximum(R, 1e-12)
    assert np.abs(vr).max() < 1e-9
    r = np.linalg.norm(pos, axis=1)
    v2 = (vel ** 2).sum(1)
    order = np.argsort(r)
    menc = np.empty(n)
    menc[order] = np.arange(1, n + 1) / n
    assert np.allclose(v2 * np.maximum(r, 1e-6), menc, rtol=1e-9)


def test_clumpy_widths_and_counts():
    n = 128_000
    rng = np.random.default_rng(4)
    pos, vel = scenes.clumpy(n, rng)
    assert (vel == 0).all()
    # re-derive the clump centres with the same seed and check the per-clump spread
    rng2 = np.random.default_rng(4)
    cen = rng2.random((64, 3)) - 0.5
    d = np.linalg.norm(pos[:, None, :] - cen[None, :, :], axis=-1)
    lab = d.argmin(1)
    counts = np.bincount(lab, minlength=64)
    assert abs(counts.mean() - n / 64) < 1e-9 and counts.std() < 4 * math.sqrt(n / 64)
    off = pos - cen[lab]
    assert abs(off.std() / 0.02 - 1.0) < 0.05


def test_flyby_and_uniform():
    n = 100_000
    pos, vel = scenes.flyby(n, np.random.default_rng(5))
    h = n // 2
    c1, c2 = pos[:h].mean(0), pos[h:].mean(0)
    assert abs((c2 - c1)[0] - 0.3) < 0.005 and np.abs((c2 - c1)[1:]).max() < 0.005
    dv = vel[h:].mean(0) - vel[:h].mean(0)
    assert abs(dv[1] + 0.5) < 0.01
    u, _ = scenes.uniform(n, np.random.default_rng(6))
    assert np.abs(u.mean(0)).max() < 5 * math.sqrt(1 / 12 / n)
    assert np.abs(u.var(0) - 1 / 12).max() < 0.01 / 12 * 5


@pytest.mark.parametrize("kind", scenes.SCENES)
def test_make_scene_is_seeded_and_in_the_box(kind):
    a = scenes.make_scene(kind, 5000, seed=9100)
    b = scenes.make_scene(kind, 5000, seed=9100)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    pos, vel, mass = a
    assert pos.dtype == np.float32 and (pos >= -0.5).all() and (pos < 0.5).all()
    assert abs(float(mass.astype(np.float64).sum()) - 1.0) < 1e-6
