"""Self-consistency of the oracle's 3D periodic restatement (no reference implementation exists)."""
import numpy as np

from oracle import pm_oracle as O


def test_single_mode_poisson_is_analytic():
    G, E = 32, 1.0
    x = (np.arange(G) + 0.5) / G * E - E / 2
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    kx = 2 * np.pi * 3 / E
    rho = 1.0 + 0.5 * np.cos(kx * xx)
    F = O.poisson_periodic(rho, E, 1.0)
    # nabla^2 phi = 4 pi (rho - mean) -> phi = -4 pi 0.5 cos / k^2 ; a_x = -dphi/dx
    phi = -4 * np.pi * 0.5 * np.cos(kx * xx) / kx ** 2
    ax = -4 * np.pi * 0.5 * np.sin(kx * xx) / kx
    assert np.allclose(F[..., 3], phi, atol=1e-12)
    assert np.allclose(F[..., 0], ax, atol=1e-10)
    assert np.allclose(F[..., 1], 0, atol=1e-10) and np.allclose(F[..., 2], 0, atol=1e-10)


def test_periodic_pm_conserves_momentum():
    rng = np.random.default_rng(1)
    n, G = 2000, 32
    pos = ((rng.random((n, 3)) - 0.5) * 0.6).astype(np.float32)
    mass = np.full(n, 1.0 / n)
    a, _ = O.pm_force_periodic(pos, mass, np.ones(n), G)
    p = (mass[:, None] * a).sum(0)
    assert np.abs(p).max() < 1e-9 * np.abs(mass[:, None] * a).sum()


def test_fixed_point_deposit_is_order_independent_and_exact():
    rng = np.random.default_rng(2)
    n, G = 5000, 16
    pos = ((rng.random((n, 3)) - 0.5)).astype(np.float32)
    mass = rng.random(n).astype(np.float32)
    mask = (rng.random(n) > 0.2).astype(np.float32)
    a = O.deposit_fixed(pos, mass, mask, G, 1.0, True)
    perm = rng.permutation(n)
    b = O.deposit_fixed(pos[perm], mass[perm], mask[perm], G, 1.0, True)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    r = O.deposit_ref(pos, mass, mask, G, 1.0, True)
    assert np.abs(a - r).max() <= 1e-6 * np.abs(r).max()
    assert abs(a.sum() / G ** 3 - (mass * mask).sum()) < 1e-5 * (mass * mask).sum()


def test_ewald_unit_is_odd_and_vanishes_on_symmetry_points():
    x = np.array([[0.5, 0.0, 0.0], [0.5, 0.5, 0.5], [0.0, 0.5, 0.0]])
    a = O.ewald_unit(x)
    assert np.abs(a).max() < 1e-10
    y = np.array([[0.1, 0.2, -0.3]])
    assert np.allclose(O.ewald_unit(y), -O.ewald_unit(-y), atol=1e-12)


def test_ewald_matches_pm_on_a_pair():
    """Far from the source the periodic PM force approaches the Ewald force."""
    G, E = 64, 1.0
    src = np.array([[0.0, 0.0, 0.0]], np.float32)
    tgt = np.array([[0.3, 0.1, -0.2]], np.float32)
    pos = np.concatenate([src, tgt])
    mass = np.array([1.0, 1e-9])
    a, _ = O.pm_force_periodic(pos, mass, np.ones(2), G)
    ew = O.direct_sum_periodic(tgt, src, eps=0.0, box=E)
    assert np.linalg.norm(a[1] - ew[0]) < 0.02 * np.linalg.norm(ew[0])
