"""CPU oracle for the PM gravity path — TEST INFRASTRUCTURE ONLY.

This module restates, in numpy, the arithmetic of the reference's particle-mesh path
(Faraday-dot-py/Augur, scripts/scatter_field.py and scripts/pm_baseline_force_error.py)
and its 3D periodic generalisation. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import it; the product (augur_gb300) never does.

Parity pins: the 2D functions are checked against outputs of the reference itself
(tests/golden/, generated by tests/golden/make_golden.py from the reference's own
code: ScatterField._corners, ScatterField.scatter/gather, pm_acc, exact_acc, and the
published plain-PM medians of results/pm_baseline_force_error.json).

Conventions (all from the reference):
  * grid covers [-E/2, E/2)^D, h = E/G, cell-centred CIC:
    u = (x + E/2)/h - 0.5 ; i0 = floor(u) ; w = u - i0          (scatter_field.py:179-182)
  * corner weights w or 1-w per axis, multiplied x then y (then z)  (scatter_field.py:203-209)
  * density channel m*mask*w/h^D                                  (scatter_field.py:238-241)
  * isolated PM: 2G zero-padded FFT convolution with -1/sqrt(d^2+eps^2), times h^2,
    crop, zero-padded central difference                          (pm_baseline_force_error.py:68-76,
                                                                   scatter_field.py:551-555)
  * periodic 3D (no reference implementation; the build's own spec):
    phi_k = -4 pi G rho_k / |k|^2, k = 2 pi m / E, k=0 -> 0; a_k = -i k phi_k with the
    Nyquist term of the differentiated axis set to 0; numpy rfftn/irfftn normalisation.
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32


# ----------------------------------------------------------------------------------
# cell index (scripts/scatter_field.py:179-182), bit-exact fp32
# ----------------------------------------------------------------------------------
def cell_index(pos, G: int, E: float):
    """u = (x + E/2)/h - 0.5 in IEEE fp32 with true division, i0 = floor(u), w = u - i0."""
    p = np.asarray(pos, dtype=F32)
    t = (p + F32(E / 2)).astype(F32)
    u = ((t / F32(E / G)).astype(F32) - F32(0.5)).astype(F32)
    f = np.floor(u).astype(F32)
    return f.astype(np.int64), (u - f).astype(F32)


def _axis_w(w, o):
    return w if o else (F32(1.0) - w).astype(F32)


def corners(D: int):
    """Corner order of ScatterField._corner_iter (ox outer, then oy, then oz)."""
    if D == 2:
        return [(ox, oy, 0) for ox in (0, 1) for oy in (0, 1)]
    return [(ox, oy, oz) for ox in (0, 1) for oy in (0, 1) for oz in (0, 1)]


def corner_weight(w, o, D):
    wt = (_axis_w(w[:, 0], o[0]) * _axis_w(w[:, 1], o[1])).astype(F32)
    if D == 3:
        wt = (wt * _axis_w(w[:, 2], o[2])).astype(F32)
    return wt


# ----------------------------------------------------------------------------------
# deposit
# ----------------------------------------------------------------------------------
def qscale(mm):
    """Fixed-point scale of the deterministic deposit: contributions c <= max(m) < 2^e
    are quantised as trunc(c * 2^(26-e)) (< 2^26, so 32 of them fit a 32-bit warp sum)
    and summed exactly in uint64."""
    mmax = float(np.max(mm)) if mm.size else 0.0
    e = math.frexp(mmax)[1] if mmax > 0 else 0
    S = 26 - e
    S1 = int(S / 2)
    return F32(math.ldexp(1.0, S1)), F32(math.ldexp(1.0, S - S1)), S


def deposit_fixed(pos, mass, mask, G: int, E: float, periodic: bool):
    """The GPU deposit's arithmetic, bit for bit: fp32 weights, uint32 quanta, exact
    uint64 sums, one fp32 rounding of the sum and one of the scale."""
    pos = np.asarray(pos, F32)
    D = pos.shape[1]
    mm = (np.asarray(mass, F32) * np.asarray(mask, F32)).astype(F32)
    q1, q2, S = qscale(np.maximum(mm, 0))
    h = E / G
    inv_hD = F32(1.0 / (h * h * h if D == 3 else h * h))
    outscale = F32(np.ldexp(inv_hD, -S))
    i0, w = cell_index(pos, G, E)
    acc = np.zeros(G ** D, dtype=np.uint64)
    live = mm > 0
    for o in corners(D):
        wt = corner_weight(w, o, D)
        c = (wt * mm).astype(F32)
        q = ((c * q1).astype(F32) * q2).astype(F32)
        q = np.trunc(q).astype(np.uint64)
        idx = [i0[:, d] + o[d] for d in range(D)]
        if periodic:
            idx = [np.mod(ix, G) for ix in idx]
            ok = live
        else:
            ok = live.copy()
            for ix in idx:
                ok &= (ix >= 0) & (ix < G)
            idx = [np.clip(ix, 0, G - 1) for ix in idx]
        flat = idx[0] + G * idx[1] + (G * G * idx[2] if D == 3 else 0)
        np.add.at(acc, flat[ok], q[ok])
    rho = (acc.astype(F32) * outscale).astype(F32)
    return rho.reshape((G,) * D)


def deposit_ref(pos, mass, mask, G: int, E: float, periodic: bool, dtype=np.float64):
    """ScatterField.scatter mass channel in the reference's idiom (index_add over corners):
    fp32 cell index, weights and values as the reference, accumulation in `dtype`."""
    pos = np.asarray(pos, F32)
    D = pos.shape[1]
    h = E / G
    i0, w = cell_index(pos, G, E)  # fp32, bit-exact with the reference
    val = ((np.asarray(mass, F32) * np.asarray(mask, F32)).astype(F32) * F32(1.0 / h ** D)).astype(F32)
    out = np.zeros(G ** D, dtype=dtype)
    for o in corners(D):
        wt = corner_weight(w, o, D).astype(dtype)
        idx = [i0[:, d] + o[d] for d in range(D)]
        if periodic:
            idx = [np.mod(ix, G) for ix in idx]
            ok = np.ones(len(pos), bool)
        else:
            ok = np.ones(len(pos), bool)
            for ix in idx:
                ok &= (ix >= 0) & (ix < G)
            idx = [np.clip(ix, 0, G - 1) for ix in idx]
        flat = idx[0] + G * idx[1] + (G * G * idx[2] if D == 3 else 0)
        np.add.at(out, flat[ok], (val * wt)[ok])
    return out.reshape((G,) * D)


# ----------------------------------------------------------------------------------
# Poisson solves
# ----------------------------------------------------------------------------------
def poisson_periodic(rho, E: float, g_newton: float = 1.0):
    """3D periodic: returns F (G,G,G,4) float64 = (a_x, a_y, a_z, phi), grid [z][y][x]."""
    rho = np.asarray(rho, np.float64)
    G = rho.shape[0]
    rk = np.fft.rfftn(rho)  # axes (z, y, x), x halved
    m_full = np.fft.fftfreq(G, 1.0 / G)  # 0..G/2-1, -G/2..-1
    mz = m_full[:, None, None]
    my = m_full[None, :, None]
    mx = np.arange(G // 2 + 1, dtype=np.float64)[None, None, :]
    kf = 2 * np.pi / E
    k2 = kf * kf * (mx ** 2 + my ** 2 + mz ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        green = np.where(k2 > 0, -4 * np.pi * g_newton / k2, 0.0)
    phik = rk * green
    out = np.empty((G, G, G, 4), np.float64)
    for c, m in enumerate((mx, my, mz)):
        mm = np.where(np.abs(m) == G // 2, 0.0, m)  # Nyquist of the differentiated axis -> 0
        out[..., c] = np.fft.irfftn(-1j * kf * mm * phik, s=(G, G, G), axes=(0, 1, 2))
    out[..., 3] = np.fft.irfftn(phik, s=(G, G, G), axes=(0, 1, 2))
    return out


def kernel_lattice_2d(G: int, h: float, eps: float):
    """-1/sqrt(d^2 + eps^2) on the 2G min-image lattice (pm_baseline_force_error.py:70-73), fp32."""
    idx = np.arange(2 * G, dtype=F32)
    d = (np.minimum(idx, F32(2 * G) - idx) * F32(h)).astype(F32)
    s = ((d[:, None] ** 2).astype(F32) + (d[None, :] ** 2).astype(F32)).astype(F32) + F32(eps * eps)
    return (F32(-1.0) / np.sqrt(s.astype(F32))).astype(F32)


def isolated_phi_2d(rho, E: float, eps: float, dtype=np.float64):
    """h^2 * irfft2(rfft2(rho, 2G) * rfft2(K))[:G, :G] (pm_baseline_force_error.py:74)."""
    G = rho.shape[0]
    h = E / G
    K = kernel_lattice_2d(G, h, eps).astype(dtype)
    full = np.fft.irfft2(np.fft.rfft2(np.asarray(rho, dtype), s=(2 * G, 2 * G)) * np.fft.rfft2(K), s=(2 * G, 2 * G))
    return (full * h ** 2)[:G, :G]


def neg_grad_2d(phi, h: float):
    """Zero-padded central difference (scatter_field.py:551-555) -> (G, G, 4) (a_x, a_y, 0, phi)."""
    p = np.pad(np.asarray(phi), 1)
    gx = (p[1:-1, 2:] - p[1:-1, :-2]) / (2 * h)
    gy = (p[2:, 1:-1] - p[:-2, 1:-1]) / (2 * h)
    out = np.zeros(phi.shape + (4,), dtype=phi.dtype)
    out[..., 0], out[..., 1], out[..., 3] = -gx, -gy, phi
    return out


def _gelu(x):
    from math import erf
    v = np.vectorize(erf)
    return 0.5 * x * (1.0 + v(x / np.sqrt(2.0)))


def kernel_lattice_mlp_2d(params, ncol: int, extra, flags: int, split_radius: float, eps: float, G: int, h: float):
    """Learned radial kernel on the 2G min-image lattice (ScatterField._kernel_fft,
    scatter_field.py:263-272), float64: K = kmlp(features(r)) with kmlp = Linear(ncol, 64), GELU,
    Linear(64, 64), GELU, Linear(64, 1); features [r, log(r + h)] or (flags & 1, cell units)
    [r/h, log(r/h + 1), log(0.5/h)] (:141-151) plus the constant extras; flags & 2: prior
    K = -(1 + K)/sqrt(r^2 + eps^2); flags & 4: split window 1 - (1 - min(r/rs, 1)^2)^2."""
    p = np.asarray(params, np.float64)
    H = 64
    o = 0
    W1 = p[o:o + H * ncol].reshape(H, ncol); o += H * ncol
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    L = 2 * G
    idx = np.arange(L, dtype=np.float64)
    d = np.minimum(idx, L - idx) * h
    r = np.sqrt(d[:, None] ** 2 + d[None, :] ** 2)
    if flags & 1:
        feats = [r / h, np.log(r / h + 1.0), np.full_like(r, np.log(0.5 / h))]
    else:
        feats = [r, np.log(r + h)]
    feats += [np.full_like(r, float(e)) for e in extra]
    f = np.stack(feats, -1)
    h1 = _gelu(f @ W1.T + b1)
    h2 = _gelu(h1 @ W2.T + b2)
    K = h2 @ W3 + b3
    if flags & 2:
        K = -(1.0 + K) / np.sqrt(r ** 2 + eps ** 2)
    if flags & 4:
        u = np.minimum(r / split_radius, 1.0) ** 2
        K = K * (1.0 - (1.0 - u) ** 2)
    return K


def kernel_acc_2d(rho, params, ncol: int, extra, flags: int, split_radius: float, eps: float, E: float):
    """ScatterField.kernel_acc (scatter_field.py:274-289) for one (G, G) density, float64:
    phi = h^2 irfft2(rfft2(rho, 2G) rfft2(K)); kpad "zero" (flags & 8 == 0): zero-padded central
    difference of phi[:G, :G]; kpad "ext": the difference reads phi at rows/columns -1 .. G of
    the 2G transform. Returns (G, G, 2) = (a_x, a_y)."""
    rho = np.asarray(rho, np.float64)
    G = rho.shape[0]
    h = E / G
    K = kernel_lattice_mlp_2d(params, ncol, extra, flags, split_radius, eps, G, h)
    full = np.fft.irfft2(np.fft.rfft2(rho, s=(2 * G, 2 * G)) * np.fft.rfft2(K), s=(2 * G, 2 * G)) * h ** 2
    if flags & 8:
        idx = [2 * G - 1] + list(range(G + 1))
        p = full[np.ix_(idx, idx)]
    else:
        p = np.pad(full[:G, :G], 1)
    gx = (p[1:-1, 2:] - p[1:-1, :-2]) / (2 * h)
    gy = (p[2:, 1:-1] - p[:-2, 1:-1]) / (2 * h)
    return np.stack([-gx, -gy], -1)


def _mlp64(params, ncol, f):
    """Linear(ncol, 64), GELU, Linear(64, 64), GELU, Linear(64, 1) on features f (..., ncol), float64."""
    p = np.asarray(params, np.float64)
    H = 64
    o = 0
    W1 = p[o:o + H * ncol].reshape(H, ncol); o += H * ncol
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    return _gelu(_gelu(f @ W1.T + b1) @ W2.T + b2) @ W3 + p[o]


def pair_acc_2d(pos, mass, mask, params, ncol: int, extra, flags: int, ppe: float, eps: float, h: float,
                knn: int = 16, queries=None):
    """ScatterField.pp_acc (scripts/scatter_field.py:291-300, 500-521), float64 brute force: for every
    body with mask > 0, the knn nearest other bodies with mask > 0 (r = sqrt(d^2 + 1e-8)); weight
    w = g(r) (1 - u)^2 with g = ppmlp(features(r)), u = min(r/ppe, 1)^2, features [r, log(r + 0.05)]
    or (flags & 1) [r/h, log(r/h + 0.1), log(0.5/h)] plus the extras; flags & 2 adds the prior
    r/q^3 - a_mesh, q = sqrt(r^2 + eps^2), a_mesh = -4 (1 - u) r / (ppe^2 q) + (1 - (1 - u)^2) r / q^3.
    acc_i = sum_j w m_j (x_j - x_i) / r. (The reference's cell-list mode searches the 3 x 3 cells of
    side ppe, which hold every body closer than ppe; weights vanish beyond ppe, so it agrees.)
    params None: g = 0 (the prior alone). queries: body indices to evaluate (default all); the
    other rows stay 0."""
    pos = np.asarray(pos, np.float64)
    mass = np.asarray(mass, np.float64)
    mask = np.asarray(mask, np.float64)
    n = pos.shape[0]
    out = np.zeros((n, 2))
    valid = mask > 0
    rows = np.nonzero(valid)[0] if queries is None else [int(q) for q in queries if valid[int(q)]]
    for i in rows:
        d = pos - pos[i]
        r = np.sqrt((d ** 2).sum(1) + 1e-8)
        cand = valid.copy()
        cand[i] = False
        idx = np.nonzero(cand)[0]
        sel = idx[np.argsort(r[idx], kind="stable")[:knn]]
        rs = r[sel]
        if flags & 1:
            f = [rs / h, np.log(rs / h + 0.1), np.full_like(rs, np.log(0.5 / h))]
        else:
            f = [rs, np.log(rs + 0.05)]
        f += [np.full_like(rs, float(e)) for e in extra]
        g = _mlp64(params, ncol, np.stack(f, -1)) if params is not None else np.zeros_like(rs)
        u = np.minimum(rs / ppe, 1.0) ** 2
        win = (1 - u) ** 2
        w = g * win
        if flags & 2:
            q = np.sqrt(rs ** 2 + eps ** 2)
            a_mesh = -4 * (1 - u) * rs / ppe ** 2 / q + (1 - win) * rs / q ** 3
            w = w + (rs / q ** 3 - a_mesh)
        out[i] = ((w * mass[sel])[:, None] * d[sel] / rs[:, None]).sum(0)
    return out


# ----------------------------------------------------------------------------------
# gather (scripts/scatter_field.py:252-261)
# ----------------------------------------------------------------------------------
def gather_f32(F4, pos, G: int, E: float, periodic: bool):
    """fp32 gather in the GPU's (and the reference's) corner and operation order.
    F4: (G,)*D + (4,) float32. Returns (acc (N, D), phi (N,))."""
    pos = np.asarray(pos, F32)
    D = pos.shape[1]
    F = np.asarray(F4, F32).reshape(-1, 4)
    i0, w = cell_index(pos, G, E)
    a = np.zeros((len(pos), D), F32)
    ph = np.zeros(len(pos), F32)
    for o in corners(D):
        wt = corner_weight(w, o, D)
        idx = [i0[:, d] + o[d] for d in range(D)]
        if periodic:
            idx = [np.mod(ix, G) for ix in idx]
        else:
            ok = np.ones(len(pos), bool)
            for ix in idx:
                ok &= (ix >= 0) & (ix < G)
            wt = np.where(ok, wt, F32(0)).astype(F32)
            idx = [np.clip(ix, 0, G - 1) for ix in idx]
        flat = idx[0] + G * idx[1] + (G * G * idx[2] if D == 3 else 0)
        f = F[flat]
        for d in range(D):
            a[:, d] = (a[:, d] + (f[:, d] * wt).astype(F32)).astype(F32)
        ph = (ph + (f[:, 3] * wt).astype(F32)).astype(F32)
    return a, ph


def gather_ref(F, pos, G: int, E: float, periodic: bool, dtype=np.float64):
    """Gather with the reference's fp32 weights, accumulated in `dtype` (float64 for tolerance checks)."""
    pos = np.asarray(pos, F32)
    D = pos.shape[1]
    i0, w = cell_index(pos, G, E)  # fp32 cell index and weights as the reference
    Ff = np.asarray(F, dtype).reshape(-1, F.shape[-1])
    out = np.zeros((len(pos), F.shape[-1]), dtype)
    for o in corners(D):
        wt = corner_weight(w, o, D).astype(dtype)
        idx = [i0[:, d] + o[d] for d in range(D)]
        if periodic:
            idx = [np.mod(ix, G) for ix in idx]
        else:
            ok = np.ones(len(pos), bool)
            for ix in idx:
                ok &= (ix >= 0) & (ix < G)
            wt = np.where(ok, wt, 0.0)
            idx = [np.clip(ix, 0, G - 1) for ix in idx]
        flat = idx[0] + G * idx[1] + (G * G * idx[2] if D == 3 else 0)
        out += Ff[flat] * wt[:, None]
    return out


# ----------------------------------------------------------------------------------
# full force evaluations
# ----------------------------------------------------------------------------------
def pm_force_periodic(pos, mass, mask, G: int, E: float = 1.0, g_newton: float = 1.0, fixed_deposit=True):
    """3D periodic plain PM force at the bodies, float64 FFT. Returns (acc (N,3), phi (N,))."""
    if fixed_deposit:
        rho = deposit_fixed(pos, mass, mask, G, E, True).astype(np.float64)
    else:
        rho = deposit_ref(pos, mass, mask, G, E, True)
    F = poisson_periodic(rho, E, g_newton)
    out = gather_ref(F, pos, G, E, True)
    m = np.asarray(mask, np.float64)[:, None]
    return out[:, :3] * m, out[:, 3] * m[:, 0]


def pm_acc_isolated_2d(pos, mass, mask, G: int, E: float, eps: float, fixed_deposit=False, f32=False):
    """pm_acc (scripts/pm_baseline_force_error.py:68-76) for one scene.

    f32=False: float64 throughout (after the fp32 cell index and weights).
    f32=True: rounds where the reference's float32 pipeline rounds — density and
    potential grids to fp32, then the central difference and gather in fp32. The
    potential is O(N/r) while the force is its difference across two cells, so that
    rounding of phi sets the reference's own force noise (~1e-5 relative)."""
    h = E / G
    if fixed_deposit:
        rho = deposit_fixed(pos, mass, mask, G, E, False).astype(np.float64)
    else:
        rho = deposit_ref(pos, mass, mask, G, E, False)
    if f32:
        rho = rho.astype(F32).astype(np.float64)
    phi = isolated_phi_2d(rho, E, eps)
    if f32:
        F = neg_grad_2d(phi.astype(F32), h).astype(F32)
        a, _ = gather_f32(F, pos, G, E, False)
        return (a * np.asarray(mask, F32)[:, None]).astype(np.float64)
    F = neg_grad_2d(phi, h)
    out = gather_ref(F, pos, G, E, False)
    return out[:, :2] * np.asarray(mask, np.float64)[:, None]


# ----------------------------------------------------------------------------------
# FP64 direct sums (scripts/scatter_scaling_ops.py:57-72) and Ewald
# ----------------------------------------------------------------------------------
def direct_sum(targets, sources, eps: float, mass=None, target_index=None, chunk=2048):
    """a_t = sum_j m_j (x_j - x_t) (|x_j - x_t|^2 + eps^2)^-1.5, self pair excluded."""
    tg = np.asarray(targets, np.float64)
    src = np.asarray(sources, np.float64)
    m = np.ones(len(src)) if mass is None else np.asarray(mass, np.float64)
    out = np.zeros_like(tg)
    for s in range(0, len(tg), chunk):
        d = src[None, :, :] - tg[s:s + chunk, None, :]
        r2 = (d ** 2).sum(-1) + eps ** 2
        inv = r2 ** -1.5
        if target_index is not None:
            ti = np.asarray(target_index)[s:s + chunk]
            rows = np.nonzero(ti >= 0)[0]
            inv[rows, ti[rows]] = 0.0
        out[s:s + chunk] = (d * (inv * m[None, :])[..., None]).sum(1)
    return out


def ewald_unit(x, alpha=2.0, nmax=2, hmax2=10):
    """Periodic (unit box) acceleration at displacements x (K,3) from a unit mass at the origin,
    including every image (no minimum-image split). Hernquist, Bouchet & Suto (1991)."""
    x = np.asarray(x, np.float64)
    a = np.zeros_like(x)
    rng = range(-nmax, nmax + 1)
    for nx in rng:
        for ny in rng:
            for nz in rng:
                d = x - np.array([nx, ny, nz], np.float64)
                r2 = (d ** 2).sum(-1)
                r = np.sqrt(r2)
                with np.errstate(divide="ignore", invalid="ignore"):
                    f = (_erfc(alpha * r) + 2 * alpha * r / np.sqrt(np.pi) * np.exp(-alpha ** 2 * r2)) / (r2 * r)
                f = np.where(r2 > 0, f, 0.0)
                a -= d * f[:, None]
    hr = range(-3, 4)
    for hx in hr:
        for hy in hr:
            for hz in hr:
                h2 = hx * hx + hy * hy + hz * hz
                if h2 == 0 or h2 > hmax2:
                    continue
                hv = np.array([hx, hy, hz], np.float64)
                f = 2.0 / h2 * np.exp(-np.pi ** 2 * h2 / alpha ** 2) * np.sin(2 * np.pi * (x @ hv))
                a -= f[:, None] * hv[None, :]
    return a


def _erfc(x):
    from scipy.special import erfc

    return erfc(x)


def direct_sum_periodic(targets, sources, eps: float, box: float, mass=None, target_index=None):
    """Periodic FP64 truth: softened minimum-image Newtonian + exact Ewald correction
    (periodic sum minus the nearest image), evaluated without tabulation."""
    tg = np.asarray(targets, np.float64)
    src = np.asarray(sources, np.float64)
    m = np.ones(len(src)) if mass is None else np.asarray(mass, np.float64)
    out = np.zeros_like(tg)
    for t in range(len(tg)):
        d = src - tg[t]
        d -= box * np.rint(d / box)
        r2 = (d ** 2).sum(-1)
        keep = np.ones(len(src), bool)
        if target_index is not None and target_index[t] >= 0:
            keep[target_index[t]] = False
        inv = (r2 + eps ** 2) ** -1.5
        a = (d * (inv * m)[:, None])[keep].sum(0)
        u = -d / box
        corr = ewald_unit(u)
        r = np.sqrt(r2)[:, None] / box
        with np.errstate(divide="ignore", invalid="ignore"):
            newt = np.where(r > 0, -u / np.maximum(r, 1e-300) ** 3, 0.0)
        corr = (corr - newt) / box ** 2
        a += (corr * m[:, None])[keep].sum(0)
        out[t] = a
    return out


def ewald_table(n: int = 64):
    """The Ewald correction for a unit mass in a unit box (periodic sum minus the nearest-image
    Newtonian term) on an (n+1)^3 grid over the positive octant [0, 1/2]^3, indexed [z][y][x]:
    the table the GPU's periodic direct sum interpolates. Zero at the origin."""
    P = n + 1
    g = 0.5 * np.arange(P) / n
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    X = np.stack([x.ravel(), y.ravel(), z.ravel()], -1)
    a = ewald_unit(X)
    r = np.linalg.norm(X, axis=-1)
    with np.errstate(divide="ignore", invalid="ignore"):
        newt = np.where(r[:, None] > 0, -X / np.maximum(r, 1e-300)[:, None] ** 3, 0.0)
    corr = a - newt
    corr[r == 0] = 0.0
    return corr.reshape(P, P, P, 3)


def ewald_interp(tab, u):
    """Trilinear interpolation of ewald_table at unit-box displacements u (K,3) in [-1/2, 1/2]^3,
    folded into the positive octant (the correction is odd in each component)."""
    n = tab.shape[0] - 1
    u = np.asarray(u, np.float64)
    s = np.where(u < 0, -1.0, 1.0)
    v = np.minimum(np.abs(u) * (2 * n), n)
    i = np.minimum(v.astype(np.int64), n - 1)
    f = v - i
    out = np.zeros_like(u)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
                out += w[:, None] * tab[i[:, 2] + dz, i[:, 1] + dy, i[:, 0] + dx]
    return s * out


def direct_sum_periodic_tabulated(targets, sources, eps: float, box: float, tab, mass=None, target_index=None):
    """direct_sum_periodic with the Ewald correction read from ewald_table by trilinear
    interpolation instead of summed exactly: the arithmetic of the GPU's periodic direct sum."""
    tg = np.asarray(targets, np.float64)
    src = np.asarray(sources, np.float64)
    m = np.ones(len(src)) if mass is None else np.asarray(mass, np.float64)
    out = np.zeros_like(tg)
    for t in range(len(tg)):
        d = src - tg[t]
        d -= box * np.rint(d / box)
        r2 = (d ** 2).sum(-1)
        keep = np.ones(len(src), bool)
        if target_index is not None and target_index[t] >= 0:
            keep[target_index[t]] = False
        inv = (r2 + eps ** 2) ** -1.5
        corr = ewald_interp(tab, -d / box) / box ** 2
        out[t] = ((d * (inv * m)[:, None]) + corr * m[:, None])[keep].sum(0)
    return out


def energy_sums(vel, mass, mask, phi=None):
    """float64 reference of the compensated reductions: kinetic energy sum m v^2 / 2, momentum
    sum m v, mass sum m and potential energy sum m phi / 2, with m = mass * mask (fp32 product)."""
    m = (np.asarray(mass, F32) * np.asarray(mask, F32)).astype(np.float64)
    v = np.asarray(vel, np.float64)
    out = {"ke": float(0.5 * (m * (v ** 2).sum(-1)).sum()), "momentum": (m[:, None] * v).sum(0).tolist(),
           "mass": float(m.sum()), "pe": 0.0}
    if phi is not None:
        out["pe"] = float(0.5 * (m * np.asarray(phi, np.float64)).sum())
    return out


# ----------------------------------------------------------------------------------
# integrators
# ----------------------------------------------------------------------------------
def wrap_f32(x, E: float):
    x = np.asarray(x, F32)
    h = F32(E / 2)
    x = np.where(x >= h, (x - F32(E)).astype(F32), x)
    x = np.where(x < -h, (x + F32(E)).astype(F32), x)
    return x.astype(F32)


def run_kdk(pos, vel, mass, mask, G, E, dt, nsteps, force_fn):
    """Merged kick-drift-kick as the GPU run loop: v += dt/2 a ; then per step x += dt v (wrapped),
    a = F(x), v += dt a (last kick dt/2). force_fn(pos) -> acc (float32 arrays)."""
    x = np.asarray(pos, F32).copy()
    v = np.asarray(vel, F32).copy()
    a = force_fn(x)
    v = (v + (F32(0.5 * dt) * a).astype(F32)).astype(F32)
    for s in range(nsteps):
        x = wrap_f32((x + (F32(dt) * v).astype(F32)).astype(F32), E)
        a = force_fn(x)
        k = F32(dt) if s < nsteps - 1 else F32(0.5 * dt)
        v = (v + (k * a).astype(F32)).astype(F32)
    return x, v, a


# ----------------------------------------------------------------------------------
# metrics (scripts/pm_baseline_force_error.py:88-92)
# ----------------------------------------------------------------------------------
def errs(a, at, mask=None):
    """Per-body |a - a_true| / rms(|a_true|) and |a - a_true| / |a_true|."""
    a = np.asarray(a, np.float64)
    at = np.asarray(at, np.float64)
    m = np.ones(len(a)) if mask is None else np.asarray(mask, np.float64)
    rms = np.sqrt((np.linalg.norm(at, axis=-1) ** 2 * m).sum() / m.sum())
    e = np.linalg.norm(a - at, axis=-1) / rms
    rel = np.linalg.norm(a - at, axis=-1) / np.maximum(np.linalg.norm(at, axis=-1), 1e-12)
    return e[m > 0], rel[m > 0]


def median_lower(x):
    """torch.Tensor.median() as the reference's `stats` uses it (pm_baseline_force_error.py:95):
    the lower of the two middle values for an even count, not their mean."""
    x = np.sort(np.asarray(x).ravel())
    return float(x[(len(x) - 1) // 2])


def rel_rms(a, b):
    """||a - b||_2 / ||b||_2 over all bodies and components."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))
