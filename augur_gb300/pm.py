"""Host-side API of the GB300 PM gravity step.

`PMPlan` wraps one C-ABI plan (include/augur_pm.h): a grid geometry plus its device
workspace. Every method takes CUDA float32 tensors in the reference's layouts
((N, D) positions/velocities, (N,) masses and masks), enqueues the native kernels on
the current torch stream and returns without synchronising. There is no CPU path:
CPU tensors, wrong dtypes or a missing library raise.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import AUGUR_MODE_ISOLATED_SOFTENED, AUGUR_MODE_PERIODIC

MODES = {"periodic": AUGUR_MODE_PERIODIC, "isolated": AUGUR_MODE_ISOLATED_SOFTENED,
         "isolated_softened": AUGUR_MODE_ISOLATED_SOFTENED}


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _need(t: torch.Tensor, name: str, dtype=torch.float32, shape=None, device=None) -> torch.Tensor:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the PM path has no CPU implementation)")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if device is not None and t.device != device:
        raise ValueError(f"{name} is on {t.device}, the plan is on {device}")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t


class _DeviceBuffer:
    """__cuda_array_interface__ view of plan-owned device memory (float32)."""

    def __init__(self, addr: int, nbytes: int, device):
        self.__cuda_array_interface__ = {"shape": (nbytes // 4,), "typestr": "<f4", "data": (int(addr), False),
                                         "version": 3, "strides": None}


class PMPlan:
    """One grid geometry + workspace for up to ``max_bodies`` bodies.

    dim=3, mode="periodic": unit-cell periodic box of side ``extent`` (phi_k = -4 pi G rho_k/k^2).
    dim=2, mode="isolated": the reference's plain PM (scripts/pm_baseline_force_error.py:68-76).
    """

    def __init__(self, dim: int, grid: int, max_bodies: int, mode: str = "periodic", extent: float = 1.0,
                 eps: float = 0.5, g_newton: float = 1.0, device=None, tiles="cache"):
        self.lib = _lib.load()
        self.dim, self.grid, self.max_bodies = int(dim), int(grid), int(max_bodies)
        self.mode, self.extent, self.eps, self.g_newton = mode, float(extent), float(eps), float(g_newton)
        self.h = self.extent / self.grid
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("PMPlan needs a CUDA device")
        self._p = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.augur_pm_plan_create(C.byref(self._p), self.dim, self.grid, self.max_bodies,
                                               MODES[mode], self.extent, self.eps, self.g_newton)
        _lib.check(rc, "augur_pm_plan_create")
        # tiles: "cache" = the autotuner's measured shapes for this grid and body count when the
        # cache has them (periodic 3D), None = the library's defaults, or a dict of shapes
        if tiles == "cache" and self.dim == 3 and mode == "periodic":
            from . import autotune

            tiles = autotune.cached_tiles(self.grid, self.max_bodies)
        if isinstance(tiles, dict) and tiles:
            self.set_tiles(tiles)

    # ---- lifetime --------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_p", None) and self._p.value:
            with torch.cuda.device(self.device):
                torch.cuda.synchronize(self.device)
                self.lib.augur_pm_plan_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def workspace_bytes(self) -> int:
        return int(self.lib.augur_pm_plan_workspace_bytes(self._p))

    @property
    def tiles(self) -> dict:
        """The kernels' tile shapes (augur_pm_tiles as a dict)."""
        t = _lib.Tiles()
        _lib.check(self.lib.augur_pm_plan_get_tiles(self._p, C.byref(t)), "augur_pm_plan_get_tiles")
        return t.as_dict()

    def set_tiles(self, tiles: dict) -> None:
        """Apply tile shapes (keys of augur_pm_tiles; missing keys keep their value). Outputs do not
        depend on them. Synchronises the device when the deposit shape changes."""
        cur = self.tiles
        cur.update(tiles)
        with torch.cuda.device(self.device):
            rc = self.lib.augur_pm_plan_set_tiles(self._p, C.byref(_lib.Tiles.from_dict(cur)))
        _lib.check(rc, "augur_pm_plan_set_tiles")

    def bind_force_grid(self, grid4: torch.Tensor | None) -> None:
        """Use grid4 ((G, G, G, 4) float32 CUDA tensor, e.g. one slice of a batched grid) as the force
        grid of the run loop; None returns to the plan's own grid."""
        if grid4 is not None:
            _need(grid4, "grid4", shape=self.grid_shape + (4,), device=self.device)
        self._bound = grid4
        _lib.check(self.lib.augur_pm_plan_bind_force_grid(self._p, _ptr(grid4)), "augur_pm_plan_bind_force_grid")

    def set_kernel_mlp(self, params, ncol: int, extra=(), cell_units: bool = False, prior: bool = False,
                       split: bool = False, split_radius: float = 0.0, eps: float = 0.0, pad_ext: bool = False) -> None:
        """Isolated 2D plans: use the learned radial kernel of ScatterField.kernel_acc
        (scripts/scatter_field.py:263-289) in the Poisson solve. params: the kmlp's parameters
        flattened in order W1 (64 x ncol), b1, W2 (64 x 64), b2, W3 (1 x 64), b3 (fp32, any device);
        extra: the constant feature values after the two (three in cell units) distance features."""
        p = torch.as_tensor(params, dtype=torch.float32).reshape(-1).contiguous()
        if p.numel() != 64 * ncol + 64 * 64 + 3 * 64 + 1:
            raise ValueError(f"params must hold {64 * ncol + 64 * 64 + 3 * 64 + 1} values for ncol={ncol}")
        if p.is_cuda and p.device != self.device:
            raise ValueError(f"params are on {p.device}, the plan is on {self.device}")
        ex = (C.c_float * max(1, len(extra)))(*[float(e) for e in extra])
        flags = (1 if cell_units else 0) | (2 if prior else 0) | (4 if split else 0) | (8 if pad_ext else 0)
        self._kparams = p
        with torch.cuda.device(self.device):
            rc = self.lib.augur_pm_set_kernel_mlp(self._p, p.data_ptr(), int(ncol), ex, len(extra), flags,
                                                  float(split_radius), float(eps), _stream(self.device))
            if not p.is_cuda:
                torch.cuda.synchronize(self.device)  # the host copy is read asynchronously
        _lib.check(rc, "augur_pm_set_kernel_mlp")

    def pair_acc(self, pos, mass=None, mask=None, ppe: float = 2.0, knn: int = 16, params=None, ncol: int = 2,
                 extra=(), cell_units: bool = False, prior: bool = False, eps: float = 0.0) -> torch.Tensor:
        """Isolated 2D plans: the pair term of ScatterField.pp_acc (scripts/scatter_field.py:291-300,
        324-364, 500-521) -- the knn nearest bodies within ppe weighted by the ppmlp (params in the
        kmlp layout of set_kernel_mlp, or None for the prior alone) and the prior's near-field
        difference. ppe is the pair radius in length units (ScatterField.ppe())."""
        n = self._n(pos)
        mass, mask = self._mm(n, mass, mask)
        p = None
        if params is not None:
            p = torch.as_tensor(params, dtype=torch.float32).reshape(-1).contiguous()
            if p.numel() != 64 * ncol + 64 * 64 + 3 * 64 + 1:
                raise ValueError(f"params must hold {64 * ncol + 64 * 64 + 3 * 64 + 1} values for ncol={ncol}")
            p = p.to(self.device)
        ex = (C.c_float * max(1, len(extra)))(*[float(e) for e in extra])
        flags = (1 if cell_units else 0) | (2 if prior else 0)
        acc = torch.empty((n, 2), dtype=torch.float32, device=self.device)
        self._call("augur_pm_pair_acc", pos.data_ptr(), mass.data_ptr(), mask.data_ptr(), n, float(ppe), int(knn),
                   _ptr(p), int(ncol), ex, len(extra), flags, float(eps), acc.data_ptr())
        return acc

    def reset_kernel(self) -> None:
        """Back to the plan's softened -1/sqrt(d^2 + eps^2) kernel with zero-padded gradient."""
        self._call("augur_pm_reset_kernel")

    @property
    def last_launches(self) -> int:
        """Kernel launches issued by the last plan call."""
        return int(self.lib.augur_pm_last_launches(self._p))

    @property
    def grid_shape(self) -> tuple[int, ...]:
        return (self.grid,) * self.dim

    def _n(self, pos: torch.Tensor) -> int:
        _need(pos, "pos", device=self.device)
        if pos.dim() != 2 or pos.shape[1] != self.dim:
            raise ValueError(f"pos must be (N, {self.dim}), got {tuple(pos.shape)}")
        n = pos.shape[0]
        if n > self.max_bodies:
            raise ValueError(f"{n} bodies exceed the plan's max_bodies={self.max_bodies}")
        return n

    def _mm(self, n, mass, mask):
        if mass is None:
            mass = torch.ones(n, device=self.device)
        if mask is None:
            mask = torch.ones(n, device=self.device)
        return _need(mass, "mass", shape=(n,), device=self.device), _need(mask, "mask", shape=(n,), device=self.device)

    def _call(self, name: str, *args) -> None:
        with torch.cuda.device(self.device):
            rc = getattr(self.lib, name)(self._p, *args, _stream(self.device))
        _lib.check(rc, name)

    # ---- sub-ops (ScatterField building blocks) ------------------------------------------
    def cell_index(self, pos: torch.Tensor):
        """Bit-exact CIC base cell and fraction (ScatterField._corners, scripts/scatter_field.py:179-182)."""
        n = self._n(pos)
        i0 = torch.empty((n, self.dim), dtype=torch.int32, device=self.device)
        w = torch.empty((n, self.dim), dtype=torch.float32, device=self.device)
        self._call("augur_pm_cell_index", pos.data_ptr(), n, i0.data_ptr(), w.data_ptr())
        return i0, w

    def deposit(self, pos, mass=None, mask=None) -> torch.Tensor:
        """CIC mass density (mass channel of ScatterField.scatter, scripts/scatter_field.py:237-250)."""
        n = self._n(pos)
        mass, mask = self._mm(n, mass, mask)
        rho = torch.empty(self.grid_shape, dtype=torch.float32, device=self.device)
        self._call("augur_pm_deposit", pos.data_ptr(), mass.data_ptr(), mask.data_ptr(), n, rho.data_ptr())
        return rho

    def poisson(self, rho: torch.Tensor) -> torch.Tensor:
        """Force grid (..., 4) = (a_x, a_y, a_z, phi) from a density grid."""
        _need(rho, "rho", shape=self.grid_shape, device=self.device)
        out = torch.empty(self.grid_shape + (4,), dtype=torch.float32, device=self.device)
        self._call("augur_pm_poisson", rho.data_ptr(), out.data_ptr())
        return out

    def gather(self, force4: torch.Tensor, pos: torch.Tensor, mask=None):
        """CIC gather of a (..., 4) force grid (ScatterField.gather, scripts/scatter_field.py:252-261)."""
        n = self._n(pos)
        _need(force4, "force", shape=self.grid_shape + (4,), device=self.device)
        _, mask = self._mm(n, None, mask)
        acc = torch.empty((n, self.dim), dtype=torch.float32, device=self.device)
        phi = torch.empty((n,), dtype=torch.float32, device=self.device)
        self._call("augur_pm_gather", force4.data_ptr(), pos.data_ptr(), mask.data_ptr(), n, acc.data_ptr(),
                   phi.data_ptr())
        return acc, phi

    # ---- force / integrators --------------------------------------------------------------
    def force(self, pos, mass=None, mask=None, with_phi: bool = False):
        """Plain PM acceleration at the bodies (pm_acc, scripts/pm_baseline_force_error.py:68-76)."""
        n = self._n(pos)
        mass, mask = self._mm(n, mass, mask)
        acc = torch.empty((n, self.dim), dtype=torch.float32, device=self.device)
        phi = torch.empty((n,), dtype=torch.float32, device=self.device) if with_phi else None
        self._call("augur_pm_force", pos.data_ptr(), mass.data_ptr(), mask.data_ptr(), n, acc.data_ptr(), _ptr(phi))
        return (acc, phi) if with_phi else acc

    def step(self, pos, vel, acc, mass=None, mask=None, dt: float = 1e-3, have_acc: bool = True) -> None:
        """One velocity-Verlet step in place (ScatterField._step, scripts/scatter_field.py:677-688)."""
        n = self._n(pos)
        _need(vel, "vel", shape=pos.shape, device=self.device)
        _need(acc, "acc", shape=pos.shape, device=self.device)
        mass, mask = self._mm(n, mass, mask)
        self._call("augur_pm_step", pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), mass.data_ptr(),
                   mask.data_ptr(), n, float(dt), int(bool(have_acc)))

    def step_host(self, pos, vel, acc, mass=None, mask=None, dt: float = 1e-3, have_acc: bool = True) -> None:
        """``step`` on host tensors: pos, vel, acc are (N, D) float32 CPU tensors (pinned for the
        copies to overlap the kernels), updated in place once the plan's stream has finished;
        mass and mask are device tensors. Same results as ``step`` on device copies."""
        for t, name in ((pos, "pos"), (vel, "vel"), (acc, "acc")):
            if not isinstance(t, torch.Tensor) or t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
                raise ValueError(f"{name} must be a contiguous float32 CPU tensor")
            if t.dim() != 2 or t.shape[1] != self.dim or t.shape != pos.shape:
                raise ValueError(f"{name} must be (N, {self.dim}) like pos, got {tuple(t.shape)}")
        n = pos.shape[0]
        if n > self.max_bodies:
            raise ValueError(f"{n} bodies exceed the plan's max_bodies={self.max_bodies}")
        mass, mask = self._mm(n, mass, mask)
        self._call("augur_pm_step_host", pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), mass.data_ptr(),
                   mask.data_ptr(), n, float(dt), int(bool(have_acc)))

    def run(self, pos, vel, mass=None, mask=None, dt: float = 1e-3, nsteps: int = 1, want_acc: bool = False):
        """nsteps merged kick-drift-kick steps in place on the sorted device state."""
        n = self._n(pos)
        _need(vel, "vel", shape=pos.shape, device=self.device)
        mass, mask = self._mm(n, mass, mask)
        acc = torch.empty_like(pos) if want_acc else None
        self._call("augur_pm_run", pos.data_ptr(), vel.data_ptr(), mass.data_ptr(), mask.data_ptr(), n, float(dt),
                   int(nsteps), _ptr(acc))
        return acc

    def run_begin(self, pos, vel, mass=None, mask=None, dt: float = 1e-3) -> None:
        n = self._n(pos)
        _need(vel, "vel", shape=pos.shape, device=self.device)
        mass, mask = self._mm(n, mass, mask)
        self._keep = (mass, mask)
        self._call("augur_pm_run_begin", pos.data_ptr(), vel.data_ptr(), mass.data_ptr(), mask.data_ptr(), n,
                   float(dt))

    def run_steps(self, k: int) -> None:
        self._call("augur_pm_run_steps", int(k))

    # ---- run loop in pieces (the CNN-corrected step edits the force grid in between) ---------
    def run_load(self, pos, vel, mass=None, mask=None, dt: float = 1e-3) -> None:
        n = self._n(pos)
        _need(vel, "vel", shape=pos.shape, device=self.device)
        mass, mask = self._mm(n, mass, mask)
        self._keep = (mass, mask)
        self._call("augur_pm_run_load", pos.data_ptr(), vel.data_ptr(), mass.data_ptr(), mask.data_ptr(), n,
                   float(dt))

    def run_grid(self, rho_out: torch.Tensor | None = None, with_phi: bool = False) -> torch.Tensor:
        """Deposit + solve for the current state; returns the plan's force grid (G,)*3 + (4,) (a view
        of plan-owned memory, valid until the next grid call)."""
        if rho_out is not None:
            _need(rho_out, "rho_out", shape=self.grid_shape, device=self.device)
        self._call("augur_pm_run_grid", _ptr(rho_out), int(bool(with_phi)))
        return self.force_grid()

    def force_grid(self) -> torch.Tensor:
        addr = self.lib.augur_pm_force_grid(self._p)
        if not addr:
            raise RuntimeError("augur_pm_force_grid returned NULL")
        n = self.grid ** self.dim * 4
        holder = _DeviceBuffer(addr, n * 4, self.device)
        return torch.as_tensor(holder, device=self.device).view(self.grid_shape + (4,))

    def run_kick(self, kick: float, drift: bool, want_acc_like: torch.Tensor | None = None,
                 energy_out: torch.Tensor | None = None, esync: float = 0.0):
        """Gather + kick (+ drift). energy_out: device float64 (2,) <- (kinetic at v + esync a,
        potential), needs the preceding run_grid(with_phi=True)."""
        acc = torch.empty_like(want_acc_like) if want_acc_like is not None else None
        if energy_out is not None:
            _need(energy_out, "energy_out", torch.float64, shape=(2,), device=self.device)
        self._call("augur_pm_run_kick", float(kick), int(bool(drift)), _ptr(acc), _ptr(energy_out), float(esync))
        return acc

    def run_unload(self, pos, vel) -> None:
        self._call("augur_pm_run_unload", pos.data_ptr(), vel.data_ptr())

    STAGES = ("sort", "deposit_r2c", "fft_y_fwd", "fft_z_green", "fft_y_inv", "c2r", "gather_kd")

    def run_profile(self, k: int) -> dict:
        """Mean device ms per stage over k steps of an active run (CUDA events between stages)."""
        out = (C.c_float * len(self.STAGES))()
        with torch.cuda.device(self.device):
            rc = self.lib.augur_pm_run_profile(self._p, int(k), out, len(self.STAGES), _stream(self.device))
        _lib.check(rc, "augur_pm_run_profile")
        return dict(zip(self.STAGES, [float(x) for x in out]))

    def run_end(self, pos, vel, want_acc: bool = False):
        acc = torch.empty_like(pos) if want_acc else None
        self._call("augur_pm_run_end", pos.data_ptr(), vel.data_ptr(), _ptr(acc))
        return acc

    def check(self) -> None:
        """Synchronise and raise if a kernel flagged non-finite state."""
        self._call("augur_pm_check")


def direct_sum_fp64(targets: torch.Tensor, sources: torch.Tensor, mass: torch.Tensor | None = None,
                    eps: float = 0.5, box: float = 0.0, target_index: torch.Tensor | None = None) -> torch.Tensor:
    """FP64 softened direct sum on the GPU (exact_acc, scripts/scatter_scaling_ops.py:57-72).

    box > 0 makes the sum periodic (minimum image + tabulated Ewald correction)."""
    lib = _lib.load()
    dev = targets.device
    _need(targets, "targets", torch.float64)
    _need(sources, "sources", torch.float64, device=dev)
    d = targets.shape[1]
    if mass is not None:
        _need(mass, "mass", torch.float64, shape=(sources.shape[0],), device=dev)
    if target_index is not None:
        _need(target_index, "target_index", torch.int64, shape=(targets.shape[0],), device=dev)
    out = torch.empty_like(targets)
    with torch.cuda.device(dev):
        rc = lib.augur_direct_sum_fp64(targets.data_ptr(), _ptr(target_index), targets.shape[0], sources.data_ptr(),
                                       _ptr(mass), sources.shape[0], d, float(eps), float(box), out.data_ptr(),
                                       _stream(dev))
    _lib.check(rc, "augur_direct_sum_fp64")
    return out


def energy_fp64(vel: torch.Tensor, mass: torch.Tensor, mask: torch.Tensor, phi: torch.Tensor | None = None) -> dict:
    """Compensated reductions: kinetic energy, momentum, mass and PM potential energy."""
    lib = _lib.load()
    dev = vel.device
    _need(vel, "vel")
    n, d = vel.shape
    _need(mass, "mass", shape=(n,), device=dev)
    _need(mask, "mask", shape=(n,), device=dev)
    if phi is not None:
        _need(phi, "phi", shape=(n,), device=dev)
    out = torch.zeros(d + 3, dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        rc = lib.augur_energy_fp64(vel.data_ptr(), mass.data_ptr(), mask.data_ptr(), _ptr(phi), n, d, out.data_ptr(),
                                   _stream(dev))
    _lib.check(rc, "augur_energy_fp64")
    o = out.tolist()
    return {"ke": o[0], "momentum": o[1:1 + d], "mass": o[d + 1], "pe": o[d + 2]}
