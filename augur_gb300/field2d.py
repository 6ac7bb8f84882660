"""The reference's production 2D scatter-field model on the GPU, behind its call signature.

Reference: ScatterField(grid=128, extent=64, net="unet", dt=0.1, kernel=True, pp=2.0, split=True,
potential=True, verlet=True) -- the configuration of its browser port (web/scatter/weights.json) --
in scripts/scatter_field.py:
    force(pos, vel, mass, mask, field) -> (acc, field)           :561-615
    step(pos, vel, mass, mask, field)  -> (pos, vel, field, dv)  :668-688
    init_field(B, device)                                        :557-559
    load_state_dict(...) with its parameter names (ppmlp.*, kmlp.*, net.*)
One force evaluation per scene: three-channel CIC scatter, the learned radial kernel's
acceleration (FFT convolution on the isolated 2D plan), the 5-level U-Net on
[scatter, kernel acceleration, previous potential], minus the potential's gradient plus the
kernel acceleration gathered at the bodies, the k-nearest pair term, the momentum fix.
Every stage is a kernel of libaugur_gb300 (include/augur_field2d.h, include/augur_pm.h); this
module only sequences them and owns the buffers. Layouts are the reference's: pos/vel
(B, N, 2) float32, mass/mask (B, N), field (B, 1, G, G).
"""
from __future__ import annotations


import torch

from . import _lib
from .pm import PMPlan, _stream


def _ptr(t):
    return None if t is None else t.data_ptr()


class UNetScatterField:
    def __init__(self, grid: int = 128, extent: float = 64.0, dt: float = 0.1, width: int = 32, levels: int = 5,
                 pp: float = 2.0, knn: int = 16, split: bool = True, momfix: bool = True, in_scale: float = 1.0,
                 eps: float = 0.5, device=None, graph: bool = False, prior: bool = False, cu: bool = False,
                 kpad: str = "zero"):
        self.lib = _lib.load()
        self.grid, self.extent, self.h = int(grid), float(extent), float(extent) / int(grid)
        self.dt, self.width, self.levels = float(dt), int(width), int(levels)
        self.pp, self.knn, self.split, self.momfix = float(pp), int(knn), bool(split), bool(momfix)
        self.in_scale, self.eps = float(in_scale), float(eps)
        # variants: prior (kernel -(1 + K)/sqrt(r^2 + eps^2) and the pair prior) and cell units (cu:
        # features in units of h, ppe = pp h / 0.5), scripts/scatter_field.py:138-151, 263-300
        self.prior, self.cu = bool(prior), bool(cu)
        if kpad not in ("zero", "ext"):
            raise ValueError("kpad: 'zero' or 'ext'")
        self.kpad = kpad  # "ext": the kernel potential's central difference reads one cell beyond the grid
        self.ncol = 3 if self.cu else 2
        self.cf, self.cin = 1, 6  # potential field; inputs [m, m vx, m vy, k_x, k_y, field]
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if self.grid % (1 << self.levels):
            raise ValueError(f"grid {grid} is not divisible by 2^{levels}")
        self.n_net = int(self.lib.augur_unet2d_param_count(self.cin, self.cf, self.width, self.levels))
        self.plan: PMPlan | None = None
        self.net = self.kparams = self.pparams = None
        G, dev = self.grid, self.device
        self._ws = torch.empty(int(self.lib.augur_field2d_scatter_work_bytes(G)), dtype=torch.uint8, device=dev)
        self._wf = torch.empty(int(self.lib.augur_field2d_finish_work_bytes()), dtype=torch.uint8, device=dev)
        self._batch = 0
        self._buffers(1)
        # graph=True: Verlet steps with a previous acceleration are captured once per input shape
        # in a CUDA graph and replayed (the reference's "graph" option, scripts/scatter_field.py:567-589)
        self.graph = bool(graph)
        self._graphs: dict = {}

    def _buffers(self, B: int) -> None:
        """Per-batch buffers: input stacks (B, 6, G, G), acceleration grids (B, G, G, 4), U-Net work."""
        if B <= self._batch:
            return
        G, dev = self.grid, self.device
        self._x = torch.zeros((B, self.cin, G, G), device=dev)
        self._f4a = torch.empty((B, G, G, 4), device=dev)
        self._wu_bytes = int(self.lib.augur_unet2d_work_bytes(G, self.width, self.levels, B))
        self._wu = torch.empty(self._wu_bytes, dtype=torch.uint8, device=dev)
        self._batch = B

    # ---- parameters ------------------------------------------------------------------------
    def ppe(self) -> float:
        return self.pp * self.h / 0.5 if self.cu else self.pp

    def load_state_dict(self, sd: dict) -> None:
        """Parameters under the reference's names (ppmlp.*, kmlp.*, net.*), any float dtype/device."""
        t = {k: torch.as_tensor(v).to(self.device, torch.float32).reshape(-1) for k, v in sd.items()}

        def mlp(prefix):
            return torch.cat([t[f"{prefix}.{i}.{w}"] for i in (0, 2, 4) for w in ("weight", "bias")]).contiguous()

        self.pparams = mlp("ppmlp") if self.pp > 0 else None
        self.kparams = mlp("kmlp")
        names = ["net.inp.weight", "net.inp.bias"]
        for blk in [f"enc.{l}" for l in range(self.levels + 1)] + [f"dec.{l}" for l in range(self.levels)]:
            names += [f"net.{blk}.{i}.{w}" for i in (0, 2) for w in ("weight", "bias")]
        names += ["net.out.weight", "net.out.bias"]
        net = torch.cat([t[k] for k in names]).contiguous()
        if net.numel() != self.n_net:
            raise ValueError(f"U-Net parameters: {net.numel()} values, expected {self.n_net}")
        self.net = torch.empty(int(self.lib.augur_unet2d_prepared_count(self.cin, self.cf, self.width, self.levels)),
                               device=self.device)
        self._call("augur_unet2d_prepare", net.data_ptr(), self.cin, self.cf, self.width, self.levels,
                   self.net.data_ptr())
        torch.cuda.synchronize(self.device)
        self._plan(1)

    def _plan(self, n: int) -> PMPlan:
        if self.plan is None or self.plan.max_bodies < n:
            if self.plan is not None:
                self.plan.close()
            self.plan = PMPlan(2, self.grid, max(int(n), 1), "isolated", self.extent, eps=self.eps, device=self.device)
            if self.kparams is not None:
                self.plan.set_kernel_mlp(self.kparams, self.ncol, cell_units=self.cu, prior=self.prior,
                                         split=self.split, split_radius=self.ppe(), eps=self.eps,
                                         pad_ext=self.kpad == "ext")
        return self.plan

    def close(self) -> None:
        if self.plan is not None:
            self.plan.close()
            self.plan = None

    # ---- reference interface ---------------------------------------------------------------
    def init_field(self, B: int, device=None, dtype=torch.float32):
        return (torch.zeros(B, self.cf, self.grid, self.grid, device=device or self.device, dtype=dtype), None)

    def _call(self, name, *args):
        with torch.cuda.device(self.device):
            rc = getattr(self.lib, name)(*args, _stream(self.device))
        _lib.check(rc, name)

    def scatter(self, pos, vel, mass, mask):
        """(B, 3, G, G): [m, m vx, m vy] * in_scale / h^2 (ScatterField.scatter, :237-250)."""
        B, N = pos.shape[:2]
        out = torch.empty((B, 3, self.grid, self.grid), device=self.device)
        for b in range(B):
            self._call("augur_field2d_scatter", pos[b].data_ptr(), vel[b].data_ptr(), mass[b].data_ptr(),
                       mask[b].data_ptr(), N, self.grid, self.extent, self.in_scale, out[b].data_ptr(),
                       self._ws.data_ptr())
        return out

    def unet(self, x: torch.Tensor) -> torch.Tensor:
        """The grid net alone: (B, 6, G, G) -> (B, 1, G, G), all scenes in the same launches."""
        x = x.to(self.device, torch.float32).contiguous()
        B = x.shape[0]
        self._buffers(B)
        y = torch.empty((B, self.cf, self.grid, self.grid), device=self.device)
        self._call("augur_unet2d_forward", self.net.data_ptr(), self.cin, self.cf, self.width, self.levels,
                   self.grid, B, x.data_ptr(), y.data_ptr(), self._wu.data_ptr(), self._wu_bytes)
        return y

    def _forces(self, pos, vel, mass, mask, field, acc_out, field_out):
        """One force evaluation of B scenes: per-scene scatter and kernel term, one U-Net call for
        the batch, per-scene gradient, gather, pair term and momentum fix."""
        B, n = pos.shape[:2]
        plan = self._plan(n)
        self._buffers(B)
        x, G = self._x, self.grid
        f4k = []
        for b in range(B):
            self._call("augur_field2d_scatter", pos[b].data_ptr(), vel[b].data_ptr(), mass[b].data_ptr(),
                       mask[b].data_ptr(), n, G, self.extent, self.in_scale, x[b].data_ptr(), self._ws.data_ptr())
            f4k.append(plan.poisson(x[b, 0]))  # the learned kernel's acceleration (kernel_acc)
            self._call("augur_field2d_inputs", f4k[b].data_ptr(), field[b].data_ptr(), self.cf, G, x[b].data_ptr())
        self._call("augur_unet2d_forward", self.net.data_ptr(), self.cin, self.cf, self.width, self.levels, G, B,
                   x.data_ptr(), field_out.data_ptr(), self._wu.data_ptr(), self._wu_bytes)
        for b in range(B):
            self._call("augur_field2d_accel", field_out[b].data_ptr(), f4k[b].data_ptr(), G, self.h,
                       self._f4a[b].data_ptr())
            a_grid, _ = plan.gather(self._f4a[b], pos[b])
            a_pair = None
            if self.pparams is not None:
                a_pair = plan.pair_acc(pos[b], mass[b], mask[b], ppe=self.ppe(), knn=self.knn, params=self.pparams,
                                       ncol=self.ncol, cell_units=self.cu, prior=self.prior, eps=self.eps)
            self._call("augur_field2d_finish", a_grid.data_ptr(), _ptr(a_pair), mass[b].data_ptr(),
                       mask[b].data_ptr(), n, int(self.momfix), acc_out[b].data_ptr(), self._wf.data_ptr())

    def _check(self, pos, vel, mass, mask):
        if self.net is None:
            raise RuntimeError("load_state_dict first")
        for name, t in (("pos", pos), ("vel", vel), ("mass", mass), ("mask", mask)):
            if not (t.is_cuda and t.device == self.device and t.dtype == torch.float32 and t.is_contiguous()):
                raise ValueError(f"{name} must be a contiguous float32 tensor on {self.device}")
        if pos.dim() != 3 or pos.shape[2] != 2 or vel.shape != pos.shape or mass.shape != pos.shape[:2] \
                or mask.shape != pos.shape[:2]:
            raise ValueError("pos/vel must be (B, N, 2) and mass/mask (B, N)")

    def force(self, pos, vel, mass, mask, field):
        """(acc (B, N, 2), new field (B, 1, G, G)) -- ScatterField.force (:561-615)."""
        self._check(pos, vel, mass, mask)
        B = pos.shape[0]
        acc = torch.empty_like(pos)
        out = torch.empty((B, self.cf, self.grid, self.grid), device=self.device)
        field = field.to(self.device, torch.float32).contiguous()
        self._forces(pos, vel, mass, mask, field, acc, out)
        return acc, out

    def step(self, pos, vel, mass, mask, field):
        """One velocity-Verlet step, ScatterField._step (:677-688): field = (potential, a_prev)."""
        self._check(pos, vel, mass, mask)
        if self.graph and field[1] is not None and not torch.cuda.is_current_stream_capturing():
            return self._graphed_step(pos, vel, mass, mask, field)
        return self._step(pos, vel, mass, mask, field)

    def _graphed_step(self, pos, vel, mass, mask, field):
        f, a_prev = field
        args = (pos, vel, mass, mask, f.to(self.device, torch.float32).contiguous(), a_prev.contiguous())
        key = tuple((tuple(t.shape), t.dtype) for t in args)
        ent = self._graphs.get(key)
        if ent is None:
            static = [t.clone() for t in args]
            cur = torch.cuda.current_stream(self.device)
            side = torch.cuda.Stream(self.device)
            side.wait_stream(cur)
            with torch.cuda.stream(side):  # warm-up: plan growth, scratch allocation, attribute opt-ins
                for _ in range(2):
                    self._step(*static[:4], (static[4], static[5]))
            cur.wait_stream(side)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                out = self._step(*static[:4], (static[4], static[5]))
            ent = self._graphs[key] = (g, static, out)
        g, static, out = ent
        for dst, src in zip(static, args):
            dst.copy_(src)
        g.replay()
        p, v, (fo, a), dv = out
        return p.clone(), v.clone(), (fo.clone(), a.clone()), dv.clone()

    def _step(self, pos, vel, mass, mask, field):
        f, a_prev = field
        if a_prev is None:
            a_prev, f = self.force(pos, vel, mass, mask, f)
        n = pos.numel() // 2
        pos_new, vel_pred = torch.empty_like(pos), torch.empty_like(vel)
        self._call("augur_field2d_drift", pos.data_ptr(), vel.data_ptr(), a_prev.data_ptr(), n, self.dt,
                   pos_new.data_ptr(), vel_pred.data_ptr())
        a_new, f = self.force(pos_new, vel_pred, mass, mask, f)
        vel_new, dv = torch.empty_like(vel), torch.empty_like(vel)
        self._call("augur_field2d_kick", vel.data_ptr(), a_prev.data_ptr(), a_new.data_ptr(), n, self.dt,
                   vel_new.data_ptr(), dv.data_ptr())
        return pos_new, vel_new, (f, a_new), dv


class ChunkedTick2D:
    """The reference's large-N tick, Sim (scripts/scatter_bh_1b.py:107-146), on a loaded
    UNetScatterField: unit-mass bodies whose (N, 2) position and momentum tensors are stored in
    float32, float16 or bfloat16 and updated in place. State is kept half-kicked (M = p + dt/2 a):
    tick = drift with the relativistic speed fused into the scatter, grid force (learned kernel,
    U-Net with the recurrent potential, -grad + kernel acceleration), the density-weighted mean
    acceleration from the grid, gather fused with the kick. The reference loops over chunks of
    bodies to bound its fp32 temporaries; here every kernel widens one body at a time, so there
    are no temporaries and no chunking."""

    DTYPES = {torch.float32: 0, torch.float16: 1, torch.bfloat16: 2}

    def __init__(self, model: UNetScatterField, n: int, c: float = 10.0, dt: float = 0.1,
                 pos_dtype=torch.float16, mom_dtype=torch.float16, mom_scale: float = 1.0):
        if model.net is None:
            raise RuntimeError("load the model's weights first")
        if pos_dtype not in self.DTYPES or mom_dtype not in self.DTYPES:
            raise ValueError("state dtypes: float32, float16 or bfloat16")
        self.m, self.n, self.c, self.dt, self.ms = model, int(n), float(c), float(dt), float(mom_scale)
        self.pd, self.md = pos_dtype, mom_dtype
        G, dev = model.grid, model.device
        self.field = torch.zeros(model.cf, G, G, device=dev)
        self.x = torch.zeros(model.cin, G, G, device=dev)
        self.wu_bytes = int(model.lib.augur_unet2d_work_bytes(G, model.width, model.levels, 1))
        self.wu = torch.empty(self.wu_bytes, dtype=torch.uint8, device=dev)
        self.f4a = torch.empty(G, G, 4, device=dev)
        self.abar = torch.zeros(2, device=dev)
        self.work = torch.empty(int(model.lib.augur_tick2d_work_bytes(G)), dtype=torch.uint8, device=dev)

    def _check(self, pos, mom):
        for name, t, dt in (("pos", pos, self.pd), ("mom", mom, self.md)):
            if t.dtype != dt or t.shape != (self.n, 2) or not t.is_contiguous() or t.device != self.m.device:
                raise ValueError(f"{name} must be a contiguous ({self.n}, 2) {dt} tensor on {self.m.device}")

    def _scatter(self, pos, mom, drift: bool):
        m = self.m
        m._call("augur_tick2d_drift_scatter", pos.data_ptr(), mom.data_ptr(), self.n, self.DTYPES[self.pd],
                self.DTYPES[self.md], self.ms, self.c, self.dt, int(bool(drift)), m.grid, m.extent, m.in_scale,
                self.x.data_ptr(), self.work.data_ptr())

    def scatter_pass(self, pos, mom, drift: bool) -> torch.Tensor:
        """Sim.scatter_pass: (3, G, G) scatter of [1, vx, vy]; with drift=True pos is drifted first."""
        self._check(pos, mom)
        self._scatter(pos, mom, drift)
        if drift:
            self.m._call("augur_tick2d_drift", pos.data_ptr(), mom.data_ptr(), self.n, self.DTYPES[self.pd],
                         self.DTYPES[self.md], self.ms, self.c, self.dt)
        return self.x[:3]

    def grid_force(self):
        """Sim.grid_force on the current scatter: (acceleration grid (G, G, 4), abar (2,))."""
        m, G = self.m, self.m.grid
        f4k = m.plan.poisson(self.x[0])
        m._call("augur_field2d_inputs", f4k.data_ptr(), self.field.data_ptr(), m.cf, G, self.x.data_ptr())
        m._call("augur_unet2d_forward", m.net.data_ptr(), m.cin, m.cf, m.width, m.levels, G, 1, self.x.data_ptr(),
                self.field.data_ptr(), self.wu.data_ptr(), self.wu_bytes)
        m._call("augur_field2d_accel", self.field.data_ptr(), f4k.data_ptr(), G, m.h, self.f4a.data_ptr())
        m._call("augur_tick2d_mean_acc", self.f4a.data_ptr(), self.x.data_ptr(), G, m.h * m.h / m.in_scale, self.n,
                self.abar.data_ptr(), self.work.data_ptr())
        return self.f4a, self.abar

    def _kick(self, pos, mom, kick, drift: bool):
        m = self.m
        m._call("augur_tick2d_gather_kick", self.f4a.data_ptr(), pos.data_ptr(), mom.data_ptr(), self.n,
                self.DTYPES[self.pd], self.DTYPES[self.md], self.ms, kick, self.abar.data_ptr(), m.grid, m.extent,
                int(bool(drift)), self.c, self.dt)

    def tick(self, pos, mom) -> None:
        """Sim.tick: drift, scatter, grid force, mom += dt (a - abar) / ms, in place. The scatter
        reads the drifted positions without storing them; the gather-kick stores them."""
        self._check(pos, mom)
        self._scatter(pos, mom, True)
        self.grid_force()
        self._kick(pos, mom, self.dt, True)

    def init_kick(self, pos, mom) -> None:
        """Sim.init_kick: the first half kick, mom += dt/2 (a - abar) / ms."""
        self._check(pos, mom)
        self._scatter(pos, mom, False)
        self.grid_force()
        self._kick(pos, mom, 0.5 * self.dt, False)
