/*
 * augur_pm.h — C ABI of the GB300 (sm_103a) particle-mesh gravity step.
 *
 * Every entry point takes plain device pointers, element counts and a CUDA stream
 * (passed as void*; NULL means the legacy default stream). Nothing here uses torch
 * types. Functions return 0 on success or a negative status (AUGUR_E*); the text of
 * a status comes from augur_status_string(). No entry point synchronises the device
 * unless its comment says so, and none traps on the device: device-side problems
 * (non-finite positions, grids too large for a launch) set a per-plan error word
 * that augur_pm_check() reads.
 *
 * Layouts follow the reference's ScatterField tensors (scripts/scatter_field.py):
 *   pos, vel  : (N, D) float32, contiguous (D = 2 or 3)
 *   mass, mask: (N,)   float32; mask in {0,1}; masked bodies deposit nothing and get
 *               zero force (scripts/scatter_field.py:238-241, :615)
 *   grids     : row-major [z][y][x] (3D) or [y][x] (2D) float32, x fastest
 * The grid covers [-extent/2, extent/2)^D (scripts/scatter_field.py:82-83, :179-182).
 *
 * Modes:
 *   AUGUR_MODE_PERIODIC          D=3 periodic box: phi_k = -4 pi G rho_k / k^2 (k=0 -> 0),
 *                                spectral gradient a_k = -i k phi_k (Nyquist -> 0).
 *   AUGUR_MODE_ISOLATED_SOFTENED D=2 isolated box, the reference's plain PM
 *                                (scripts/pm_baseline_force_error.py:68-76): 2G x 2G
 *                                zero-padded convolution with K = -1/sqrt(d^2+eps^2),
 *                                central-difference gradient (scripts/scatter_field.py:551-555).
 */
#ifndef AUGUR_PM_H
#define AUGUR_PM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AUGUR_OK          0
#define AUGUR_EINVAL    (-22)  /* bad shape, size, mode or pointer            */
#define AUGUR_ENOMEM    (-12)  /* device allocation failed                    */
#define AUGUR_ETIMEDOUT (-110) /* a device wait ran out of its budget         */
#define AUGUR_ERANGE    (-34)  /* a count or grid index outside what is supported */
#define AUGUR_EIO       (-5)   /* non-finite body state seen on the device    */
#define AUGUR_ECUDA     (-1000)/* CUDA runtime error (launch or copy)         */

#define AUGUR_MODE_PERIODIC          0
#define AUGUR_MODE_ISOLATED_SOFTENED 1

typedef struct augur_pm_plan augur_pm_plan;

/* Human-readable text of a status code (static storage). */
const char *augur_status_string(int status);

/* Library version, 0xMMmmpp. */
int augur_version(void);

/*
 * Plan: the grid geometry and all device workspace for up to max_bodies bodies.
 * Replaces the geometry held by ScatterField.__init__ (scripts/scatter_field.py:76-140)
 * and the workspace PyTorch allocated per call. extent is the box side; eps is the
 * softening of the isolated kernel (ignored by the periodic mode); g_newton scales
 * the periodic Green's function. The plan allocates its workspace with cudaMalloc on
 * the current device and owns it until augur_pm_plan_destroy().
 */
int augur_pm_plan_create(augur_pm_plan **out, int dim, int grid, int64_t max_bodies,
                         int mode, double extent, double eps, double g_newton);
int augur_pm_plan_destroy(augur_pm_plan *plan);
/* Bytes of device memory the plan holds. */
int64_t augur_pm_plan_workspace_bytes(const augur_pm_plan *plan);

/*
 * Tile shapes of the plan's kernels. They change the launch geometry only: every output
 * is bit-identical for any valid shape (the deposit sums in fixed point, the transforms
 * do the same arithmetic per row), so an autotuner may pick them by speed alone.
 * No counterpart in the reference, whose kernels are cuFFT's and torch's own.
 */
typedef struct augur_pm_tiles {
  int deposit_rows_y; /* y rows per deposit row block; divides grid */
  int deposit_rows_z; /* z planes per deposit row block; 3D: 1..15 dividing grid, 2D: 1 */
  int deposit_chunk;  /* minimum bodies per deposit work item, 1024 .. 2^19 */
  int green_tile_y;   /* y columns per z-transform + Green block: 8 or 16, divides grid */
  int c2r_rows;       /* x rows per C2R block: power of two <= 32 */
  int fft_rows;       /* rows per y-transform block: 1..256 */
  int deposit_aggregate; /* 1: warp-aggregate deposit atomics (cells dense in bodies), 0: plain */
} augur_pm_tiles;

int augur_pm_plan_get_tiles(const augur_pm_plan *plan, augur_pm_tiles *out);
/*
 * Validates the shapes against the grid and the device's shared memory (AUGUR_EINVAL if
 * one does not fit) and applies them. A new deposit shape re-sizes the deposit tables:
 * that synchronises the device, so call it outside stream capture, between runs.
 */
int augur_pm_plan_set_tiles(augur_pm_plan *plan, const augur_pm_tiles *tiles);

/*
 * Periodic 3D plans: use the caller's device buffer (grid^3 float4, 16-byte aligned) as
 * the force grid that run_grid writes and run_kick reads, so that several plans can fill
 * the slices of one batched (B, G, G, G, 4) grid that a network then edits in one launch;
 * NULL returns to the plan's own grid. The caller keeps the buffer alive while bound.
 * No counterpart in the reference (its batch shares one grid tensor, scatter_field.py:779-794).
 */
int augur_pm_plan_bind_force_grid(augur_pm_plan *plan, float *grid4);

/*
 * Learned kernel term of the isolated 2D plan: ScatterField._kernel_fft / kernel_acc
 * (scripts/scatter_field.py:263-289). Replaces the plan's kernel spectrum with rfft2 of K on
 * the 2G x 2G minimum-image lattice (distance r per lattice point), where
 *   K(r) = kmlp(features(r)),  kmlp = Linear(ncol, 64), GELU, Linear(64, 64), GELU, Linear(64, 1)
 * with torch's layouts and exact (erf) GELU; params: device or host fp32, W1 (64 x ncol), b1 (64),
 * W2 (64 x 64), b2 (64), W3 (64), b3 (1). features = [r, log(r + h)], or with
 * AUGUR_KERNEL_CELL_UNITS [r/h, log(r/h + 1), log(0.5/h)] (:141-151), followed by the n_extra
 * constant features `extra` (host array; the reference's log(eps/0.5) and dt features); ncol is
 * the total. AUGUR_KERNEL_PRIOR: K = -(1 + K)/sqrt(r^2 + eps^2); AUGUR_KERNEL_SPLIT:
 * K *= 1 - (1 - min(r/split_radius, 1)^2)^2; AUGUR_KERNEL_PAD_EXT: the gradient reads the
 * potential's wrapped neighbours (kpad = "ext", :286-288) instead of zero padding.
 * augur_pm_poisson / augur_pm_force then use this kernel; augur_pm_reset_kernel restores the
 * softened -1/sqrt(d^2 + eps^2) kernel with zero padding.
 */
#define AUGUR_KERNEL_CELL_UNITS 1
#define AUGUR_KERNEL_PRIOR      2
#define AUGUR_KERNEL_SPLIT      4
#define AUGUR_KERNEL_PAD_EXT    8
int augur_pm_set_kernel_mlp(augur_pm_plan *plan, const float *params, int ncol, const float *extra,
                            int n_extra, int flags, double split_radius, double eps, void *stream);
int augur_pm_reset_kernel(augur_pm_plan *plan, void *stream);

/*
 * Pair term of the isolated 2D plan: ScatterField.pp_acc / pp_acc_cell / _pair_w
 * (scripts/scatter_field.py:291-300, 302-311, 324-364, 500-521). Bodies with mask > 0 are
 * sorted by cells of side ppe (clamped into ceil(extent/ppe)^2 cells, as _cell_keys); for every
 * such body the knn (1..32) nearest other such bodies in the 3 x 3 cells around its own, with
 * r = sqrt(|d|^2 + 1e-8), give
 *   acc_out_i = sum_j w(r) m_j mask_j d / r,   w = g(r) (1 - u)^2 (+ prior),   u = min(r/ppe, 1)^2,
 * g = ppmlp(features(r)) in the kmlp layout of augur_pm_set_kernel_mlp (params NULL: g = 0;
 * its 64 x 64 layer runs on the tensor cores as three BF16 products of a hi + lo split, ~2^-16
 * relative, and its GELUs use erfc from Abramowitz & Stegun 7.1.26, |erf error| <= 1.5e-7),
 * features [r, log(r + 0.05)], or with AUGUR_KERNEL_CELL_UNITS [r/h, log(r/h + 0.1), log(0.5/h)]
 * (h = extent/grid), then the n_extra constants; AUGUR_KERNEL_PRIOR adds
 * r/q^3 - a_mesh, q = sqrt(r^2 + eps^2), a_mesh = -4 (1 - u) r / (ppe^2 q) + (1 - (1 - u)^2) r / q^3.
 * Bodies with mask <= 0 get 0. The weight is exactly 0 once r/ppe rounds to 1, so only the knn
 * nearest within ppe count, as in every mode of the reference; the search runs on cells of side
 * ppe/4 (coarser when that needs more than 2048 a side) and ranks candidates by
 * (|d|^2 + 1e-8, index), so the result does not depend on the order of the bodies. The first call
 * (and one that needs more cells or a larger knn than before) allocates scratch: make it before
 * any stream capture. pos (N, 2), mass, mask (N,), acc_out (N, 2): device float32.
 */
int augur_pm_pair_acc(augur_pm_plan *plan, const float *pos, const float *mass, const float *mask,
                      int64_t n, double ppe, int knn, const float *params, int ncol,
                      const float *extra, int n_extra, int flags, double eps, float *acc_out,
                      void *stream);

/*
 * CIC base cell and fraction, bit-exact with ScatterField._corners
 * (scripts/scatter_field.py:179-182): u = (x + extent/2) / h - 0.5 in IEEE float32
 * (round-to-nearest, true division by float32(h)), i0 = floor(u), w = u - i0.
 * i0_out: (N, D) int32 (not wrapped), w_out: (N, D) float32.
 */
int augur_pm_cell_index(augur_pm_plan *plan, const float *pos, int64_t n,
                        int32_t *i0_out, float *w_out, void *stream);

/*
 * CIC mass deposit rho = sum m*mask*w / h^D, the mass channel of ScatterField.scatter
 * (scripts/scatter_field.py:237-250). Deterministic: contributions are accumulated in
 * 64-bit fixed point in shared memory after a counting sort by grid row, so the
 * result does not depend on body order or on scheduling. Periodic mode wraps corner
 * indices mod G; isolated mode drops out-of-grid corners (:208). rho_out: G^D floats.
 */
int augur_pm_deposit(augur_pm_plan *plan, const float *pos, const float *mass,
                     const float *mask, int64_t n, float *rho_out, void *stream);

/*
 * Grid force from a density grid: the FFT Poisson solve and gradient of
 * pm_acc (scripts/pm_baseline_force_error.py:69-75) for the isolated mode, the
 * periodic Green's function + spectral gradient for the periodic mode.
 * force_out: G^D cells x 4 floats (a_x, a_y, a_z, phi); in 2D the a_z lane is 0.
 */
int augur_pm_poisson(augur_pm_plan *plan, const float *rho, float *force_out, void *stream);

/*
 * CIC gather of a 4-lane force grid at body positions, ScatterField.gather
 * (scripts/scatter_field.py:252-261): acc_out (N, D) = sum_corners w * F[corner].
 * phi_out (N,) may be NULL.
 */
int augur_pm_gather(augur_pm_plan *plan, const float *force, const float *pos,
                    const float *mask, int64_t n, float *acc_out, float *phi_out,
                    void *stream);

/*
 * Plain PM force at the bodies: pm_acc (scripts/pm_baseline_force_error.py:68-76)
 * for the isolated mode, the periodic PM force otherwise. acc_out (N, D) is
 * multiplied by mask. phi_out (N,) (potential at the bodies) may be NULL.
 */
int augur_pm_force(augur_pm_plan *plan, const float *pos, const float *mass,
                   const float *mask, int64_t n, float *acc_out, float *phi_out,
                   void *stream);

/*
 * One velocity-Verlet step, ScatterField._step with verlet=True
 * (scripts/scatter_field.py:677-688):
 *   pos += dt*vel + dt^2/2 * acc ; a_new = F(pos) ; vel += dt/2 * (acc + a_new) ; acc = a_new
 * pos, vel, acc are updated in place. If have_acc is 0, acc is first set to F(pos)
 * (the reference's a_prev is None branch). Periodic mode wraps positions into the box.
 */
int augur_pm_step(augur_pm_plan *plan, float *pos, float *vel, float *acc,
                  const float *mass, const float *mask, int64_t n, float dt,
                  int have_acc, void *stream);

/*
 * augur_pm_step on the caller's HOST arrays: pos, vel, acc (N, D) in host memory (page-locked,
 * e.g. cudaHostAlloc, for the copies to run asynchronously and overlap; pageable memory works but
 * each copy then blocks), updated in place when the stream reaches the end of the call; mass and
 * mask (N,) are device pointers. Same results as copying the arrays to the device, calling
 * augur_pm_step and copying them back. With have_acc set, the bodies move in chunks: a chunk's
 * drift and row keys start as soon as its copy has landed, the drifted positions go back while
 * the grid is solved, and the kicked velocities and new accelerations go back chunk by chunk
 * (two internal copy streams ordered against `stream` by events; the call's work, copies
 * included, is complete when `stream` reaches its end). The plan keeps 3 N D floats of device
 * staging from the first call. Replaces the host round trip around ScatterField._step
 * (scripts/scatter_field.py:677-688) with its arrays on the host.
 */
int augur_pm_step_host(augur_pm_plan *plan, float *pos, float *vel, float *acc,
                       const float *mass, const float *mask, int64_t n, float dt,
                       int have_acc, void *stream);

/*
 * nsteps leapfrog steps (kick-drift-kick, merged between steps as in Sim.tick,
 * scripts/scatter_bh_1b.py:123-146) with the body state kept sorted by grid row on the
 * device between steps; one force evaluation per step plus one at the start. The
 * positions and velocities are written back to pos/vel in the caller's order.
 * acc_out (N, D) receives the force at the final positions and may be NULL.
 * Periodic mode only.
 */
int augur_pm_run(augur_pm_plan *plan, float *pos, float *vel, const float *mass,
                 const float *mask, int64_t n, float dt, int nsteps, float *acc_out,
                 void *stream);

/*
 * Split form of augur_pm_run, for callers that time or graph-capture single steps:
 * run_begin loads and sorts the bodies and applies the opening half kick; run_steps
 * advances k merged kick-drift steps (no host synchronisation, capture-safe; every step
 * swaps the plan's two body buffers, so a captured graph replays correctly when it holds
 * an even number of steps);
 * run_end applies the closing half kick and writes pos/vel (and acc_out if not NULL)
 * back in the caller's order.
 */
int augur_pm_run_begin(augur_pm_plan *plan, const float *pos, const float *vel,
                       const float *mass, const float *mask, int64_t n, float dt,
                       void *stream);
int augur_pm_run_steps(augur_pm_plan *plan, int k, void *stream);

/*
 * Batch of scenes stepped together: every plan (periodic, after augur_pm_run_begin, each with
 * its own body count and grid) keeps its state, and augur_pm_batch_run_steps advances all of
 * them by k merged steps with one launch per stage for the whole batch (11 launches per step:
 * re-sort scans and scatter, deposit planning and deposit + x transform, y transform, z
 * transform with the Green's function, inverse y transforms, x C2R, gather + kick-drift); each
 * launch's blocks are dealt to the scenes by a table of block offsets, and every scene computes
 * exactly what its own augur_pm_run_steps would, bit for bit. Replaces the reference's padded
 * (B, Nmax, D) batch with one grid per batch (to_tensors, scripts/scatter_field.py:779-794);
 * scenes here keep uneven body counts and grids. The plans must share the z-transform tile
 * (green_tile_y) and the deposit variant (deposit_aggregate); their tile shapes, force-grid
 * bindings and body counts are read at creation, so a batch is created again after any of them
 * changes. augur_pm_run_end (or run_unload) of each plan ends the run as usual. create allocates
 * the block tables (device memory) and synchronises the device; run_steps does not.
 */
typedef struct augur_pm_batch augur_pm_batch;
int augur_pm_batch_create(augur_pm_batch **out, augur_pm_plan *const *plans, int nplans);
int augur_pm_batch_run_steps(augur_pm_batch *batch, int k, void *stream);
int augur_pm_batch_size(const augur_pm_batch *batch);
int augur_pm_batch_destroy(augur_pm_batch *batch);
int augur_pm_run_end(augur_pm_plan *plan, float *pos, float *vel, float *acc_out,
                     void *stream);

/*
 * Run loop in pieces, for callers that modify the force grid between the Poisson solve
 * and the gather (the CNN-corrected step adds its correction field there):
 *   run_load   sort the caller's bodies into the device state (no force yet)
 *   run_grid   re-sort if a kick moved the bodies, deposit (density also written to
 *              rho_out when not NULL), FFT solve; with_phi = 1 fills the potential lane
 *   force_grid the plan's float4 force grid (G^3 cells: a_x, a_y, a_z, phi), device memory
 *   run_kick   gather the grid at the bodies, v += kick * a; drift = 1 also moves the
 *              bodies x += dt * v (wrapped) and prepares the next sort; acc_out as run_end.
 *              energy_out (device, 2 doubles, may be NULL; needs a with_phi grid) receives
 *              sum m |v + esync a|^2 / 2 and sum m phi / 2 over the bodies (fixed-order sums):
 *              esync = dt/2 gives the energy at the synchronised time of a merged step
 *   run_unload write positions and velocities back in the caller's order
 * A leapfrog step is run_grid + run_kick(dt, 1); the opening and closing half kicks use
 * kick = dt/2 (drift 1 and 0). Replaces the body of Sim.tick (scripts/scatter_bh_1b.py:133-138).
 */
int augur_pm_run_load(augur_pm_plan *plan, const float *pos, const float *vel, const float *mass,
                      const float *mask, int64_t n, float dt, void *stream);
int augur_pm_run_grid(augur_pm_plan *plan, float *rho_out, int with_phi, void *stream);
float *augur_pm_force_grid(augur_pm_plan *plan);
int augur_pm_run_kick(augur_pm_plan *plan, float kick, int drift, float *acc_out, double *energy_out,
                      float esync, void *stream);
int augur_pm_run_unload(augur_pm_plan *plan, float *pos, float *vel, void *stream);

/*
 * Measurement aid: k merged steps like augur_pm_run_steps with a CUDA event recorded on
 * the stream between the stages of each step; synchronises after every step and writes
 * the mean device milliseconds per stage to stage_ms[0..AUGUR_PM_NSTAGE-1] in the order
 * sort (scan + scatter), deposit + x R2C, forward y FFT, z FFT + Green + gradient +
 * inverse z, inverse y FFT, x C2R, gather + kick-drift + keys. Requires an active run.
 */
#define AUGUR_PM_NSTAGE 7
int augur_pm_run_profile(augur_pm_plan *plan, int k, float *stage_ms, int nstage, void *stream);

/* Kernel launches issued by the last plan call (for launch accounting). */
int64_t augur_pm_last_launches(const augur_pm_plan *plan);

/*
 * Synchronise the stream, read and clear the plan's device error word. Returns
 * AUGUR_OK, AUGUR_EIO (non-finite body state) or AUGUR_ERANGE.
 */
int augur_pm_check(augur_pm_plan *plan, void *stream);

/*
 * FP64 softened direct sum, exact_acc (scripts/scatter_scaling_ops.py:57-72)
 * generalised to D=2,3: acc[t] = sum_j m_j (x_j - x_t) / (|x_j - x_t|^2 + eps^2)^1.5
 * with the self pair excluded (target index t_idx[t] is a source index, or -1 if the
 * target is not a source). targets (T, D) f64, sources (N, D) f64, mass (N,) f64 or
 * NULL for unit masses. acc_out (T, D) f64.
 * If box > 0 the sum is periodic (Ewald; box side = box, minimum image plus a tabulated
 * Ewald correction), else isolated. The Newtonian pair sum is FP64; the Ewald correction is read
 * from a 65^3 table (FP64 sums stored as fp32) and interpolated trilinearly in fp32, a part of the
 * force whose fp32 rounding moves the total by ~1e-8, below the table's interpolation error
 * (about 1e-6 relative RMS on 2048-body scenes).
 */
int augur_direct_sum_fp64(const double *targets, const int64_t *t_idx, int64_t t,
                          const double *sources, const double *mass, int64_t n,
                          int dim, double eps, double box, double *acc_out, void *stream);

/*
 * The isolated FP64 direct sum above (box = 0) without any device allocation, for callers
 * that cannot call cudaMalloc: code issuing work while a CUDA stream is being captured (where
 * cudaMalloc is not allowed), and processes whose device memory is already reserved by
 * another allocator (PyTorch's caching allocator keeps what it holds), where an extra
 * allocation can fail. It has no counterpart in the reference.
 * Its scratch is one static device array of 4 MiB (2^19 doubles) that every GPU loading
 * this library keeps until the process exits; t * dim must not exceed 2^19 (else
 * AUGUR_ERANGE). The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that call before any stream
 * capture. The address is kept for the life of the process: after cudaDeviceReset (or a
 * release and re-creation of the device's primary context) it is stale, so the entry point
 * must not be called again in that process. All calls share the array: calls whose kernels overlap on the GPU (for example
 * on two streams) race and give wrong results; serialise them on one stream. Results match
 * augur_direct_sum_fp64 up to the order of the per-chunk partial sums.
 */
int augur_direct_sum_fp64_noalloc(const double *targets, const int64_t *t_idx, int64_t t,
                                  const double *sources, const double *mass, int64_t n,
                                  int dim, double eps, double *acc_out, void *stream);

/*
 * Compensated FP64 reductions over bodies (scripts/scatter_field.py:759-769):
 * out[0] = kinetic energy sum m v^2 / 2, out[1..D] = momentum sum m v,
 * out[D+1] = mass sum, out[D+2] = PM potential energy sum m phi / 2 (phi may be NULL -> 0).
 * out must hold D+3 doubles (device memory).
 */
int augur_energy_fp64(const float *vel, const float *mass, const float *mask,
                      const float *phi, int64_t n, int dim, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* AUGUR_PM_H */
