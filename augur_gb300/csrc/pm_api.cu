// pm_api.cu — C ABI of the PM gravity step: plan, workspace and kernel orchestration.
//
// One plan = one grid geometry + the device workspace for up to max_bodies bodies.
// Every call enqueues kernels on the caller's stream and returns without a host
// synchronisation (augur_pm_check is the exception), so a step can be captured in a
// CUDA graph by the caller.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "pm_kernels.cuh"

using namespace augur;

// Chunks of caller bodies in the host-buffer step: the copies of one chunk overlap the kernels of
// the chunks before it (3M bodies on GB300: 1.69 ms per step with 2 chunks, 1.76 with 1 and with
// 4, 1.84 with 8, 1.94 with 16; each chunk's copies and launches carry a fixed cost).
constexpr int HS_CHUNKS = 2;

struct augur_pm_plan {
  int dim, G, mode;
  double extent, eps, gnewton;
  int64_t max_n;
  GridParams gp;
  int nrow, ntiles;
  int L, M, Lt;  // transform length (G periodic, 2G isolated), half length, twiddle table length
  FftShape sh_M, sh_L;
  int dep_RY, dep_RZ, green_TY, c2r_RB, rows_RB, r2c_RB;
  int dep_chunk_min;  // minimum bodies per deposit work item
  int dep_agg;        // warp-aggregated deposit atomics (dense cells)
  size_t smem_dep, smem_green, smem_c2r, smem_rows, smem_r2c;
  size_t smem_max;  // the device's opt-in dynamic shared memory per block
  float2 *tw;
  float4 *pos4[2], *vel4[2];
  int cur;
  uint32_t *key, *slot, *row_count, *row_start, *tile_sum, *tile_off;
  unsigned *d_err, *d_mmax;
  // deposit work items (row blocks split into body chunks) and partial fixed-point tiles
  int nblk;
  uint32_t *dep_nch, *dep_item_off, *dep_slot_off, *dep_counters, *dep_item_blk;
  uint4 *dep_seg_tab;
  size_t dep_items_max;
  unsigned long long *dep_scratch;
  size_t dep_slots;
  size_t dep_bytes;  // device bytes of the deposit tables (re-sized with the tile shape)
  int64_t cur_n;  // bodies in the sorted state
  float2 *spec, *spec3, *khat;
  float4 *F4;      // force grid in use: F4_own, or a caller's buffer bound by augur_pm_plan_bind_force_grid
  float4 *F4_own;
  float *real_tmp, *phi2d, *rho2d;
  float *phi_ext;  // isolated, kpad = "ext": potential at rows/columns -1 .. G, (G+2)^2
  float *kparams;  // learned kernel MLP parameters (device copy)
  int kpad_ext;
  // pair term: cell key and rank per body, the bodies in cell order, the two-level cell scan
  uint32_t *pair_key, *pair_rank, *pair_cnt, *pair_start, *pair_tsum, *pair_toff;
  float4 *pair_sorted;
  uint32_t *pair_nbj;  // neighbour lists, max_n x pair_kp
  float *pair_nbq;
  int pair_kp;
  size_t pair_cells_cap;
  float *pair_params;
  int64_t run_n;
  float run_dt;
  int run_active;
  int ncomp_last;  // components of the last force grid (3, or 4 with the potential)
  double *epart;   // energy tap partials
  unsigned epart_n;
  int64_t launches;
  size_t bytes;
  // host-buffer step (augur_pm_step_host): device copies of the caller's pos, vel, acc, two copy
  // streams, and the events that order chunks between them and the caller's stream
  float *hs_buf;
  cudaStream_t hs_in, hs_out;
  cudaEvent_t hs_ev[3 * HS_CHUNKS + 2];
};

namespace {

int cuda_status(cudaError_t e) { return e == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA; }

// scratch buffers of the z transform in fft_z_green_kernel (two stages ping-pong through one)
int green_nbuf(int G) { return fft_nstages(G) > 2 ? 2 : 1; }

#define AUGUR_LAUNCH_CHECK(plan)                      \
  do {                                                \
    (plan)->launches++;                               \
    cudaError_t _e = cudaGetLastError();              \
    if (_e != cudaSuccess) {                          \
      fprintf(stderr, "augur: launch failed: %s (%s:%d)\n", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return AUGUR_ECUDA;                             \
    }                                                 \
  } while (0)

bool factor(int L, FftShape &sh) {
  sh.L = L;
  sh.nstages = 0;
  int r = L;
  while (r % 3 == 0) {
    sh.radix[sh.nstages++] = 3;
    r /= 3;
  }
  int e = 0;
  while (r % 2 == 0) {
    r /= 2;
    ++e;
  }
  if (r != 1) return false;
  if (e == 1) {
    sh.radix[sh.nstages++] = 2;
  } else if (e > 1) {
    int q = e / 3, rem = e % 3;
    if (rem == 1) {
      q -= 1;
      sh.radix[sh.nstages++] = 4;
      sh.radix[sh.nstages++] = 4;
    } else if (rem == 2) {
      sh.radix[sh.nstages++] = 4;
    }
    for (int i = 0; i < q; ++i) sh.radix[sh.nstages++] = 8;
  }
  return sh.nstages <= 12;
}

template <typename T>
int dalloc(augur_pm_plan *p, T **ptr, size_t count) {
  *ptr = nullptr;
  if (count == 0) return AUGUR_OK;
  size_t b = count * sizeof(T);
  if (cudaMalloc((void **)ptr, b) != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    return AUGUR_ENOMEM;
  }
  p->bytes += b;
  return AUGUR_OK;
}

unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

constexpr int DEP_CHUNK_MIN = 2048;
constexpr int DEP_THREADS = 256;
// bodies per deposit work item: at least the plan's minimum, ~1024 chunks for large inputs, and
// at most DEP_ITEM_MAX (the bound under which a work item's 32-bit shared sums cannot overflow),
// so that any n < 2^31 takes at most DEP_NCH_MAX chunks
constexpr int64_t DEP_NCH_MAX = 4096;
uint32_t dep_chunk(const augur_pm_plan *p, int64_t n) {
  int64_t c = (n + 1023) / 1024;
  return (uint32_t)std::min<int64_t>(DEP_ITEM_MAX, std::max<int64_t>(p->dep_chunk_min, c));
}
int64_t dep_nchunks(const augur_pm_plan *p, int64_t n) { return (n + dep_chunk(p, n) - 1) / dep_chunk(p, n); }

cudaStream_t S(void *s) { return (cudaStream_t)s; }

// ---- pipeline pieces ----------------------------------------------------------------

// Keys, slots and the row histogram of caller bodies off .. off + cnt - 1 (the arrays are the
// caller's whole arrays; key/slot are indexed like them), with the optional velocity-Verlet drift.
int keys_hist_range(augur_pm_plan *p, float *pos, const float *vel, const float *acc, const float *mass,
                    const float *mask, int64_t off, int64_t cnt, bool drift, float dt, cudaStream_t st) {
  if (cnt <= 0) return AUGUR_OK;
  const GridParams &g = p->gp;
  const int D = p->dim;
  const unsigned nb = blocks_for(cnt, 256);
  const float hdt2 = (float)(0.5 * (double)dt * (double)dt);
  float *ps = pos + off * D;
  const float *vs = vel ? vel + off * D : nullptr, *as = acc ? acc + off * D : nullptr;
  const float *ms = mass + off, *ks = mask + off;
  uint32_t *key = p->key + off, *slot = p->slot + off;
  if (D == 3) {
    if (drift)
      keys_hist_aos_kernel<3, true><<<nb, 256, 0, st>>>(ps, vs, as, ms, ks, cnt, g, dt, hdt2, key, slot, p->row_count,
                                                       p->d_mmax, p->d_err);
    else
      keys_hist_aos_kernel<3, false><<<nb, 256, 0, st>>>(ps, vs, as, ms, ks, cnt, g, dt, hdt2, key, slot,
                                                        p->row_count, p->d_mmax, p->d_err);
  } else {
    if (drift)
      keys_hist_aos_kernel<2, true><<<nb, 256, 0, st>>>(ps, vs, as, ms, ks, cnt, g, dt, hdt2, key, slot, p->row_count,
                                                       p->d_mmax, p->d_err);
    else
      keys_hist_aos_kernel<2, false><<<nb, 256, 0, st>>>(ps, vs, as, ms, ks, cnt, g, dt, hdt2, key, slot,
                                                        p->row_count, p->d_mmax, p->d_err);
  }
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

int sort_begin(augur_pm_plan *p, int64_t n, cudaStream_t st) {
  p->cur_n = n;
  if (cudaMemsetAsync(p->row_count, 0, sizeof(uint32_t) * p->nrow, st) != cudaSuccess) return AUGUR_ECUDA;
  if (cudaMemsetAsync(p->d_mmax, 0, sizeof(unsigned), st) != cudaSuccess) return AUGUR_ECUDA;
  return AUGUR_OK;
}

// scan of the histogram and the scatter of the caller's bodies into sorted order
int sort_finish(augur_pm_plan *p, const float *pos, const float *vel, const float *mass, const float *mask, int64_t n,
                cudaStream_t st) {
  scan_local_kernel<<<p->ntiles, 1024, 0, st>>>(p->row_count, p->row_start, p->tile_sum, p->nrow);
  AUGUR_LAUNCH_CHECK(p);
  scan_tiles_kernel<<<1, 1024, 0, st>>>(p->tile_sum, p->tile_off, p->ntiles);
  AUGUR_LAUNCH_CHECK(p);
  if (n > 0) {
    const unsigned nb = blocks_for(n, 256);
    if (p->dim == 3)
      scatter_aos_kernel<3><<<nb, 256, 0, st>>>(pos, vel, mass, mask, n, p->key, p->slot, p->row_start, p->tile_off,
                                                p->pos4[p->cur], p->vel4[p->cur]);
    else
      scatter_aos_kernel<2><<<nb, 256, 0, st>>>(pos, vel, mass, mask, n, p->key, p->slot, p->row_start, p->tile_off,
                                                p->pos4[p->cur], p->vel4[p->cur]);
    AUGUR_LAUNCH_CHECK(p);
  }
  return AUGUR_OK;
}

int sort_from_aos(augur_pm_plan *p, float *pos, const float *vel, const float *acc, const float *mass,
                  const float *mask, int64_t n, bool drift, float dt, cudaStream_t st) {
  int rc = sort_begin(p, n, st);
  if (!rc) rc = keys_hist_range(p, pos, vel, acc, mass, mask, 0, n, drift, dt, st);
  if (!rc) rc = sort_finish(p, pos, vel, mass, mask, n, st);
  return rc;
}

// re-sort the run state after a gather that produced keys + histogram
int resort(augur_pm_plan *p, cudaStream_t st) {
  const int64_t n = p->run_n;
  p->cur_n = n;
  scan_local_kernel<<<p->ntiles, 1024, 0, st>>>(p->row_count, p->row_start, p->tile_sum, p->nrow);
  AUGUR_LAUNCH_CHECK(p);
  scan_tiles_kernel<<<1, 1024, 0, st>>>(p->tile_sum, p->tile_off, p->ntiles);
  AUGUR_LAUNCH_CHECK(p);
  if (n > 0) {
    const int c = p->cur;
    scatter_sorted_kernel<<<blocks_for(n, 256), 256, 0, st>>>(p->pos4[c], p->vel4[c], n, p->key, p->slot,
                                                              p->row_start, p->tile_off, p->pos4[c ^ 1],
                                                              p->vel4[c ^ 1]);
    AUGUR_LAUNCH_CHECK(p);
    p->cur ^= 1;
  }
  return AUGUR_OK;
}

DepositArgs dep_args(const augur_pm_plan *p) {
  DepositArgs a;
  a.g = p->gp;
  a.RY = p->dep_RY;
  a.RZ = p->dim == 3 ? p->dep_RZ : 1;
  a.fsh = p->sh_M;
  a.twmul = p->Lt / p->M;
  a.Lt = p->Lt;
  a.nblk = p->nblk;
  a.chunk = dep_chunk(p, p->cur_n);
  a.fdG = make_fastdiv(p->G);
  a.fdRR = make_fastdiv(a.RY * a.RZ);
  a.fdRY = make_fastdiv(a.RY);
  return a;
}

// work-item plan + deposit of the sorted state: MODE 0 writes rho, MODE 1 the x-transformed spectrum
template <int D, int MODE>
int launch_deposit(augur_pm_plan *p, float *rho, float2 *spec, cudaStream_t st) {
  DepositArgs a = dep_args(p);
  deposit_count_kernel<D><<<blocks_for(p->nblk, 256), 256, 0, st>>>(p->row_start, p->tile_off, a, p->dep_nch,
                                                                      p->dep_seg_tab, p->d_err);
  AUGUR_LAUNCH_CHECK(p);
  deposit_plan_kernel<D><<<1, 1024, 0, st>>>(p->row_start, p->tile_off, a, p->dep_nch, p->dep_item_off,
                                              p->dep_slot_off, p->dep_seg_tab, p->dep_item_blk, p->d_err);
  AUGUR_LAUNCH_CHECK(p);
  const int64_t items = (int64_t)p->nblk + 4 * dep_nchunks(p, p->cur_n) + 1;
  if ((size_t)items > p->dep_items_max) return AUGUR_ERANGE;
  if (p->dep_agg)
    deposit_kernel<D, MODE, true><<<(unsigned)items, DEP_THREADS, p->smem_dep, st>>>(
        p->pos4[p->cur], p->d_mmax, a, p->tw, rho, spec, p->d_err, p->dep_item_off, p->dep_slot_off, p->dep_seg_tab,
        p->dep_item_blk, p->dep_scratch, p->dep_counters);
  else
    deposit_kernel<D, MODE, false><<<(unsigned)items, DEP_THREADS, p->smem_dep, st>>>(
        p->pos4[p->cur], p->d_mmax, a, p->tw, rho, spec, p->d_err, p->dep_item_off, p->dep_slot_off, p->dep_seg_tab,
        p->dep_item_blk, p->dep_scratch, p->dep_counters);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

int deposit_rho(augur_pm_plan *p, float *rho, cudaStream_t st) {
  return p->dim == 3 ? launch_deposit<3, 0>(p, rho, nullptr, st) : launch_deposit<2, 0>(p, rho, nullptr, st);
}

size_t rowst_smem(const augur_pm_plan *p) {
  return 128 + (size_t)ROWST_STAGES * p->rows_RB * p->L * 8 +
         (size_t)(fft_nstages(p->L) > 2 ? 2 : 1) * p->rows_RB * fft_row_stride(p->L) * 8 + (size_t)p->Lt * 8;
}

int fft_rows(augur_pm_plan *p, float2 *data, int64_t nrows, bool inverse, cudaStream_t st) {
  const int L = p->L;
  const int RB = p->rows_RB;
  // persistent bulk-copy form: multi-stage lengths, 16-byte aligned rows, and transforms large
  // enough for the pipeline to pay (measured on GB300: faster at 256^3, slower for 128^3 and below)
  if (L >= 32 && nrows * L >= ((int64_t)1 << 22) && (reinterpret_cast<uintptr_t>(data) & 15) == 0 &&
      rowst_smem(p) <= p->smem_max &&
      !raise_dyn_smem((const void *)rows_tma_kernel, rowst_smem(p))) {
    const int64_t nbatch = (nrows + RB - 1) / RB;
    const int per_sm = rowst_smem(p) * 2 + 4096 <= p->smem_max + 1024 ? 2 : 1;  // 228 KB per SM
    const int grid = (int)std::min<int64_t>(nbatch, (int64_t)per_sm * current_sm_count());
    rows_tma_kernel<<<grid, 256, rowst_smem(p), st>>>(data, nrows, RB, L, p->Lt / L, p->Lt, p->tw, inverse ? 1 : 0,
                                                      p->d_err);
    AUGUR_LAUNCH_CHECK(p);
    return AUGUR_OK;
  }
  fft_rows_kernel<<<blocks_for(nrows, RB), 256, p->smem_rows, st>>>(data, nrows, RB, L, make_fastdiv(L), p->Lt / L,
                                                                     p->Lt, p->tw, inverse ? 1 : 0);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

// x C2R of ncomp gradient spectra (spec3) into the float4 force grid
int launch_c2r(augur_pm_plan *p, int ncomp, float4 *F4, cudaStream_t st) {
  const int G = p->G, M = p->M;
  C2RArgs ca{};
  ca.L = G;
  ca.nrows = G * G;
  ca.RB = p->c2r_RB;
  ca.ncomp = ncomp;
  ca.Lt = p->Lt;
  ca.nkeep = G * G;
  ca.Lkeep = G;
  ca.scale = 1.f;
  ca.fsh = p->sh_M;
  ca.twmul = p->Lt / M;
  ca.fdRB = make_fastdiv(ca.RB);
  ca.fdM = make_fastdiv(ca.L / 2);
  ca.fdL = make_fastdiv(ca.L);
  ca.nbx = (M <= 128 && c2r_smem_bytes(M, ca.RB, G, ncomp, 2, p->Lt) <= p->smem_c2r) ? 2 : 1;
  const size_t smem = c2r_smem_bytes(M, ca.RB, G, ncomp, ca.nbx, p->Lt);
  c2r_rows_kernel<true><<<(unsigned)(G * G / p->c2r_RB), 512, smem, st>>>(p->spec3, ca, p->tw,
                                                                          reinterpret_cast<float *>(F4));
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

// z transform + Green's function + spectral gradient of spec into ncomp spectra (spec3)
int launch_green(augur_pm_plan *p, int ncomp, cudaStream_t st) {
  const int G = p->G, M = p->M;
  GreenArgs ga;
  ga.G = G;
  ga.TY = p->green_TY;
  ga.ncomp = ncomp;
  ga.Lt = p->Lt;
  ga.nbuf = green_nbuf(G);
  ga.fsh = p->sh_L;
  ga.kfund = (float)(2.0 * M_PI / p->extent);
  ga.gfac = (float)(-4.0 * M_PI * p->gnewton / ((double)G * G * G));
  if (p->green_TY == 16)
    fft_z_green_kernel<16><<<(unsigned)((M + 1) * (G / 16)), green_threads(G, 16), p->smem_green, st>>>(p->spec, ga, p->tw, p->spec3);
  else
    fft_z_green_kernel<8><<<(unsigned)((M + 1) * (G / 8)), green_threads(G, 8), p->smem_green, st>>>(p->spec, ga, p->tw, p->spec3);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

// periodic 3D: spec (after R2C along x) -> F4 force grid
int periodic_tail(augur_pm_plan *p, int ncomp, float4 *F4, cudaStream_t st) {
  const int G = p->G, M = p->M;
  int rc = fft_rows(p, p->spec, (int64_t)(M + 1) * G, false, st);
  if (!rc) rc = launch_green(p, ncomp, st);
  if (!rc) rc = fft_rows(p, p->spec3, (int64_t)ncomp * (M + 1) * G, true, st);
  if (!rc) rc = launch_c2r(p, ncomp, F4, st);
  return rc;
}

int r2c_rows(augur_pm_plan *p, const float *in, int Lin, int nin, int nout, float2 *out, cudaStream_t st) {
  RowsArgs ra;
  ra.L = p->L;
  ra.Lin = Lin;
  ra.nin = nin;
  ra.nout = nout;
  ra.RB = p->r2c_RB;
  ra.Lt = p->Lt;
  ra.fsh = p->sh_M;
  ra.twmul = p->Lt / p->M;
  ra.fdL = make_fastdiv(ra.L);
  ra.fdRB = make_fastdiv(ra.RB);
  r2c_rows_kernel<<<blocks_for(nout, ra.RB), 256, p->smem_r2c, st>>>(in, ra, p->tw, out);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

// isolated 2D: rho (G x G) -> F4 (G x G)
int isolated_from_rho(augur_pm_plan *p, const float *rho, float4 *F4, cudaStream_t st) {
  const int G = p->G, L = p->L;
  int rc = r2c_rows(p, rho, G, G, L, p->spec, st);
  if (rc) return rc;
  rc = fft_rows(p, p->spec, (int64_t)(p->M + 1), false, st);
  if (rc) return rc;
  const int64_t ns = (int64_t)(p->M + 1) * L;
  kmul_kernel<<<blocks_for(ns, 256), 256, 0, st>>>(p->spec, p->khat, ns);
  AUGUR_LAUNCH_CHECK(p);
  rc = fft_rows(p, p->spec, (int64_t)(p->M + 1), true, st);
  if (rc) return rc;
  C2RArgs ca{};
  ca.L = L;
  ca.nrows = L;
  ca.RB = p->c2r_RB;
  ca.ncomp = 1;
  ca.Lt = p->Lt;
  ca.nkeep = G;
  ca.Lkeep = G;
  const double h = p->extent / G;
  ca.scale = (float)(h * h / ((double)L * L));
  ca.fsh = p->sh_M;
  ca.twmul = p->Lt / p->M;
  ca.fdRB = make_fastdiv(ca.RB);
  ca.fdM = make_fastdiv(ca.L / 2);
  ca.fdL = make_fastdiv(ca.L);
  ca.ext = p->kpad_ext;
  if (p->kpad_ext) {
    // rows 0..G and 2G-1 are needed: transform every row (the others are not stored)
    c2r_rows_kernel<false><<<(unsigned)((L + p->c2r_RB - 1) / p->c2r_RB), 512, p->smem_c2r, st>>>(p->spec, ca, p->tw,
                                                                                                 p->phi_ext);
    AUGUR_LAUNCH_CHECK(p);
    fd_grad2d_ext_kernel<<<blocks_for((int64_t)G * G, 256), 256, 0, st>>>(p->phi_ext, G, (float)(2.0 * h), F4);
    AUGUR_LAUNCH_CHECK(p);
    return AUGUR_OK;
  }
  c2r_rows_kernel<false><<<(unsigned)((G + p->c2r_RB - 1) / p->c2r_RB), 512, p->smem_c2r, st>>>(p->spec, ca, p->tw,
                                                                                               p->phi2d);
  AUGUR_LAUNCH_CHECK(p);
  fd_grad2d_kernel<<<blocks_for((int64_t)G * G, 256), 256, 0, st>>>(p->phi2d, G, (float)(2.0 * h), F4);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

// sorted bodies -> F4 (the grid force of the plan's mode); rho_out (optional) also
// receives the density grid
int grid_force(augur_pm_plan *p, int ncomp, cudaStream_t st, float *rho_out = nullptr) {
  p->ncomp_last = ncomp;
  if (p->mode == AUGUR_MODE_PERIODIC) {
    int rc = rho_out ? launch_deposit<3, 2>(p, rho_out, p->spec, st) : launch_deposit<3, 1>(p, nullptr, p->spec, st);
    if (rc) return rc;
    return periodic_tail(p, ncomp, p->F4, st);
  }
  int rc = deposit_rho(p, p->rho2d, st);
  if (rc) return rc;
  return isolated_from_rho(p, p->rho2d, p->F4, st);
}

GatherArgs gather_args(const augur_pm_plan *p, float kick, float dt, int drift) {
  GatherArgs a;
  a.g = p->gp;
  a.kick = kick;
  a.dt = dt;
  a.drift = drift;
  a.esync = 0.f;
  a.epart = nullptr;
  return a;
}

// Gather at the sorted bodies (after sort_from_aos) into the caller's order: gather_sorted puts
// the sorted accelerations (float4: a * mask, phi * mask) in the free half of the body double
// buffer, then accel_to_caller writes acc / phi for caller bodies off .. off + cnt - 1 (vel == null)
// or applies the velocity-Verlet kick to their vel and acc.
float4 *gather_sorted(augur_pm_plan *p, const float4 *F4, int64_t n, cudaStream_t st) {
  GatherArgs a = gather_args(p, 0.f, 0.f, 0);
  float4 *acc4s = p->pos4[p->cur ^ 1];
  const unsigned nb = blocks_for(n, 256);
  float *a4 = reinterpret_cast<float *>(acc4s);
  if (p->dim == 3)
    gather_kernel<3, MODE_FORCE><<<nb, 256, 0, st>>>(F4, p->pos4[p->cur], p->vel4[p->cur], n, a, a4, nullptr,
                                                     nullptr, nullptr, nullptr, nullptr, p->d_err);
  else
    gather_kernel<2, MODE_FORCE><<<nb, 256, 0, st>>>(F4, p->pos4[p->cur], p->vel4[p->cur], n, a, a4, nullptr,
                                                     nullptr, nullptr, nullptr, nullptr, p->d_err);
  return acc4s;
}

int accel_to_caller(augur_pm_plan *p, const float4 *acc4s, int64_t off, int64_t cnt, float *acc, float *phi,
                    float *vel, float kick, cudaStream_t st) {
  if (cnt <= 0) return AUGUR_OK;
  const int D = p->dim;
  const unsigned nb = blocks_for(cnt, 256);
  const uint32_t *k = p->key + off, *sl = p->slot + off, *rs = p->row_start, *to = p->tile_off;
  float *ac = acc + off * D, *ph = phi ? phi + off : nullptr, *ve = vel ? vel + off * D : nullptr;
  if (vel) {
    if (D == 3)
      accel_to_caller_kernel<3, true><<<nb, 256, 0, st>>>(acc4s, cnt, k, sl, rs, to, kick, ac, ph, ve);
    else
      accel_to_caller_kernel<2, true><<<nb, 256, 0, st>>>(acc4s, cnt, k, sl, rs, to, kick, ac, ph, ve);
  } else {
    if (D == 3)
      accel_to_caller_kernel<3, false><<<nb, 256, 0, st>>>(acc4s, cnt, k, sl, rs, to, 0.f, ac, ph, nullptr);
    else
      accel_to_caller_kernel<2, false><<<nb, 256, 0, st>>>(acc4s, cnt, k, sl, rs, to, 0.f, ac, ph, nullptr);
  }
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

int gather_force(augur_pm_plan *p, const float4 *F4, int64_t n, float *acc, float *phi, cudaStream_t st,
                 float *vel = nullptr, float kick = 0.f) {
  if (n == 0) return AUGUR_OK;
  const float4 *acc4s = gather_sorted(p, F4, n, st);
  AUGUR_LAUNCH_CHECK(p);
  return accel_to_caller(p, acc4s, 0, n, acc, phi, vel, kick, st);
}

// ---- tile shapes ----------------------------------------------------------------------

augur_pm_tiles default_tiles(const augur_pm_plan *p) {
  // measured on GB300 over Plummer / clumpy / disk scenes of 1e4..3e6 bodies: single-plane
  // row blocks, small work items (more CTAs than SM slots even when the bodies concentrate)
  augur_pm_tiles t;
  const int G = p->G, L = p->L;
  // from 512 up the row block's shared memory limits residency: RY = 4096 / G keeps several CTAs
  // per SM (1024^3 with 10^9 bodies: RY 8 -> 4 takes the deposit from 49.9 to 40.4 ms)
  t.deposit_rows_y = G <= 64 ? 4 : (G <= 96 ? 8 : (G <= 256 ? 16 : 4096 / G));
  t.deposit_rows_z = 1;
  t.deposit_chunk = DEP_CHUNK_MIN;
  t.green_tile_y = (3 * G * 16 * 8 <= 200000) ? 16 : 8;
  t.c2r_rows = L <= 128 ? 32 : (L <= 512 ? 16 : (L <= 1024 ? 4 : 8));
  t.fft_rows = L >= 4096 ? 1 : std::min(4096 / L, L <= 64 ? 16 : 64);
  t.deposit_aggregate = 0;
  return t;
}

// Validates t against the plan's geometry and the device's shared memory; unless
// check_only, stores it with the shared-memory sizes that follow from it.
int apply_tiles(augur_pm_plan *p, const augur_pm_tiles *t, bool check_only) {
  const int G = p->G, M = p->M, L = p->L, Lt = p->Lt;
  const bool d3 = p->dim == 3;
  const int RY = t->deposit_rows_y, RZ = t->deposit_rows_z;
  if (RY < 1 || RY > G || G % RY != 0) return AUGUR_EINVAL;
  if (d3 ? (RZ < 1 || RZ > 15 || G % RZ != 0) : RZ != 1) return AUGUR_EINVAL;
  if (t->deposit_chunk < 1024 || t->deposit_chunk > DEP_ITEM_MAX) return AUGUR_EINVAL;
  if (!(t->green_tile_y == 8 || t->green_tile_y == 16) || G % t->green_tile_y != 0) return AUGUR_EINVAL;
  const int RB = t->c2r_rows;
  if (RB < 1 || RB > 32 || (RB & (RB - 1)) != 0) return AUGUR_EINVAL;
  if (d3 && ((G * G) % RB) != 0) return AUGUR_EINVAL;
  if (t->fft_rows < 1 || t->fft_rows > 256) return AUGUR_EINVAL;
  if (t->deposit_aggregate != 0 && t->deposit_aggregate != 1) return AUGUR_EINVAL;
  // shared memory of each kernel (layouts in pm_kernels.cuh; transform rows padded by fft_row_stride)
  const size_t PM = (size_t)fft_row_stride(M), PL = (size_t)fft_row_stride(L);
  const size_t s_dep = (size_t)RY * RZ * (2 * PM * 8 + (size_t)(G + 2) * 4) + (size_t)Lt * 8;
  const size_t s_green = (size_t)(1 + green_nbuf(G)) * G * t->green_tile_y * 8 + (size_t)Lt * 8;
  // periodic: four result planes with one input block (force + potential), and, where it fits,
  // three with two (force only, the next component copied in during a transform)
  size_t s_c2r = c2r_smem_bytes(M, RB, L, p->gp.periodic ? 4 : 1, 1, Lt);
  if (p->gp.periodic && M <= 128 && c2r_smem_bytes(M, RB, L, 3, 2, Lt) <= p->smem_max)
    s_c2r = std::max(s_c2r, c2r_smem_bytes(M, RB, L, 3, 2, Lt));
  const size_t s_rows = (size_t)2 * t->fft_rows * PL * 8 + (size_t)Lt * 8;
  const size_t s_r2c = (size_t)16 * ((M + 1) + 2 * PM) * 8 + (size_t)Lt * 8;
  const size_t lim = p->smem_max;
  if (s_dep > lim || s_green > lim || s_c2r > lim || s_rows > lim || s_r2c > lim) return AUGUR_EINVAL;
  if (check_only) return AUGUR_OK;
  p->dep_RY = RY;
  p->dep_RZ = RZ;
  p->dep_chunk_min = t->deposit_chunk;
  p->green_TY = t->green_tile_y;
  p->c2r_RB = RB;
  p->rows_RB = t->fft_rows;
  p->dep_agg = t->deposit_aggregate;
  p->r2c_RB = 16;
  p->smem_dep = s_dep;
  p->smem_green = s_green;
  p->smem_c2r = s_c2r;
  p->smem_rows = s_rows;
  p->smem_r2c = s_r2c;
  return AUGUR_OK;
}

// Deposit work-item tables and partial-tile scratch for the plan's tile shape and body bound.
int alloc_deposit_tables(augur_pm_plan *p) {
  void *old[] = {p->dep_nch, p->dep_item_off, p->dep_slot_off, p->dep_counters, p->dep_item_blk, p->dep_seg_tab,
                 p->dep_scratch};
  for (void *q : old)
    if (q) cudaFree(q);
  p->dep_nch = p->dep_item_off = p->dep_slot_off = p->dep_counters = p->dep_item_blk = nullptr;
  p->dep_seg_tab = nullptr;
  p->dep_scratch = nullptr;
  p->bytes -= p->dep_bytes;
  const size_t bytes0 = p->bytes;
  const int G = p->G;
  p->nblk = (p->dim == 3) ? (G / p->dep_RY) * (G / p->dep_RZ) : G / p->dep_RY;
  // chunks of any n <= max_n: ceil(n / dep_chunk) <= min(ceil(max_n / chunk_min), DEP_NCH_MAX)
  const int64_t nch = std::min<int64_t>((p->max_n + p->dep_chunk_min - 1) / p->dep_chunk_min, DEP_NCH_MAX);
  // one 64-bit accumulator tile per row block split over several work items: a split block has
  // at least two items, and there are at most nblk + 4 nch items, so at most min(nblk, 4 nch)
  p->dep_slots = (size_t)std::min<int64_t>(p->nblk, 4 * nch) + 1;
  p->dep_items_max = (size_t)p->nblk + 4 * (size_t)nch + 1;
  int rc = AUGUR_OK;
  rc |= dalloc(p, &p->dep_nch, (size_t)p->nblk);
  rc |= dalloc(p, &p->dep_item_off, (size_t)p->nblk + 1);
  rc |= dalloc(p, &p->dep_slot_off, (size_t)p->nblk);
  rc |= dalloc(p, &p->dep_counters, (size_t)p->nblk);
  rc |= dalloc(p, &p->dep_item_blk, p->dep_items_max);
  rc |= dalloc(p, &p->dep_seg_tab, (size_t)p->nblk * (MAXSEGB + 1));
  rc |= dalloc(p, &p->dep_scratch, p->dep_slots * (size_t)p->dep_RY * p->dep_RZ * G);
  p->dep_bytes = p->bytes - bytes0;
  if (rc != AUGUR_OK) return AUGUR_ENOMEM;
  if (cudaMemset(p->dep_counters, 0, sizeof(uint32_t) * p->nblk) != cudaSuccess) return AUGUR_ECUDA;
  // the split blocks' accumulator tiles start at zero; the last work item of a block clears its
  // tile after reading it, so they are zero again at the start of every deposit
  if (cudaMemset(p->dep_scratch, 0, p->dep_slots * (size_t)p->dep_RY * p->dep_RZ * G * 8) != cudaSuccess)
    return AUGUR_ECUDA;
  return AUGUR_OK;
}

// The dynamic shared-memory opt-in is a property of the kernel, shared by every plan in the
// process: it is only ever raised, so that a plan with smaller tiles never lowers the limit
// another plan's launches rely on.
template <typename K>
int raise_smem(K *kernel, size_t bytes) {
  return raise_dyn_smem((const void *)kernel, bytes);
}

int raise_smem_limits(const augur_pm_plan *p) {
  int rc = AUGUR_OK;
  rc |= raise_smem(deposit_kernel<3, 0, false>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<3, 1, false>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<3, 2, false>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<2, 0, false>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<3, 0, true>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<3, 1, true>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<3, 2, true>, p->smem_dep);
  rc |= raise_smem(deposit_kernel<2, 0, true>, p->smem_dep);
  rc |= raise_smem(fft_z_green_kernel<16>, p->smem_green);
  rc |= raise_smem(fft_z_green_kernel<8>, p->smem_green);
  rc |= raise_smem(c2r_rows_kernel<true>, p->smem_c2r);
  rc |= raise_smem(c2r_rows_kernel<false>, p->smem_c2r);
  rc |= raise_smem(fft_rows_kernel, p->smem_rows);
  rc |= raise_smem(r2c_rows_kernel, p->smem_r2c);
  return rc ? AUGUR_ECUDA : AUGUR_OK;
}

// the isolated plan's kernel spectrum from the lattice in real_tmp
int lattice_to_khat(augur_pm_plan *p, cudaStream_t st) {
  const int L = p->L;
  int rc = r2c_rows(p, p->real_tmp, L, L, L, p->khat, st);
  if (!rc) rc = fft_rows(p, p->khat, (int64_t)(p->M + 1), false, st);
  return rc;
}

// the reference's plain-PM kernel K = -1/sqrt(d^2 + eps^2) (pm_baseline_force_error.py:70-73)
int softened_kernel(augur_pm_plan *p, cudaStream_t st) {
  const int L = p->L;
  kernel_lattice_kernel<<<blocks_for((int64_t)L * L, 256), 256, 0, st>>>(p->real_tmp, L, (float)(p->extent / p->G),
                                                                         (float)(p->eps * p->eps));
  AUGUR_LAUNCH_CHECK(p);
  p->kpad_ext = 0;
  return lattice_to_khat(p, st);
}

int check_plan(const augur_pm_plan *p, int64_t n) {
  if (!p) return AUGUR_EINVAL;
  if (n < 0 || n > p->max_n) return AUGUR_EINVAL;
  return AUGUR_OK;
}

}  // namespace

// =====================================================================================
// C ABI
// =====================================================================================
extern "C" {

const char *augur_status_string(int status) {
  switch (status) {
    case AUGUR_OK: return "ok";
    case AUGUR_EINVAL: return "invalid argument (shape, size, mode or pointer)";
    case AUGUR_ENOMEM: return "device allocation failed";
    case AUGUR_ETIMEDOUT: return "a device wait ran out of its budget";
    case AUGUR_ERANGE: return "count or index outside the supported range";
    case AUGUR_EIO: return "non-finite body state seen on the device";
    case AUGUR_ECUDA: return "CUDA runtime error";
    default: return "unknown status";
  }
}

int augur_version(void) { return 0x000100; }

int augur_pm_plan_destroy(augur_pm_plan *p) {
  if (!p) return AUGUR_OK;
  void *ptrs[] = {p->tw, p->pos4[0], p->pos4[1], p->vel4[0], p->vel4[1], p->key, p->slot, p->row_count,
                  p->row_start, p->tile_sum, p->tile_off, p->d_err, p->d_mmax, p->spec, p->spec3, p->khat,
                  p->F4_own, p->real_tmp, p->phi2d, p->rho2d, p->phi_ext, p->kparams, p->dep_nch, p->dep_item_off, p->dep_slot_off,
                  p->dep_counters, p->dep_scratch, p->dep_item_blk, p->dep_seg_tab, p->epart,
                  p->pair_key, p->pair_rank, p->pair_cnt, p->pair_start, p->pair_tsum, p->pair_toff,
                  p->pair_sorted, p->pair_params, p->pair_nbj, p->pair_nbq};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (p->hs_buf) {
    cudaFree(p->hs_buf);
    cudaStreamDestroy(p->hs_in);
    cudaStreamDestroy(p->hs_out);
    for (cudaEvent_t e : p->hs_ev) cudaEventDestroy(e);
  }
  delete p;
  return AUGUR_OK;
}

int augur_pm_plan_create(augur_pm_plan **out, int dim, int grid, int64_t max_bodies, int mode, double extent,
                         double eps, double g_newton) {
  if (!out) return AUGUR_EINVAL;
  *out = nullptr;
  if (!(dim == 3 && mode == AUGUR_MODE_PERIODIC) && !(dim == 2 && mode == AUGUR_MODE_ISOLATED_SOFTENED))
    return AUGUR_EINVAL;
  if (grid < 16 || grid > 1024 || (grid % 16) != 0) return AUGUR_EINVAL;
  if (max_bodies < 1 || max_bodies > 0x7fffffffLL) return AUGUR_EINVAL;
  if (!(extent > 0.0) || !std::isfinite(extent)) return AUGUR_EINVAL;
  augur_pm_plan *p = new (std::nothrow) augur_pm_plan();
  if (!p) return AUGUR_ENOMEM;
  memset(p, 0, sizeof(*p));
  p->dim = dim;
  p->G = grid;
  p->mode = mode;
  p->extent = extent;
  p->eps = eps;
  p->gnewton = g_newton;
  p->max_n = max_bodies;
  const int G = grid;
  const double h = extent / G;
  GridParams &g = p->gp;
  g.G = G;
  g.D = dim;
  g.periodic = mode == AUGUR_MODE_PERIODIC;
  g.h = (float)h;
  g.half_ext = (float)(extent / 2.0);
  g.ext = (float)extent;
  g.inv_hD = (float)(1.0 / (dim == 3 ? h * h * h : h * h));
  {
    int ex = 0;
    float mant = std::frexp(g.h, &ex);
    g.inv_h = (mant == 0.5f) ? 1.0f / g.h : 0.0f;  // exact reciprocal of a power of two
  }
  p->nrow = (dim == 3) ? G * G : G + 2;
  g.nrow = p->nrow;
  p->ntiles = (p->nrow + SCAN_TILE - 1) / SCAN_TILE;
  p->L = g.periodic ? G : 2 * G;
  p->M = p->L / 2;
  p->Lt = p->L;
  if (!factor(p->M, p->sh_M) || !factor(p->L, p->sh_L) || !fft_length_supported(p->M) ||
      !fft_length_supported(p->L)) {
    delete p;
    return AUGUR_EINVAL;
  }
  // default tile shapes (an autotuner may replace them through augur_pm_plan_set_tiles)
  {
    int dev = 0, smax = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
      cudaGetLastError();
      smax = 232448;
    }
    p->smem_max = (size_t)smax;
  }
  augur_pm_tiles t = default_tiles(p);
  if (apply_tiles(p, &t, /*check_only=*/false) != AUGUR_OK) {
    delete p;
    return AUGUR_EINVAL;
  }
  const int M = p->M, L = p->L, Lt = p->Lt;

  int rc = AUGUR_OK;
  const int64_t N = max_bodies;
  const size_t ncell = (dim == 3) ? (size_t)G * G * G : (size_t)G * G;
  const size_t nspec = (size_t)(M + 1) * (dim == 3 ? (size_t)G * G : (size_t)L);
  rc |= dalloc(p, &p->tw, (size_t)Lt);
  for (int b = 0; b < 2; ++b) {
    rc |= dalloc(p, &p->pos4[b], (size_t)N);
    rc |= dalloc(p, &p->vel4[b], (size_t)N);
  }
  rc |= dalloc(p, &p->key, (size_t)N);
  rc |= dalloc(p, &p->slot, (size_t)N);
  rc |= dalloc(p, &p->row_count, (size_t)p->nrow);
  rc |= dalloc(p, &p->row_start, (size_t)(p->ntiles + 1) * SCAN_TILE);
  rc |= dalloc(p, &p->tile_sum, (size_t)p->ntiles + 1);
  rc |= dalloc(p, &p->tile_off, (size_t)p->ntiles + 1);
  rc |= dalloc(p, &p->d_err, 1);
  rc |= dalloc(p, &p->d_mmax, 1);
  rc |= dalloc(p, &p->spec, nspec);
  rc |= dalloc(p, &p->F4_own, ncell);
  p->F4 = p->F4_own;
  rc |= alloc_deposit_tables(p);
  if (dim == 3) {
    rc |= dalloc(p, &p->spec3, 4 * nspec);
  } else {
    rc |= dalloc(p, &p->khat, nspec);
    rc |= dalloc(p, &p->real_tmp, (size_t)L * L);
    rc |= dalloc(p, &p->phi2d, ncell);
    rc |= dalloc(p, &p->phi_ext, (size_t)(G + 2) * (G + 2));
    rc |= dalloc(p, &p->kparams, (size_t)KMLP_H * KMLP_MAXCOL + KMLP_H * KMLP_H + 3 * KMLP_H + 1);
    rc |= dalloc(p, &p->rho2d, ncell);
  }
  if (rc != AUGUR_OK) {
    augur_pm_plan_destroy(p);
    return AUGUR_ENOMEM;
  }
  cudaMemset(p->row_count, 0, sizeof(uint32_t) * p->nrow);
  cudaMemset(p->row_start, 0, sizeof(uint32_t) * (size_t)(p->ntiles + 1) * SCAN_TILE);
  cudaMemset(p->d_err, 0, sizeof(unsigned));
  cudaMemset(p->d_mmax, 0, sizeof(unsigned));
  // twiddles exp(-2 pi i t / Lt) in double, rounded once to float
  std::vector<float2> tw(Lt);
  for (int t = 0; t < Lt; ++t) {
    double ang = 2.0 * M_PI * (double)t / (double)Lt;
    tw[t] = make_float2((float)std::cos(ang), (float)-std::sin(ang));
  }
  if (cudaMemcpy(p->tw, tw.data(), sizeof(float2) * Lt, cudaMemcpyHostToDevice) != cudaSuccess) {
    augur_pm_plan_destroy(p);
    return AUGUR_ECUDA;
  }
  if (raise_smem_limits(p) != AUGUR_OK) {
    augur_pm_plan_destroy(p);
    return AUGUR_ECUDA;
  }
  if (mode == AUGUR_MODE_ISOLATED_SOFTENED) {
    // kernel spectrum rfft2(K) of the 2G min-image lattice, once per plan
    rc = softened_kernel(p, 0);
    if (!rc) rc = cuda_status(cudaDeviceSynchronize());
    if (rc) {
      augur_pm_plan_destroy(p);
      return rc;
    }
  }
  *out = p;
  return AUGUR_OK;
}

int64_t augur_pm_plan_workspace_bytes(const augur_pm_plan *p) { return p ? (int64_t)p->bytes : 0; }

int64_t augur_pm_last_launches(const augur_pm_plan *p) { return p ? p->launches : 0; }

int augur_pm_cell_index(augur_pm_plan *p, const float *pos, int64_t n, int32_t *i0, float *w, void *stream) {
  if (!p || n < 0 || (n > 0 && (!pos || !i0 || !w))) return AUGUR_EINVAL;
  p->launches = 0;
  if (n == 0) return AUGUR_OK;
  if (p->dim == 3)
    cell_index_kernel<3><<<blocks_for(n, 256), 256, 0, S(stream)>>>(pos, n, p->gp, i0, w, p->d_err);
  else
    cell_index_kernel<2><<<blocks_for(n, 256), 256, 0, S(stream)>>>(pos, n, p->gp, i0, w, p->d_err);
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

int augur_pm_deposit(augur_pm_plan *p, const float *pos, const float *mass, const float *mask, int64_t n, float *rho,
                     void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (!rho || (n > 0 && (!pos || !mass || !mask))) return AUGUR_EINVAL;
  p->launches = 0;
  p->run_active = 0;
  cudaStream_t st = S(stream);
  rc = sort_from_aos(p, const_cast<float *>(pos), nullptr, nullptr, mass, mask, n, false, 0.f, st);
  if (rc) return rc;
  return deposit_rho(p, rho, st);
}

int augur_pm_poisson(augur_pm_plan *p, const float *rho, float *force, void *stream) {
  if (!p || !rho || !force) return AUGUR_EINVAL;
  p->launches = 0;
  cudaStream_t st = S(stream);
  float4 *F4 = reinterpret_cast<float4 *>(force);
  if (p->mode == AUGUR_MODE_PERIODIC) {
    const int G = p->G;
    int rc = r2c_rows(p, rho, G, G * G, G * G, p->spec, st);
    if (rc) return rc;
    return periodic_tail(p, 4, F4, st);
  }
  return isolated_from_rho(p, rho, F4, st);
}

int augur_pm_gather(augur_pm_plan *p, const float *force, const float *pos, const float *mask, int64_t n, float *acc,
                    float *phi, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (!force || (n > 0 && (!pos || !mask || !acc))) return AUGUR_EINVAL;
  p->launches = 0;
  p->run_active = 0;
  cudaStream_t st = S(stream);
  // the gather reads the sorted body state; masses do not matter here (mask used as mass)
  rc = sort_from_aos(p, const_cast<float *>(pos), nullptr, nullptr, mask, mask, n, false, 0.f, st);
  if (rc) return rc;
  return gather_force(p, reinterpret_cast<const float4 *>(force), n, acc, phi, st);
}

int augur_pm_force(augur_pm_plan *p, const float *pos, const float *mass, const float *mask, int64_t n, float *acc,
                   float *phi, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (n > 0 && (!pos || !mass || !mask || !acc)) return AUGUR_EINVAL;
  p->launches = 0;
  p->run_active = 0;
  cudaStream_t st = S(stream);
  rc = sort_from_aos(p, const_cast<float *>(pos), nullptr, nullptr, mass, mask, n, false, 0.f, st);
  if (rc) return rc;
  rc = grid_force(p, phi ? 4 : 3, st);
  if (rc) return rc;
  return gather_force(p, p->F4, n, acc, phi, st);
}

int augur_pm_step(augur_pm_plan *p, float *pos, float *vel, float *acc, const float *mass, const float *mask,
                  int64_t n, float dt, int have_acc, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (n > 0 && (!pos || !vel || !acc || !mass || !mask)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  int64_t launches = 0;
  if (!have_acc) {
    rc = augur_pm_force(p, pos, mass, mask, n, acc, nullptr, stream);
    if (rc) return rc;
    launches = p->launches;
  }
  p->launches = launches;
  p->run_active = 0;
  rc = sort_from_aos(p, pos, vel, acc, mass, mask, n, true, dt, st);
  if (rc) return rc;
  rc = grid_force(p, 3, st);
  if (rc) return rc;
  return gather_force(p, p->F4, n, acc, nullptr, st, vel, (float)(0.5 * (double)dt));
}

int augur_pm_step_host(augur_pm_plan *p, float *pos, float *vel, float *acc, const float *mass, const float *mask,
                       int64_t n, float dt, int have_acc, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (n > 0 && (!pos || !vel || !acc || !mass || !mask)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  const int D = p->dim;
  if (!p->hs_buf) {
    // staging, streams and events are created together; on any failure whatever was created is
    // released again, so the next call starts from scratch
    float *buf = nullptr;
    cudaStream_t sin = nullptr, sout = nullptr;
    cudaEvent_t ev[3 * HS_CHUNKS + 2] = {};
    bool ok = cudaMalloc(&buf, sizeof(float) * 3 * (size_t)p->max_n * D) == cudaSuccess;
    const bool oom = !ok;
    ok = ok && cudaStreamCreateWithFlags(&sin, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&sout, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t &e : ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
      if (sout) cudaStreamDestroy(sout);
      if (sin) cudaStreamDestroy(sin);
      if (buf) cudaFree(buf);
      cudaGetLastError();
      return oom ? AUGUR_ENOMEM : AUGUR_ECUDA;
    }
    p->hs_buf = buf;
    p->hs_in = sin;
    p->hs_out = sout;
    for (int i = 0; i < 3 * HS_CHUNKS + 2; ++i) p->hs_ev[i] = ev[i];
    p->bytes += sizeof(float) * 3 * (size_t)p->max_n * D;
  }
  float *dpos = p->hs_buf, *dvel = dpos + (size_t)p->max_n * D, *dacc = dvel + (size_t)p->max_n * D;
  const size_t rb = sizeof(float) * D;  // bytes per body of pos, vel, acc
  auto h2d = [&](float *d, const float *h, int64_t off, int64_t cnt, cudaStream_t s) {
    return cudaMemcpyAsync(d + off * D, h + off * D, (size_t)cnt * rb, cudaMemcpyHostToDevice, s) == cudaSuccess;
  };
  auto d2h = [&](float *h, const float *d, int64_t off, int64_t cnt, cudaStream_t s) {
    return cudaMemcpyAsync(h + off * D, d + off * D, (size_t)cnt * rb, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  };
  if (!have_acc || n == 0) {
    // first step (the force at the start positions comes first): whole arrays in, out
    if (n > 0 && !(h2d(dpos, pos, 0, n, st) && h2d(dvel, vel, 0, n, st))) return AUGUR_ECUDA;
    rc = augur_pm_step(p, dpos, dvel, dacc, mass, mask, n, dt, have_acc, stream);
    if (rc) return rc;
    if (n > 0 && !(d2h(pos, dpos, 0, n, st) && d2h(vel, dvel, 0, n, st) && d2h(acc, dacc, 0, n, st)))
      return AUGUR_ECUDA;
    return AUGUR_OK;
  }
  p->launches = 0;
  p->run_active = 0;
  const int nc = (int)std::min<int64_t>(HS_CHUNKS, n);
  auto lo = [&](int c) { return n * c / nc; };
  cudaEvent_t *ev_in = p->hs_ev, *ev_drift = p->hs_ev + HS_CHUNKS, *ev_kick = p->hs_ev + 2 * HS_CHUNKS;
  cudaEvent_t ev_start = p->hs_ev[3 * HS_CHUNKS], ev_done = p->hs_ev[3 * HS_CHUNKS + 1];
  bool ok = cudaEventRecord(ev_start, st) == cudaSuccess && cudaStreamWaitEvent(p->hs_in, ev_start, 0) == cudaSuccess &&
            cudaStreamWaitEvent(p->hs_out, ev_start, 0) == cudaSuccess;
  // inputs in by chunks; each chunk's drift, keys and histogram start as soon as it has landed
  for (int c = 0; ok && c < nc; ++c) {
    const int64_t a = lo(c), cnt = lo(c + 1) - a;
    ok = h2d(dpos, pos, a, cnt, p->hs_in) && h2d(dvel, vel, a, cnt, p->hs_in) && h2d(dacc, acc, a, cnt, p->hs_in) &&
         cudaEventRecord(ev_in[c], p->hs_in) == cudaSuccess;
  }
  if (!ok) return AUGUR_ECUDA;
  rc = sort_begin(p, n, st);
  for (int c = 0; !rc && c < nc; ++c) {
    const int64_t a = lo(c), cnt = lo(c + 1) - a;
    if (cudaStreamWaitEvent(st, ev_in[c], 0) != cudaSuccess) return AUGUR_ECUDA;
    rc = keys_hist_range(p, dpos, dvel, dacc, mass, mask, a, cnt, true, dt, st);
    if (!rc && cudaEventRecord(ev_drift[c], st) != cudaSuccess) rc = AUGUR_ECUDA;
  }
  if (rc) return rc;
  // the drifted positions are final: out while the grid is solved
  for (int c = 0; ok && c < nc; ++c) {
    const int64_t a = lo(c), cnt = lo(c + 1) - a;
    ok = cudaStreamWaitEvent(p->hs_out, ev_drift[c], 0) == cudaSuccess && d2h(pos, dpos, a, cnt, p->hs_out);
  }
  if (!ok) return AUGUR_ECUDA;
  rc = sort_finish(p, dpos, dvel, mass, mask, n, st);
  if (!rc) rc = grid_force(p, 3, st);
  if (rc) return rc;
  const float4 *acc4s = gather_sorted(p, p->F4, n, st);
  AUGUR_LAUNCH_CHECK(p);
  const float kick = (float)(0.5 * (double)dt);
  for (int c = 0; !rc && c < nc; ++c) {
    const int64_t a = lo(c), cnt = lo(c + 1) - a;
    rc = accel_to_caller(p, acc4s, a, cnt, dacc, nullptr, dvel, kick, st);
    if (!rc && cudaEventRecord(ev_kick[c], st) != cudaSuccess) rc = AUGUR_ECUDA;
  }
  if (rc) return rc;
  for (int c = 0; ok && c < nc; ++c) {
    const int64_t a = lo(c), cnt = lo(c + 1) - a;
    ok = cudaStreamWaitEvent(p->hs_out, ev_kick[c], 0) == cudaSuccess && d2h(vel, dvel, a, cnt, p->hs_out) &&
         d2h(acc, dacc, a, cnt, p->hs_out);
  }
  // the caller's stream completes only after every copy
  ok = ok && cudaEventRecord(ev_done, p->hs_out) == cudaSuccess && cudaStreamWaitEvent(st, ev_done, 0) == cudaSuccess;
  return ok ? AUGUR_OK : AUGUR_ECUDA;
}

static int run_gather(augur_pm_plan *p, float kick, int drift, float *acc_out, cudaStream_t st,
                      double *energy_out = nullptr, float esync = 0.f) {
  const int64_t n = p->run_n;
  if (n == 0) return AUGUR_OK;
  GatherArgs a = gather_args(p, kick, p->run_dt, drift);
  const unsigned nb = blocks_for(n, 256);
  if (energy_out) {
    if (!p->epart || p->epart_n < nb) {
      if (p->epart) cudaFree(p->epart);
      p->epart = nullptr;
      if (cudaMalloc(&p->epart, sizeof(double) * 2 * nb) != cudaSuccess) return AUGUR_ENOMEM;
      p->epart_n = nb;
    }
    a.epart = p->epart;
    a.esync = esync;
  }
  gather_kernel<3, MODE_KD><<<nb, 256, 0, st>>>(p->F4, p->pos4[p->cur], p->vel4[p->cur], n, a, acc_out, nullptr,
                                                 nullptr, p->key, p->slot, p->row_count, p->d_err);
  AUGUR_LAUNCH_CHECK(p);
  if (energy_out) {
    energy_fold_kernel<<<1, FOLD_THREADS, 0, st>>>(p->epart, (int)nb, energy_out);
    AUGUR_LAUNCH_CHECK(p);
  }
  return AUGUR_OK;
}

int augur_pm_run_load(augur_pm_plan *p, const float *pos, const float *vel, const float *mass, const float *mask,
                      int64_t n, float dt, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (p->mode != AUGUR_MODE_PERIODIC) return AUGUR_EINVAL;
  if (n > 0 && (!pos || !vel || !mass || !mask)) return AUGUR_EINVAL;
  p->launches = 0;
  p->run_n = n;
  p->run_dt = dt;
  rc = sort_from_aos(p, const_cast<float *>(pos), vel, nullptr, mass, mask, n, false, 0.f, S(stream));
  if (rc) return rc;
  p->run_active = 2;  // loaded and sorted; the next grid call needs no re-sort
  return AUGUR_OK;
}

int augur_pm_run_grid(augur_pm_plan *p, float *rho_out, int with_phi, void *stream) {
  if (!p || !p->run_active) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  p->launches = 0;
  if (p->run_active == 1) {
    int rc = resort(p, st);
    if (rc) return rc;
  }
  p->run_active = 3;  // grid computed; the kick comes next
  return grid_force(p, with_phi ? 4 : 3, st, rho_out);
}

float *augur_pm_force_grid(augur_pm_plan *p) { return p ? reinterpret_cast<float *>(p->F4) : nullptr; }

int augur_pm_plan_get_tiles(const augur_pm_plan *p, augur_pm_tiles *out) {
  if (!p || !out) return AUGUR_EINVAL;
  out->deposit_rows_y = p->dep_RY;
  out->deposit_rows_z = p->dep_RZ;
  out->deposit_chunk = p->dep_chunk_min;
  out->green_tile_y = p->green_TY;
  out->c2r_rows = p->c2r_RB;
  out->fft_rows = p->rows_RB;
  out->deposit_aggregate = p->dep_agg;
  return AUGUR_OK;
}

int augur_pm_plan_set_tiles(augur_pm_plan *p, const augur_pm_tiles *t) {
  if (!p || !t) return AUGUR_EINVAL;
  int rc = apply_tiles(p, t, true);
  if (rc) return rc;
  const bool realloc_dep = t->deposit_rows_y != p->dep_RY || t->deposit_rows_z != p->dep_RZ ||
                           t->deposit_chunk != p->dep_chunk_min;
  if (realloc_dep && cudaDeviceSynchronize() != cudaSuccess) return AUGUR_ECUDA;
  apply_tiles(p, t, false);
  if (realloc_dep) {
    rc = alloc_deposit_tables(p);
    if (rc) return rc;
  }
  return raise_smem_limits(p);
}

int augur_pm_set_kernel_mlp(augur_pm_plan *p, const float *params, int ncol, const float *extra, int n_extra,
                            int flags, double split_radius, double eps, void *stream) {
  if (!p || !params) return AUGUR_EINVAL;
  if (p->mode != AUGUR_MODE_ISOLATED_SOFTENED) return AUGUR_EINVAL;
  const int nbase = (flags & AUGUR_KERNEL_CELL_UNITS) ? 3 : 2;
  if (n_extra < 0 || ncol != nbase + n_extra || ncol > KMLP_MAXCOL || (n_extra > 0 && !extra)) return AUGUR_EINVAL;
  if ((flags & AUGUR_KERNEL_SPLIT) && !(split_radius > 0.0)) return AUGUR_EINVAL;
  if ((flags & AUGUR_KERNEL_PRIOR) && !(eps >= 0.0)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  p->launches = 0;
  const size_t np = (size_t)KMLP_H * ncol + KMLP_H * KMLP_H + 3 * KMLP_H + 1;
  if (cudaMemcpyAsync(p->kparams, params, np * sizeof(float), cudaMemcpyDefault, st) != cudaSuccess)
    return AUGUR_ECUDA;
  KmlpArgs a;
  a.L = p->L;
  a.ncol = ncol;
  a.nbase = nbase;
  a.flags = ((flags & AUGUR_KERNEL_CELL_UNITS) ? 1 : 0) | ((flags & AUGUR_KERNEL_PRIOR) ? 2 : 0) |
            ((flags & AUGUR_KERNEL_SPLIT) ? 4 : 0);
  a.h = (float)(p->extent / p->G);
  a.split_r = (float)split_radius;
  a.eps2 = (float)(eps * eps);
  for (int j = 0; j < KMLP_MAXCOL; ++j) a.extra[j] = j < n_extra ? extra[j] : 0.f;
  const int L = p->L;
  kmlp_lattice_kernel<<<blocks_for((int64_t)L * L, 256), 256, np * sizeof(float), st>>>(p->kparams, a, p->real_tmp);
  AUGUR_LAUNCH_CHECK(p);
  int rc = lattice_to_khat(p, st);
  if (rc) return rc;
  p->kpad_ext = (flags & AUGUR_KERNEL_PAD_EXT) ? 1 : 0;
  return AUGUR_OK;
}

int augur_pm_reset_kernel(augur_pm_plan *p, void *stream) {
  if (!p || p->mode != AUGUR_MODE_ISOLATED_SOFTENED) return AUGUR_EINVAL;
  p->launches = 0;
  return softened_kernel(p, S(stream));
}

int augur_pm_pair_acc(augur_pm_plan *p, const float *pos, const float *mass, const float *mask, int64_t n,
                      double ppe, int knn, const float *params, int ncol, const float *extra, int n_extra, int flags,
                      double eps, float *acc, void *stream) {
  if (!p || p->dim != 2 || p->mode == AUGUR_MODE_PERIODIC) return AUGUR_EINVAL;
  if (n < 0 || n > p->max_n) return AUGUR_EINVAL;
  if (n > 0 && (!pos || !mass || !mask || !acc)) return AUGUR_EINVAL;
  if (!(ppe > 0.0) || !std::isfinite(ppe) || knn < 1 || knn > PAIR_KMAX) return AUGUR_EINVAL;
  const int nbase = (flags & AUGUR_KERNEL_CELL_UNITS) ? 3 : 2;
  if (params && (n_extra < 0 || ncol != nbase + n_extra || ncol > KMLP_MAXCOL || (n_extra > 0 && !extra)))
    return AUGUR_EINVAL;
  if ((flags & AUGUR_KERNEL_PRIOR) && !(eps >= 0.0)) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  cudaStream_t st = S(stream);
  p->launches = 0;
  // cells of side ppe / 4 (fewer candidates per search in dense regions), at most PAIR_CMAX a side
  const double E = p->extent;
  double cs = ppe / 4.0;
  if (std::ceil(E / cs) > PAIR_CMAX) cs = E / PAIR_CMAX;
  PairArgs a{};
  a.C = (int)std::max(1.0, std::min((double)PAIR_CMAX, std::ceil(E / cs)));
  a.cs = (float)cs;
  a.W = (int)std::ceil(ppe / cs) + 1;  // one ring more than the pair radius needs: rounding at cell edges
  a.knn = knn;
  a.half_ext = (float)(E / 2);
  a.inv_ppe = (float)(1.0 / ppe);
  a.thr0 = (float)(ppe * ppe * (1.0 + 1.0 / 4096));  // |d|^2 + 1e-8 >= thr0  =>  r / ppe rounds >= 1, weight 0
  a.slack = (float)((E / 2 + 2 * ppe + cs) / 65536.0);
  a.eps2 = (float)(eps * eps);
  a.h = (float)(E / p->G);
  a.flags = ((flags & AUGUR_KERNEL_CELL_UNITS) ? 1 : 0) | ((flags & AUGUR_KERNEL_PRIOR) ? 2 : 0);
  a.nbase = nbase;
  a.ncol = params ? ncol : nbase;
  for (int j = 0; j < KMLP_MAXCOL; ++j) a.extra[j] = (params && j < n_extra) ? extra[j] : 0.f;
  const size_t ncells = (size_t)a.C * a.C + 1;  // + the bucket of bodies with mask <= 0
  const int ntiles = (int)((ncells + SCAN_TILE - 1) / SCAN_TILE);
  int rc = AUGUR_OK;
  if (!p->pair_key) {
    rc |= dalloc(p, &p->pair_key, (size_t)p->max_n);
    rc |= dalloc(p, &p->pair_rank, (size_t)p->max_n);
    rc |= dalloc(p, &p->pair_sorted, (size_t)p->max_n);
    rc |= dalloc(p, &p->pair_params, (size_t)KMLP_H * KMLP_MAXCOL + KMLP_H * KMLP_H + 3 * KMLP_H + 1);
    if (rc) return AUGUR_ENOMEM;
  }
  if (ncells > p->pair_cells_cap) {
    const size_t nt = (p->pair_cells_cap + SCAN_TILE - 1) / SCAN_TILE;
    const size_t old_bytes = sizeof(uint32_t) * (p->pair_cells_cap + (nt + 1) * SCAN_TILE + 2 * nt + 1);
    for (uint32_t *q : {p->pair_cnt, p->pair_start, p->pair_tsum, p->pair_toff})
      if (q) cudaFree(q);
    if (p->pair_cnt) p->bytes -= old_bytes;
    p->pair_cnt = p->pair_start = p->pair_tsum = p->pair_toff = nullptr;
    p->pair_cells_cap = 0;
    rc |= dalloc(p, &p->pair_cnt, ncells);
    rc |= dalloc(p, &p->pair_start, (size_t)(ntiles + 1) * SCAN_TILE);
    rc |= dalloc(p, &p->pair_tsum, (size_t)ntiles);
    rc |= dalloc(p, &p->pair_toff, (size_t)ntiles + 1);
    if (rc) return AUGUR_ENOMEM;
    // the scan clears the counts it reads, so they stay zero between calls
    if (cudaMemset(p->pair_cnt, 0, ncells * sizeof(uint32_t)) != cudaSuccess) return AUGUR_ECUDA;
    p->pair_cells_cap = ncells;
  }
  int KP = 1;
  while (KP < knn) KP <<= 1;
  if (KP > p->pair_kp) {
    if (p->pair_nbj) {
      cudaFree(p->pair_nbj);
      cudaFree(p->pair_nbq);
      p->bytes -= (size_t)p->max_n * p->pair_kp * 8;
      p->pair_nbj = nullptr;
      p->pair_nbq = nullptr;
    }
    p->pair_kp = 0;
    rc |= dalloc(p, &p->pair_nbj, (size_t)p->max_n * KP);
    rc |= dalloc(p, &p->pair_nbq, (size_t)p->max_n * KP);
    if (rc) return AUGUR_ENOMEM;
    p->pair_kp = KP;
  }
  size_t np = 0;
  if (params) {
    np = (size_t)KMLP_H * ncol + KMLP_H * KMLP_H + 3 * KMLP_H + 1;
    if (cudaMemcpyAsync(p->pair_params, params, np * sizeof(float), cudaMemcpyDefault, st) != cudaSuccess)
      return AUGUR_ECUDA;
  }
  const unsigned nb = blocks_for(n, 256);
  pair_keys_kernel<<<nb, 256, 0, st>>>(pos, mask, n, a, p->pair_key, p->pair_rank, p->pair_cnt);
  AUGUR_LAUNCH_CHECK(p);
  scan_local_kernel<<<ntiles, 1024, 0, st>>>(p->pair_cnt, p->pair_start, p->pair_tsum, (int)ncells);
  AUGUR_LAUNCH_CHECK(p);
  scan_tiles_kernel<<<1, 1024, 0, st>>>(p->pair_tsum, p->pair_toff, ntiles);
  AUGUR_LAUNCH_CHECK(p);
  pair_scatter_kernel<<<nb, 256, 0, st>>>(pos, p->pair_key, p->pair_rank, n, p->pair_start, p->pair_toff,
                                          p->pair_sorted);
  AUGUR_LAUNCH_CHECK(p);
  pair_search_kernel<<<blocks_for(n, 128), 128, 0, st>>>(p->pair_sorted, n, p->pair_start, p->pair_toff, a, KP,
                                                          p->pair_nbj, p->pair_nbq);
  AUGUR_LAUNCH_CHECK(p);
  if (params) {
    // the MLP's 64 x 64 layer on the tensor cores; persistent CTAs over 128-row tiles
    if (raise_dyn_smem((const void *)pair_weight_tc_kernel, PTC_SMEM)) return AUGUR_ECUDA;
    const int sms = current_sm_count();
    const int64_t tiles = (n * KP + PTC_M - 1) / PTC_M;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)std::max(1, sms) * 4);
    pair_weight_tc_kernel<<<grid, PTC_M, PTC_SMEM, st>>>(p->pair_sorted, pos, mass, mask, n, KP, p->pair_nbj,
                                                          p->pair_nbq, p->pair_params, a, acc, p->d_err);
  } else {
    pair_weight_kernel<<<blocks_for(n * KP, 128), 128, 0, st>>>(p->pair_sorted, pos, mass, mask, n, KP, p->pair_nbj,
                                                                p->pair_nbq, nullptr, a, acc);
  }
  AUGUR_LAUNCH_CHECK(p);
  return AUGUR_OK;
}

int augur_pm_plan_bind_force_grid(augur_pm_plan *p, float *grid4) {
  if (!p) return AUGUR_EINVAL;
  if (p->dim != 3 || p->mode != AUGUR_MODE_PERIODIC) return AUGUR_EINVAL;
  if (grid4 && (reinterpret_cast<uintptr_t>(grid4) & 15) != 0) return AUGUR_EINVAL;
  p->F4 = grid4 ? reinterpret_cast<float4 *>(grid4) : p->F4_own;
  return AUGUR_OK;
}

int augur_pm_run_kick(augur_pm_plan *p, float kick, int drift, float *acc_out, double *energy_out, float esync,
                      void *stream) {
  if (!p || p->run_active != 3) return AUGUR_EINVAL;
  if (energy_out && p->ncomp_last < 4) return AUGUR_EINVAL;  // the potential lane is needed
  p->launches = 0;
  int rc = run_gather(p, kick, drift, acc_out, S(stream), energy_out, esync);
  p->run_active = 1;  // a re-sort is due before the next grid
  return rc;
}

int augur_pm_run_unload(augur_pm_plan *p, float *pos, float *vel, void *stream) {
  if (!p || !p->run_active) return AUGUR_EINVAL;
  if (p->run_n > 0 && (!pos || !vel)) return AUGUR_EINVAL;
  p->launches = 0;
  const int64_t n = p->run_n;
  if (n > 0) {
    unsort_kernel<3><<<blocks_for(n, 256), 256, 0, S(stream)>>>(p->pos4[p->cur], p->vel4[p->cur], n, pos, vel);
    AUGUR_LAUNCH_CHECK(p);
  }
  p->run_active = 0;
  return AUGUR_OK;
}

int augur_pm_run_begin(augur_pm_plan *p, const float *pos, const float *vel, const float *mass, const float *mask,
                       int64_t n, float dt, void *stream) {
  int rc = check_plan(p, n);
  if (rc) return rc;
  if (p->mode != AUGUR_MODE_PERIODIC) return AUGUR_EINVAL;
  if (n > 0 && (!pos || !vel || !mass || !mask)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  p->launches = 0;
  p->run_n = n;
  p->run_dt = dt;
  rc = sort_from_aos(p, const_cast<float *>(pos), vel, nullptr, mass, mask, n, false, 0.f, st);
  if (rc) return rc;
  rc = grid_force(p, 3, st);
  if (rc) return rc;
  rc = run_gather(p, (float)(0.5 * (double)dt), 1, nullptr, st);
  if (rc) return rc;
  p->run_active = 1;
  return AUGUR_OK;
}

int augur_pm_run_steps(augur_pm_plan *p, int k, void *stream) {
  if (!p || p->run_active != 1 || k < 0) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  p->launches = 0;
  for (int s = 0; s < k; ++s) {
    int rc = resort(p, st);
    if (rc) return rc;
    rc = grid_force(p, 3, st);
    if (rc) return rc;
    rc = run_gather(p, p->run_dt, 1, nullptr, st);
    if (rc) return rc;
  }
  return AUGUR_OK;
}

int augur_pm_run_profile(augur_pm_plan *p, int k, float *stage_ms, int nstage, void *stream) {
  if (!p || p->run_active != 1 || k < 1 || !stage_ms || nstage < AUGUR_PM_NSTAGE) return AUGUR_EINVAL;
  if (p->mode != AUGUR_MODE_PERIODIC) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  cudaEvent_t ev[AUGUR_PM_NSTAGE + 1];
  for (int i = 0; i <= AUGUR_PM_NSTAGE; ++i)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) return AUGUR_ECUDA;
  double acc[AUGUR_PM_NSTAGE] = {0};
  int rc = AUGUR_OK;
  const int G = p->G, M = p->M;
  for (int s = 0; s < k && rc == AUGUR_OK; ++s) {
    cudaEventRecord(ev[0], st);
    rc = resort(p, st);
    cudaEventRecord(ev[1], st);
    if (!rc) rc = launch_deposit<3, 1>(p, nullptr, p->spec, st);
    cudaEventRecord(ev[2], st);
    if (!rc) rc = fft_rows(p, p->spec, (int64_t)(M + 1) * G, false, st);
    cudaEventRecord(ev[3], st);
    if (!rc) rc = launch_green(p, 3, st);
    cudaEventRecord(ev[4], st);
    if (!rc) rc = fft_rows(p, p->spec3, (int64_t)3 * (M + 1) * G, true, st);
    cudaEventRecord(ev[5], st);
    if (!rc) rc = launch_c2r(p, 3, p->F4, st);
    cudaEventRecord(ev[6], st);
    if (!rc) rc = run_gather(p, p->run_dt, 1, nullptr, st);
    cudaEventRecord(ev[7], st);
    if (cudaEventSynchronize(ev[7]) != cudaSuccess) rc = AUGUR_ECUDA;
    for (int i = 0; i < AUGUR_PM_NSTAGE && rc == AUGUR_OK; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      acc[i] += ms;
    }
  }
  for (int i = 0; i <= AUGUR_PM_NSTAGE; ++i) cudaEventDestroy(ev[i]);
  for (int i = 0; i < AUGUR_PM_NSTAGE; ++i) stage_ms[i] = (float)(acc[i] / k);
  return rc;
}

int augur_pm_run_end(augur_pm_plan *p, float *pos, float *vel, float *acc_out, void *stream) {
  if (!p || p->run_active != 1) return AUGUR_EINVAL;
  if (p->run_n > 0 && (!pos || !vel)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  p->launches = 0;
  int rc = resort(p, st);
  if (rc) return rc;
  rc = grid_force(p, 3, st);
  if (rc) return rc;
  rc = run_gather(p, (float)(0.5 * (double)p->run_dt), 0, acc_out, st);
  if (rc) return rc;
  const int64_t n = p->run_n;
  if (n > 0) {
    unsort_kernel<3><<<blocks_for(n, 256), 256, 0, st>>>(p->pos4[p->cur], p->vel4[p->cur], n, pos, vel);
    AUGUR_LAUNCH_CHECK(p);
  }
  p->run_active = 0;
  return AUGUR_OK;
}

int augur_pm_run(augur_pm_plan *p, float *pos, float *vel, const float *mass, const float *mask, int64_t n, float dt,
                 int nsteps, float *acc_out, void *stream) {
  if (nsteps < 1) return AUGUR_EINVAL;
  int rc = augur_pm_run_begin(p, pos, vel, mass, mask, n, dt, stream);
  if (rc) return rc;
  int64_t total = p->launches;
  rc = augur_pm_run_steps(p, nsteps - 1, stream);
  if (rc) return rc;
  total += p->launches;
  rc = augur_pm_run_end(p, pos, vel, acc_out, stream);
  total += p->launches;
  p->launches = total;
  return rc;
}

int augur_pm_check(augur_pm_plan *p, void *stream) {
  if (!p) return AUGUR_EINVAL;
  if (cudaStreamSynchronize(S(stream)) != cudaSuccess) return AUGUR_ECUDA;
  unsigned e = 0;
  if (cudaMemcpy(&e, p->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return AUGUR_ECUDA;
  if (cudaMemset(p->d_err, 0, sizeof(unsigned)) != cudaSuccess) return AUGUR_ECUDA;
  if (e & AUGUR_ERRBIT_NONFINITE) return AUGUR_EIO;
  if (e & AUGUR_ERRBIT_RANGE) return AUGUR_ERANGE;
  if (e & AUGUR_ERRBIT_TIMEOUT) return AUGUR_ETIMEDOUT;
  return AUGUR_OK;
}

}  // extern "C"

// =====================================================================================
// Batches of scenes: one launch per stage for every scene of the batch
// =====================================================================================
struct augur_pm_batch {
  int ns;
  std::vector<augur_pm_plan *> plans;
  int parity;  // steps taken mod 2: pack set in use
  int green_ty, agg;
  int green_nt;  // threads of the z-transform launch (the largest any scene's grid wants)
  size_t smem_dep, smem_rows, smem_green, smem_c2r;
  int tot_scan, tot_scatter, tot_depcount, tot_dep, tot_rows_f, tot_rows_i, tot_green, tot_c2r, tot_gather;
  int *boff;  // device: 9 tables of ns + 1 block offsets, stage after stage
  ScanPack *scan;
  ScatterPack *scatter;   // [2][ns]
  DepPlanPack *depplan;   // [2][ns] (the plan tables do not depend on the parity; both equal)
  DepPack *dep;           // [2][ns]
  RowsPack *rows_f, *rows_i;
  GreenPack *green;
  C2RPack *c2r;
  GatherPack *gather;     // [2][ns]
  unsigned *d_err;        // not used: every scene reports through its own plan's error word
};

namespace {

enum { BS_SCAN, BS_SCATTER, BS_DEPCOUNT, BS_DEP, BS_ROWS_F, BS_GREEN, BS_ROWS_I, BS_C2R, BS_GATHER, BS_N };

template <typename T>
int batch_upload(T **dst, const std::vector<T> &v) {
  if (cudaMalloc(dst, sizeof(T) * std::max<size_t>(1, v.size())) != cudaSuccess) return AUGUR_ENOMEM;
  if (!v.empty() && cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return AUGUR_ECUDA;
  return AUGUR_OK;
}

void batch_free(augur_pm_batch *b) {
  void *q[] = {b->boff, b->scan, b->scatter, b->depplan, b->dep, b->rows_f, b->rows_i, b->green, b->c2r, b->gather};
  for (void *x : q)
    if (x) cudaFree(x);
}

}  // namespace

extern "C" {

int augur_pm_batch_create(augur_pm_batch **out, augur_pm_plan *const *plans, int nplans) {
  if (!out || !plans || nplans < 1) return AUGUR_EINVAL;
  *out = nullptr;
  augur_pm_batch *b = new (std::nothrow) augur_pm_batch();
  if (!b) return AUGUR_ENOMEM;
  b->ns = nplans;
  b->plans.assign(plans, plans + nplans);
  const int ns = nplans;
  std::vector<int> boff((size_t)BS_N * (ns + 1), 0);
  std::vector<ScanPack> scan(ns);
  std::vector<ScatterPack> scatter(2 * ns);
  std::vector<DepPlanPack> depplan(ns);
  std::vector<DepPack> dep(2 * ns);
  std::vector<RowsPack> rows_f(ns), rows_i(ns);
  std::vector<GreenPack> green(ns);
  std::vector<C2RPack> c2r(ns);
  std::vector<GatherPack> gather(2 * ns);
  int rc = AUGUR_OK;
  for (int i = 0; i < ns && rc == AUGUR_OK; ++i) {
    augur_pm_plan *p = plans[i];
    if (!p || p->mode != AUGUR_MODE_PERIODIC || p->dim != 3 || p->run_active != 1) {
      rc = AUGUR_EINVAL;
      break;
    }
    if (i == 0) {
      b->green_ty = p->green_TY;
      b->green_nt = 0;
      b->agg = p->dep_agg;
    } else if (p->green_TY != b->green_ty || p->dep_agg != b->agg) {
      rc = AUGUR_EINVAL;  // one z-transform tile and one deposit variant per batch
      break;
    }
    const int G = p->G, M = p->M;
    const int64_t n = p->run_n;
    b->green_nt = std::max(b->green_nt, green_threads(G, p->green_TY));
    int cnt[BS_N];
    cnt[BS_SCAN] = p->ntiles;
    cnt[BS_SCATTER] = (int)blocks_for(n, 256);
    cnt[BS_DEPCOUNT] = (int)blocks_for(p->nblk, 256);
    const int64_t items = (int64_t)p->nblk + 4 * dep_nchunks(p, n) + 1;
    if ((size_t)items > p->dep_items_max) {
      rc = AUGUR_ERANGE;
      break;
    }
    cnt[BS_DEP] = (int)items;
    cnt[BS_ROWS_F] = (int)blocks_for((int64_t)(M + 1) * G, p->rows_RB);
    cnt[BS_GREEN] = (M + 1) * (G / p->green_TY);
    cnt[BS_ROWS_I] = (int)blocks_for((int64_t)3 * (M + 1) * G, p->rows_RB);
    cnt[BS_C2R] = G * G / p->c2r_RB;
    cnt[BS_GATHER] = (int)blocks_for(n, 256);
    for (int st = 0; st < BS_N; ++st) boff[(size_t)st * (ns + 1) + i + 1] = boff[(size_t)st * (ns + 1) + i] + cnt[st];
    b->smem_dep = std::max(b->smem_dep, p->smem_dep);
    b->smem_rows = std::max(b->smem_rows, p->smem_rows);
    b->smem_green = std::max(b->smem_green, p->smem_green);
    b->smem_c2r = std::max(b->smem_c2r, p->smem_c2r);

    scan[i] = {p->row_count, p->row_start, p->tile_sum, p->tile_off, p->nrow, p->ntiles};
    const DepositArgs da = dep_args(p);
    depplan[i] = {p->row_start, p->tile_off, da, p->dep_nch, p->dep_item_off, p->dep_slot_off, p->dep_item_blk,
                  p->dep_seg_tab, p->d_err};
    RowsPack rp{};
    rp.data = p->spec;
    rp.nrows = (int64_t)(M + 1) * G;
    rp.RB = p->rows_RB;
    rp.L = p->L;
    rp.twmul = p->Lt / p->L;
    rp.Lt = p->Lt;
    rp.inverse = 0;
    rp.fdL = make_fastdiv(p->L);
    rp.tw = p->tw;
    rows_f[i] = rp;
    rp.data = p->spec3;
    rp.nrows = (int64_t)3 * (M + 1) * G;
    rp.inverse = 1;
    rows_i[i] = rp;
    GreenArgs ga;
    ga.G = G;
    ga.TY = p->green_TY;
    ga.ncomp = 3;
    ga.Lt = p->Lt;
    ga.nbuf = green_nbuf(G);
    ga.fsh = p->sh_L;
    ga.kfund = (float)(2.0 * M_PI / p->extent);
    ga.gfac = (float)(-4.0 * M_PI * p->gnewton / ((double)G * G * G));
    green[i] = {p->spec, ga, p->tw, p->spec3};
    C2RArgs ca{};
    ca.L = G;
    ca.nrows = G * G;
    ca.RB = p->c2r_RB;
    ca.ncomp = 3;
    ca.Lt = p->Lt;
    ca.nkeep = G * G;
    ca.Lkeep = G;
    ca.scale = 1.f;
    ca.fsh = p->sh_M;
    ca.twmul = p->Lt / M;
    ca.fdRB = make_fastdiv(ca.RB);
    ca.fdM = make_fastdiv(ca.L / 2);
    ca.fdL = make_fastdiv(ca.L);
    ca.nbx = (M <= 128 && c2r_smem_bytes(M, ca.RB, G, 3, 2, p->Lt) <= p->smem_c2r) ? 2 : 1;
    c2r[i] = {p->spec3, ca, p->tw, reinterpret_cast<float *>(p->F4)};
    const GatherArgs ga2 = gather_args(p, p->run_dt, p->run_dt, 1);
    for (int par = 0; par < 2; ++par) {
      const int c = p->cur ^ par;  // state buffers before this step's re-sort
      scatter[(size_t)par * ns + i] = {p->pos4[c], p->vel4[c], n, p->key, p->slot, p->row_start, p->tile_off,
                                       p->pos4[c ^ 1], p->vel4[c ^ 1]};
      dep[(size_t)par * ns + i] = {p->pos4[c ^ 1], p->d_mmax, da, p->tw, p->spec, p->d_err, p->dep_item_off,
                                   p->dep_slot_off, p->dep_item_blk, p->dep_seg_tab, p->dep_scratch,
                                   p->dep_counters};
      gather[(size_t)par * ns + i] = {p->F4, p->pos4[c ^ 1], p->vel4[c ^ 1], n, ga2, p->key, p->slot, p->row_count,
                                      p->d_err};
    }
  }
  if (rc == AUGUR_OK) {
    b->tot_scan = boff[(size_t)BS_SCAN * (ns + 1) + ns];
    b->tot_scatter = boff[(size_t)BS_SCATTER * (ns + 1) + ns];
    b->tot_depcount = boff[(size_t)BS_DEPCOUNT * (ns + 1) + ns];
    b->tot_dep = boff[(size_t)BS_DEP * (ns + 1) + ns];
    b->tot_rows_f = boff[(size_t)BS_ROWS_F * (ns + 1) + ns];
    b->tot_green = boff[(size_t)BS_GREEN * (ns + 1) + ns];
    b->tot_rows_i = boff[(size_t)BS_ROWS_I * (ns + 1) + ns];
    b->tot_c2r = boff[(size_t)BS_C2R * (ns + 1) + ns];
    b->tot_gather = boff[(size_t)BS_GATHER * (ns + 1) + ns];
    rc |= batch_upload(&b->boff, boff);
    rc |= batch_upload(&b->scan, scan);
    rc |= batch_upload(&b->scatter, scatter);
    rc |= batch_upload(&b->depplan, depplan);
    rc |= batch_upload(&b->dep, dep);
    rc |= batch_upload(&b->rows_f, rows_f);
    rc |= batch_upload(&b->rows_i, rows_i);
    rc |= batch_upload(&b->green, green);
    rc |= batch_upload(&b->c2r, c2r);
    rc |= batch_upload(&b->gather, gather);
    if (rc) rc = AUGUR_ENOMEM;
  }
  if (rc == AUGUR_OK) {
    rc |= raise_smem(b->agg ? deposit_multi<true> : deposit_multi<false>, b->smem_dep);
    rc |= raise_smem(fft_rows_multi, b->smem_rows);
    rc |= raise_smem(b->green_ty == 16 ? green_multi<16> : green_multi<8>, b->smem_green);
    rc |= raise_smem(c2r_multi, b->smem_c2r);
    if (rc) rc = AUGUR_ECUDA;
  }
  if (rc != AUGUR_OK) {
    batch_free(b);
    delete b;
    return rc;
  }
  *out = b;
  return AUGUR_OK;
}

int augur_pm_batch_destroy(augur_pm_batch *b) {
  if (!b) return AUGUR_OK;
  batch_free(b);
  delete b;
  return AUGUR_OK;
}

int augur_pm_batch_run_steps(augur_pm_batch *b, int k, void *stream) {
  if (!b || k < 0) return AUGUR_EINVAL;
  for (augur_pm_plan *p : b->plans)
    if (p->run_active != 1) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  const int ns = b->ns;
  const int *bo = b->boff;
  auto off = [&](int stage) { return bo + (size_t)stage * (ns + 1); };
  for (int s = 0; s < k; ++s) {
    const int par = b->parity;
    if (b->tot_scan) scan_local_multi<<<b->tot_scan, 1024, 0, st>>>(b->scan, off(BS_SCAN), ns);
    scan_tiles_multi<<<ns, 1024, 0, st>>>(b->scan);
    if (b->tot_scatter)
      scatter_sorted_multi<<<b->tot_scatter, 256, 0, st>>>(b->scatter + (size_t)par * ns, off(BS_SCATTER), ns);
    if (b->tot_depcount) deposit_count_multi<<<b->tot_depcount, 256, 0, st>>>(b->depplan, off(BS_DEPCOUNT), ns);
    deposit_plan_multi<<<ns, 1024, 0, st>>>(b->depplan);
    if (b->agg)
      deposit_multi<true><<<b->tot_dep, DEP_THREADS, b->smem_dep, st>>>(b->dep + (size_t)par * ns, off(BS_DEP), ns);
    else
      deposit_multi<false><<<b->tot_dep, DEP_THREADS, b->smem_dep, st>>>(b->dep + (size_t)par * ns, off(BS_DEP), ns);
    fft_rows_multi<<<b->tot_rows_f, 256, b->smem_rows, st>>>(b->rows_f, off(BS_ROWS_F), ns);
    if (b->green_ty == 16)
      green_multi<16><<<b->tot_green, b->green_nt, b->smem_green, st>>>(b->green, off(BS_GREEN), ns);
    else
      green_multi<8><<<b->tot_green, b->green_nt, b->smem_green, st>>>(b->green, off(BS_GREEN), ns);
    fft_rows_multi<<<b->tot_rows_i, 256, b->smem_rows, st>>>(b->rows_i, off(BS_ROWS_I), ns);
    c2r_multi<<<b->tot_c2r, 512, b->smem_c2r, st>>>(b->c2r, off(BS_C2R), ns);
    if (b->tot_gather)
      gather_multi<<<b->tot_gather, 256, 0, st>>>(b->gather + (size_t)par * ns, off(BS_GATHER), ns);
    if (cudaGetLastError() != cudaSuccess) return AUGUR_ECUDA;
    b->parity ^= 1;
    for (augur_pm_plan *p : b->plans)
      if (p->run_n > 0) p->cur ^= 1;
  }
  return AUGUR_OK;
}

int augur_pm_batch_size(const augur_pm_batch *b) { return b ? b->ns : 0; }

}  // extern "C"
