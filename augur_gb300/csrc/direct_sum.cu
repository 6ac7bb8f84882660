// direct_sum.cu — FP64 softened direct sum (isolated and Ewald-periodic) and the
// compensated energy / momentum reductions.
//
// Direct sum: exact_acc (scripts/scatter_scaling_ops.py:57-72) generalised to D = 2, 3:
//   a_t = sum_j m_j (x_j - x_t) * (|x_j - x_t|^2 + eps^2)^-1.5 , self pair excluded.
// Periodic (box > 0, D = 3): minimum-image softened Newtonian pair force plus the Ewald
// correction (periodic sum minus the nearest-image Newtonian term) for a unit mass,
// tabulated once per device (FP64 sums, stored as fp32) on a 65^3 grid over the positive octant
// of [0, 1/2]^3 and interpolated trilinearly in fp32 (the correction is odd in each displacement
// component); the Newtonian pair sum is FP64 throughout.
// The Ewald sum uses alpha = 2, real-space images |n_i| <= 2, k-space |h|^2 <= 10
// (Hernquist, Bouchet & Suto 1991, ApJS 75, 231).
//
// The targets are split over blocks and the sources over SPLIT chunks; each chunk
// writes a partial sum that a second kernel adds in a fixed order, so results are
// deterministic.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "augur_common.cuh"

namespace {

constexpr int DS_THREADS = 128;
constexpr int DS_TILE = 512;
constexpr int EW_N = 64;  // intervals per axis of the correction table over [0, 1/2]
constexpr int EW_P = EW_N + 1;

__device__ __forceinline__ double wrap_min_image(double d, double box, double inv_box) {
  return d - box * rint(d * inv_box);
}

// Ewald correction for a unit mass at the origin, unit box, displacement x in [0, 1/2]^3.
__global__ void ewald_table_kernel(double *__restrict__ tab) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= EW_P * EW_P * EW_P) return;
  const int iz = e / (EW_P * EW_P), iy = (e / EW_P) % EW_P, ix = e % EW_P;
  const double x[3] = {0.5 * ix / EW_N, 0.5 * iy / EW_N, 0.5 * iz / EW_N};
  const double alpha = 2.0, pi = 3.14159265358979323846;
  double a[3] = {0.0, 0.0, 0.0};
  const double r2x = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  // acceleration of a body at x due to a unit mass at the origin; acceleration points
  // toward the source: a = -sum_n (x - n) / |x - n|^3 [erfc(alpha r) + 2 alpha r / sqrt(pi) exp(-alpha^2 r^2)]
  for (int nx = -2; nx <= 2; ++nx)
    for (int ny = -2; ny <= 2; ++ny)
      for (int nz = -2; nz <= 2; ++nz) {
        double d[3] = {x[0] - nx, x[1] - ny, x[2] - nz};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 == 0.0) continue;
        double r = sqrt(r2);
        double f = (erfc(alpha * r) + 2.0 * alpha * r / sqrt(pi) * exp(-alpha * alpha * r2)) / (r2 * r);
        for (int c = 0; c < 3; ++c) a[c] -= d[c] * f;
      }
  for (int hx = -3; hx <= 3; ++hx)
    for (int hy = -3; hy <= 3; ++hy)
      for (int hz = -3; hz <= 3; ++hz) {
        int h2 = hx * hx + hy * hy + hz * hz;
        if (h2 == 0 || h2 > 10) continue;
        double hd = 2.0 * pi * (hx * x[0] + hy * x[1] + hz * x[2]);
        double f = 2.0 / h2 * exp(-pi * pi * h2 / (alpha * alpha)) * sin(hd);
        a[0] -= hx * f;
        a[1] -= hy * f;
        a[2] -= hz * f;
      }
  // remove the nearest-image Newtonian term -x/|x|^3
  if (r2x > 0.0) {
    double r3 = r2x * sqrt(r2x);
    for (int c = 0; c < 3; ++c) a[c] += x[c] / r3;
  } else {
    a[0] = a[1] = a[2] = 0.0;
  }
  for (int c = 0; c < 3; ++c) tab[(size_t)e * 3 + c] = a[c];
}

// The Ewald correction is interpolated in fp32 from an fp32 copy of the table: it is a small part
// of the force (its size relative to the Newtonian sum is below ~1e-1 in these scenes), so fp32's
// relative rounding (~1e-7) moves the total by ~1e-8, below the table's own interpolation error
// (~1e-6), while FP64 arithmetic on this part runs several times slower.
__device__ __forceinline__ void ewald_corr(const float *__restrict__ tab, const double d[3], double inv_box,
                                           double out[3]) {
  // d is the minimum-image displacement source - target: the acceleration of the
  // target is the unit-box correction evaluated at u = (target - source)/box, scaled by 1/box^2
  float u[3], s[3];
  for (int c = 0; c < 3; ++c) {
    const float t = (float)(-d[c] * inv_box);
    s[c] = t < 0.f ? -1.f : 1.f;
    u[c] = fminf(fabsf(t) * (2.f * EW_N), (float)EW_N);
  }
  int i[3];
  float f[3];
  for (int c = 0; c < 3; ++c) {
    int k = (int)u[c];
    if (k >= EW_N) k = EW_N - 1;
    i[c] = k;
    f[c] = u[c] - (float)k;
  }
  float r[3] = {0.f, 0.f, 0.f};
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const float w = (dx ? f[0] : 1.f - f[0]) * (dy ? f[1] : 1.f - f[1]) * (dz ? f[2] : 1.f - f[2]);
        const size_t e = ((size_t)(i[2] + dz) * EW_P + (i[1] + dy)) * EW_P + (i[0] + dx);
        for (int c = 0; c < 3; ++c) r[c] += w * __ldg(&tab[e * 3 + c]);
      }
  const double inv_b2 = inv_box * inv_box;
  for (int c = 0; c < 3; ++c) out[c] = (double)(s[c] * r[c]) * inv_b2;
}

__global__ void to_f32_kernel(const double *__restrict__ in, int n, float *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) out[e] = (float)in[e];
}

template <int D, bool PERIODIC>
__global__ void __launch_bounds__(DS_THREADS) direct_sum_partial_kernel(
    const double *__restrict__ tg, const int64_t *__restrict__ tidx, int64_t T, const double *__restrict__ src,
    const double *__restrict__ mass, int64_t N, int64_t chunk, double eps2, double box,
    const float *__restrict__ ewtab, double *__restrict__ partial) {
  __shared__ double sp[DS_TILE][4];
  const int64_t t = (int64_t)blockIdx.x * DS_THREADS + threadIdx.x;
  const int64_t s0 = (int64_t)blockIdx.y * chunk;
  const int64_t s1 = min(N, s0 + chunk);
  double x[3] = {0.0, 0.0, 0.0};
  int64_t self = -1;
  if (t < T) {
    for (int d = 0; d < D; ++d) x[d] = tg[t * D + d];
    if (tidx) self = tidx[t];
  }
  double a[3] = {0.0, 0.0, 0.0};
  const double inv_box = PERIODIC ? 1.0 / box : 0.0;
  for (int64_t b = s0; b < s1; b += DS_TILE) {
    const int nb = (int)min((int64_t)DS_TILE, s1 - b);
    __syncthreads();
    for (int k = threadIdx.x; k < nb; k += DS_THREADS) {
      for (int d = 0; d < 3; ++d) sp[k][d] = d < D ? src[(b + k) * D + d] : 0.0;
      sp[k][3] = mass ? mass[b + k] : 1.0;
    }
    __syncthreads();
    if (t < T) {
      for (int k = 0; k < nb; ++k) {
        if (b + k == self) continue;
        double d[3];
        for (int c = 0; c < 3; ++c) d[c] = sp[k][c] - x[c];
        if (PERIODIC)
          for (int c = 0; c < 3; ++c) d[c] = wrap_min_image(d[c], box, inv_box);
        double r2 = d[0] * d[0] + d[1] * d[1] + (D == 3 ? d[2] * d[2] : 0.0) + eps2;
        double inv = rsqrt(r2);
        double f = sp[k][3] * inv * inv * inv;
        for (int c = 0; c < D; ++c) a[c] += d[c] * f;
        if (PERIODIC) {
          double cr[3];
          ewald_corr(ewtab, d, inv_box, cr);
          for (int c = 0; c < 3; ++c) a[c] += sp[k][3] * cr[c];
        }
      }
    }
  }
  if (t < T)
    for (int c = 0; c < D; ++c) partial[((size_t)blockIdx.y * T + t) * D + c] = a[c];
}

__global__ void sum_partials_kernel(const double *__restrict__ partial, int split, int64_t m, double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  double s = 0.0;
  for (int k = 0; k < split; ++k) s += partial[(size_t)k * m + e];
  out[e] = s;
}

float *g_ewald[64] = {nullptr};
std::mutex g_ewald_mu;

// The correction table of the current device (fp32 copy of the FP64-evaluated sums), built once
// per device; a device reset in the process makes the cached pointer stale.
int ewald_table(float **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return AUGUR_ECUDA;
  std::lock_guard<std::mutex> lk(g_ewald_mu);
  if (!g_ewald[dev]) {
    const int n = EW_P * EW_P * EW_P;
    double *t = nullptr;
    float *t32 = nullptr;
    if (cudaMalloc(&t, sizeof(double) * 3 * n) != cudaSuccess) return AUGUR_ENOMEM;
    if (cudaMalloc(&t32, sizeof(float) * 3 * n) != cudaSuccess) {
      cudaFree(t);
      return AUGUR_ENOMEM;
    }
    ewald_table_kernel<<<(n + 127) / 128, 128>>>(t);
    to_f32_kernel<<<(3 * n + 255) / 256, 256>>>(t, 3 * n, t32);
    const bool ok = cudaDeviceSynchronize() == cudaSuccess;
    cudaFree(t);
    if (!ok) {
      cudaFree(t32);
      return AUGUR_ECUDA;
    }
    g_ewald[dev] = t32;
  }
  *out = g_ewald[dev];
  return AUGUR_OK;
}

// ---- compensated reductions ---------------------------------------------------------
constexpr int EN_THREADS = 256;
constexpr int EN_PER_THREAD = 32;
constexpr int EN_Q = 6;  // ke, px, py, pz, mass, pe

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ double value() const { return (double)s - (double)c; }
};

template <int D>
__global__ void __launch_bounds__(EN_THREADS) energy_partial_kernel(const float *__restrict__ vel,
                                                                    const float *__restrict__ mass,
                                                                    const float *__restrict__ mask,
                                                                    const float *__restrict__ phi, int64_t n,
                                                                    double *__restrict__ partial) {
  __shared__ double red[EN_Q][EN_THREADS / 32];
  const int64_t b0 = ((int64_t)blockIdx.x * EN_THREADS + threadIdx.x) * EN_PER_THREAD;
  Kahan k[EN_Q];
  for (int j = 0; j < EN_PER_THREAD; ++j) {
    int64_t i = b0 + j;
    if (i >= n) break;
    float m = __fmul_rn(mass[i], mask[i]);
    float v2 = 0.f;
    for (int d = 0; d < D; ++d) {
      float v = vel[i * D + d];
      v2 = __fadd_rn(v2, __fmul_rn(v, v));
      k[1 + d].add(__fmul_rn(m, v));
    }
    k[0].add(0.5f * __fmul_rn(m, v2));
    k[4].add(m);
    if (phi) k[5].add(0.5f * __fmul_rn(m, phi[i]));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < EN_Q; ++q) {
    double v = k[q].value();
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[q][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < EN_Q) {
    double s = 0.0;
    for (int w = 0; w < EN_THREADS / 32; ++w) s += red[threadIdx.x][w];
    partial[(size_t)blockIdx.x * EN_Q + threadIdx.x] = s;
  }
}

// Fixed-order fold of the per-block partials: thread t sums a contiguous chunk of blocks
// (Neumaier-compensated), then a fixed shared-memory tree -- deterministic and parallel (a
// serial FP64 chain over ~10^4 partials takes milliseconds on this part).
constexpr int EN_FOLD = 256;
template <int D>
__global__ void __launch_bounds__(EN_FOLD) energy_final_kernel(const double *__restrict__ partial, int nblk,
                                                              double *__restrict__ out) {
  __shared__ double sh[EN_Q][EN_FOLD];
  const int t = threadIdx.x;
  const int per = (nblk + EN_FOLD - 1) / EN_FOLD;
  const int b0 = min(nblk, t * per), b1 = min(nblk, b0 + per);
  for (int q = 0; q < EN_Q; ++q) {
    double s = 0.0, c = 0.0;
    for (int b = b0; b < b1; ++b) {
      const double v = partial[(size_t)b * EN_Q + q];
      const double u = s + v;
      c += (fabs(s) >= fabs(v)) ? (s - u) + v : (v - u) + s;
      s = u;
    }
    sh[q][t] = s + c;
  }
  __syncthreads();
  for (int w = EN_FOLD / 2; w > 0; w >>= 1) {
    if (t < w)
      for (int q = 0; q < EN_Q; ++q) sh[q][t] += sh[q][t + w];
    __syncthreads();
  }
  if (t < EN_Q) {
    const int q = t;
    const double s = sh[q][0];
    // out layout: ke, p[0..D-1], mass, pe
    if (q == 0) out[0] = s;
    else if (q <= 3) {
      if (q - 1 < D) out[q] = s;
    } else if (q == 4) out[D + 1] = s;
    else out[D + 2] = s;
  }
}

// ---- allocation-free variant ------------------------------------------------------------
// Scratch for the per-chunk partial sums of augur_direct_sum_fp64_noalloc: one file-scope
// device array (4 MiB) that every GPU loading this library keeps until the process exits.
constexpr int64_t DS_NOALLOC_DOUBLES = (int64_t)1 << 19;
static __device__ __align__(256) double g_ds_noalloc_scratch[DS_NOALLOC_DOUBLES];

double *g_ds_noalloc_ptr[64] = {nullptr};
std::mutex g_ds_noalloc_mu;

// Device address of the scratch array on the current device. In host code the array's name is
// only a host-side stand-in, so the address comes from cudaGetSymbolAddress, once per device.
int noalloc_scratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return AUGUR_ECUDA;
  std::lock_guard<std::mutex> lk(g_ds_noalloc_mu);
  if (!g_ds_noalloc_ptr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress((void **)&p, g_ds_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return AUGUR_ECUDA;
    }
    g_ds_noalloc_ptr[dev] = p;
  }
  *out = g_ds_noalloc_ptr[dev];
  return AUGUR_OK;
}

}  // namespace

extern "C" {

int augur_direct_sum_fp64_noalloc(const double *targets, const int64_t *t_idx, int64_t T, const double *sources,
                                  const double *mass, int64_t N, int dim, double eps, double *acc_out,
                                  void *stream) {
  if (T < 0 || N < 0 || (dim != 2 && dim != 3) || !(eps >= 0.0)) return AUGUR_EINVAL;
  if (T == 0) return AUGUR_OK;
  if (!targets || !acc_out || (N > 0 && !sources)) return AUGUR_EINVAL;
  if (T * dim > DS_NOALLOC_DOUBLES) return AUGUR_ERANGE;  // more targets than the scratch holds
  double *partial = nullptr;
  int rc = noalloc_scratch(&partial);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t tblocks = (T + DS_THREADS - 1) / DS_THREADS;
  int split = (int)std::max<int64_t>(1, std::min<int64_t>(64, 1216 / std::max<int64_t>(1, tblocks)));
  if (N < (int64_t)split * DS_TILE) split = (int)std::max<int64_t>(1, N / DS_TILE);
  split = (int)std::max<int64_t>(1, std::min<int64_t>(split, DS_NOALLOC_DOUBLES / (T * dim)));
  const int64_t chunk = N > 0 ? (N + split - 1) / split : 1;
  // every partial slot read below is written by the first kernel: nothing needs clearing
  dim3 grid((unsigned)tblocks, (unsigned)split);
  const double eps2 = eps * eps;
  if (dim == 3)
    direct_sum_partial_kernel<3, false><<<grid, DS_THREADS, 0, st>>>(targets, t_idx, T, sources, mass, N, chunk,
                                                                     eps2, 0.0, nullptr, partial);
  else
    direct_sum_partial_kernel<2, false><<<grid, DS_THREADS, 0, st>>>(targets, t_idx, T, sources, mass, N, chunk,
                                                                     eps2, 0.0, nullptr, partial);
  const int64_t m = T * dim;
  sum_partials_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(partial, split, m, acc_out);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_direct_sum_fp64(const double *targets, const int64_t *t_idx, int64_t T, const double *sources,
                          const double *mass, int64_t N, int dim, double eps, double box, double *acc_out,
                          void *stream) {
  if (T < 0 || N < 0 || (dim != 2 && dim != 3) || !(eps >= 0.0)) return AUGUR_EINVAL;
  if (box > 0.0 && dim != 3) return AUGUR_EINVAL;
  if (T == 0) return AUGUR_OK;
  if (!targets || !acc_out || (N > 0 && !sources)) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const float *ewtab = nullptr;
  if (box > 0.0) {
    float *t = nullptr;
    int rc = ewald_table(&t);
    if (rc) return rc;
    ewtab = t;
  }
  const int64_t tblocks = (T + DS_THREADS - 1) / DS_THREADS;
  int split = (int)std::max<int64_t>(1, std::min<int64_t>(64, 1216 / std::max<int64_t>(1, tblocks)));
  if (N < (int64_t)split * DS_TILE) split = (int)std::max<int64_t>(1, N / DS_TILE);
  const int64_t chunk = N > 0 ? (N + split - 1) / split : 1;
  double *partial = nullptr;
  const size_t pbytes = sizeof(double) * (size_t)split * T * dim;
  if (cudaMallocAsync(&partial, pbytes, st) != cudaSuccess) return AUGUR_ENOMEM;
  dim3 grid((unsigned)tblocks, (unsigned)split);
  const double eps2 = eps * eps;
  if (dim == 3) {
    if (box > 0.0)
      direct_sum_partial_kernel<3, true><<<grid, DS_THREADS, 0, st>>>(targets, t_idx, T, sources, mass, N, chunk,
                                                                      eps2, box, ewtab, partial);
    else
      direct_sum_partial_kernel<3, false><<<grid, DS_THREADS, 0, st>>>(targets, t_idx, T, sources, mass, N, chunk,
                                                                       eps2, 0.0, nullptr, partial);
  } else {
    direct_sum_partial_kernel<2, false><<<grid, DS_THREADS, 0, st>>>(targets, t_idx, T, sources, mass, N, chunk,
                                                                     eps2, 0.0, nullptr, partial);
  }
  const int64_t m = T * dim;
  sum_partials_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(partial, split, m, acc_out);
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(partial, st);
  return e == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_energy_fp64(const float *vel, const float *mass, const float *mask, const float *phi, int64_t n, int dim,
                      double *out, void *stream) {
  if (n < 0 || (dim != 2 && dim != 3) || !out) return AUGUR_EINVAL;
  if (n > 0 && (!vel || !mass || !mask)) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t per_blk = (int64_t)EN_THREADS * EN_PER_THREAD;
  const int nblk = (int)std::max<int64_t>(1, (n + per_blk - 1) / per_blk);
  double *partial = nullptr;
  if (cudaMallocAsync(&partial, sizeof(double) * EN_Q * nblk, st) != cudaSuccess) return AUGUR_ENOMEM;
  if (dim == 3) {
    energy_partial_kernel<3><<<nblk, EN_THREADS, 0, st>>>(vel, mass, mask, phi, n, partial);
    energy_final_kernel<3><<<1, EN_FOLD, 0, st>>>(partial, nblk, out);
  } else {
    energy_partial_kernel<2><<<nblk, EN_THREADS, 0, st>>>(vel, mass, mask, phi, n, partial);
    energy_final_kernel<2><<<1, EN_FOLD, 0, st>>>(partial, nblk, out);
  }
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(partial, st);
  return e == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

}  // extern "C"
