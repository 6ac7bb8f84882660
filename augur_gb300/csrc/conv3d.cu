// conv3d.cu — the scatter-field grid CNN on sm_103a.
//
// Network (the reference's LocalNet, scripts/scatter_field.py:15-26, in 3D with
// Conv3d 3x3x3, zero padding 1, widths 2 -> 32 -> 32 -> 32 -> 32 -> 3):
//   z0 = conv_in(x) ; h0 = gelu(z0)
//   z_l = conv_l(h_{l-1}) ; h_l = h_{l-1} + gelu(z_l)      l = 1..3
//   y = conv_out(h3)                                     (zero-initialised, :135-136)
// gelu is the exact erf form (torch.nn.functional.gelu default). Activations are
// channels-last BF16, [B][G][G][G][C]; accumulation is FP32.
//
// The 32-channel layers (forward, and the data gradient of the backward pass) run as an
// implicit GEMM on the tcgen05 tensor cores: one CTA tile is M = 128 voxels of one x row,
// N = output channels, K = 27 taps x input channels, accumulated in TMEM. For each (dz, dy)
// tap pair one 130-voxel input slab is copied to shared memory (cp.async, zero-filled
// outside the grid); the three dx taps are the same slab shifted by one 16-byte row, which
// the no-swizzle K-major operand layout [8-channel block][row][16 B] expresses as a
// descriptor start-address offset. The weights stay in shared memory for the CTA's life.
// The 2-channel input layer and the weight gradients run on the CUDA cores.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "augur_common.cuh"
#include "tcgen05.cuh"

using bf16 = __nv_bfloat16;

namespace augur {

constexpr int CONV_M = 128;   // voxels per tile (one x segment)
constexpr int SLAB = CONV_M + 2;
constexpr int CONV_THREADS = 128;
constexpr uint32_t WAIT_BUDGET = 1u << 20;

enum { EPI_FWD = 0, EPI_OUT = 1, EPI_BWD = 2 };

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752440f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  const float phi = 0.39894228040143267794f * expf(-0.5f * x * x);
  return 0.5f * (1.f + erff(x * 0.70710678118654752440f)) + x * phi;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;  // zero-fill when invalid
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

struct ConvArgs {
  int B, G;
  int xseg;          // ceil(G / 128)
  int yc;            // y rows per work unit
  int nyc;           // ceil(G / yc)
  int nunits;        // B * G * xseg * nyc
  float out_scale;   // EPI_OUT: added field = out_scale * (acc + bias)
};

constexpr int RING = 5;  // y rows of input slabs kept per z plane (rows y-1 .. y+2 plus one being freed)

// ---------------------------------------------------------------------------------------
// tcgen05 implicit-GEMM 3x3x3 conv. CIN in {16, 32}, N in {16, 32}.
//   EPI_FWD: z = acc + b ; h = h_in + gelu(z)         out0 = h (bf16), out1 = z (bf16, optional)
//   EPI_OUT: y = out_scale * (acc + b)[0..2]          out0 = F (float4 grid, y added to lanes 0..2)
//   EPI_BWD: g = acc + resid (fp32, optional)         out0 = g (fp32), out1 = g * gelu'(zprev) (bf16)
//
// Work unit = (batch, z, x segment, chunk of yc consecutive y rows). The CTA walks y inside
// the unit keeping a ring of RING input rows per z plane in shared memory, so each new tile
// loads one y row for each of the three z planes (prefetched one tile ahead with cp.async);
// the 54 MMAs of tile y go to TMEM accumulator y & 1 while the epilogue of tile y-1 reads
// the other one.
// ---------------------------------------------------------------------------------------
template <int CIN, int N, int EPI>
__global__ void __launch_bounds__(CONV_THREADS, 1) conv_tc_kernel(const bf16 *__restrict__ in,
                                                                  const bf16 *__restrict__ wB,
                                                                  const float *__restrict__ bias,
                                                                  const void *__restrict__ resid,
                                                                  const bf16 *__restrict__ zprev,
                                                                  void *__restrict__ out0, bf16 *__restrict__ out1,
                                                                  ConvArgs a, unsigned *__restrict__ err) {
  constexpr int CB = CIN / 8;                  // 16-byte channel blocks per voxel
  constexpr int KSTEP_PER_TAP = CIN / 16;      // K = 16 per MMA
  constexpr int WBYTES = 27 * CIN * N * 2;     // weights, UMMA B layout
  constexpr int SLAB_BYTES = CB * SLAB * 16;
  constexpr int SLAB_STRIDE = ((SLAB_BYTES + 127) / 128) * 128;
  constexpr uint32_t IDESC = idesc_bf16_f32(CONV_M, N);
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sW = smem;
  unsigned char *sSlab = smem + ((WBYTES + 127) / 128) * 128;  // [3 z planes][RING rows]
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_tmem;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = a.G;
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(wB);
    uint4 *dst = reinterpret_cast<uint4 *>(sW);
    for (int e = tid; e < WBYTES / 16; e += CONV_THREADS) dst[e] = src[e];
  }
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, 64);  // two 32-column accumulators
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t slab0 = smem_u32(sSlab);
  const uint32_t w_addr = smem_u32(sW);
  uint32_t commits[2] = {0, 0};
  bool ok = true;

  auto slab_addr = [&](int dz, int row) -> uint32_t {
    return slab0 + (uint32_t)((dz * RING + ((row + RING) % RING)) * SLAB_STRIDE);
  };
  // copy input row (z + dz - 1, row) of x segment x0 into its ring slot (zero outside the grid)
  auto load_row = [&](size_t bbase, int z, int x0, int row) {
    for (int c = tid; c < 3 * SLAB * CB; c += CONV_THREADS) {
      const int dz = c / (SLAB * CB);
      const int rem = c - dz * SLAB * CB;
      const int r = rem / CB, cb = rem - r * CB;
      const int zz = z + dz - 1, xx = x0 - 1 + r;
      const bool v = zz >= 0 && zz < G && row >= 0 && row < G && xx >= 0 && xx < G;
      const bf16 *src = v ? in + (bbase + ((size_t)zz * G + row) * G + xx) * CIN + cb * 8 : in;
      cp_async16(slab_addr(dz, row) + (uint32_t)(cb * SLAB + r) * 16u, src, v);
    }
  };
  // epilogue of the tile at (bbase, z, y, x0) from accumulator acc_sel
  auto epilogue = [&](size_t bbase, int z, int y, int x0, int acc_sel) {
    tc_fence_after();
    float acc[32];
    tmem_ld32(tmem + (uint32_t)(acc_sel * 32) + ((uint32_t)(warp * 32) << 16), acc);
    const int x = x0 + warp * 32 + lane;
    if (x < G) {
      const size_t vox = bbase + ((size_t)z * G + y) * G + x;
      if constexpr (EPI == EPI_FWD) {
        const bf16 *hin = reinterpret_cast<const bf16 *>(resid) + vox * N;
        bf16 *hout = reinterpret_cast<bf16 *>(out0) + vox * N;
#pragma unroll
        for (int n = 0; n < N; n += 8) {
          uint4 hv = *reinterpret_cast<const uint4 *>(hin + n);
          const __nv_bfloat162 *hp = reinterpret_cast<const __nv_bfloat162 *>(&hv);
          __align__(16) __nv_bfloat162 ho[4], zo[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float z0 = acc[n + 2 * q] + bias[n + 2 * q], z1 = acc[n + 2 * q + 1] + bias[n + 2 * q + 1];
            ho[q] = __floats2bfloat162_rn(__bfloat162float(hp[q].x) + gelu_f(z0),
                                          __bfloat162float(hp[q].y) + gelu_f(z1));
            zo[q] = __floats2bfloat162_rn(z0, z1);
          }
          *reinterpret_cast<uint4 *>(hout + n) = *reinterpret_cast<uint4 *>(ho);
          if (out1) *reinterpret_cast<uint4 *>(out1 + vox * N + n) = *reinterpret_cast<uint4 *>(zo);
        }
      } else if constexpr (EPI == EPI_OUT) {
        float4 *F = reinterpret_cast<float4 *>(out0) + vox;
        float4 f = *F;
        f.x += a.out_scale * (acc[0] + bias[0]);
        f.y += a.out_scale * (acc[1] + bias[1]);
        f.z += a.out_scale * (acc[2] + bias[2]);
        *F = f;
      } else {
        const float *rin = reinterpret_cast<const float *>(resid);
        float *gout = reinterpret_cast<float *>(out0) + vox * N;
#pragma unroll
        for (int n = 0; n < N; n += 4) {
          float4 g = make_float4(acc[n], acc[n + 1], acc[n + 2], acc[n + 3]);
          if (rin) {
            const float4 r = *reinterpret_cast<const float4 *>(rin + vox * N + n);
            g.x += r.x;
            g.y += r.y;
            g.z += r.z;
            g.w += r.w;
          }
          *reinterpret_cast<float4 *>(gout + n) = g;
          if (out1) {
            const __nv_bfloat162 z01 = *reinterpret_cast<const __nv_bfloat162 *>(zprev + vox * N + n);
            const __nv_bfloat162 z23 = *reinterpret_cast<const __nv_bfloat162 *>(zprev + vox * N + n + 2);
            __align__(8) __nv_bfloat162 o[2];
            o[0] = __floats2bfloat162_rn(g.x * gelu_grad(__bfloat162float(z01.x)),
                                         g.y * gelu_grad(__bfloat162float(z01.y)));
            o[1] = __floats2bfloat162_rn(g.z * gelu_grad(__bfloat162float(z23.x)),
                                         g.w * gelu_grad(__bfloat162float(z23.y)));
            *reinterpret_cast<uint2 *>(out1 + vox * N + n) = *reinterpret_cast<uint2 *>(o);
          }
        }
      }
    }
  };

  for (int unit = blockIdx.x; unit < a.nunits && ok; unit += gridDim.x) {
    int t = unit;
    const int yc = t % a.nyc;
    t /= a.nyc;
    const int xs = t % a.xseg;
    t /= a.xseg;
    const int z = t % G;
    const int b = t / G;
    const int x0 = xs * CONV_M;
    const size_t bbase = (size_t)b * G * G * G;
    const int ya = yc * a.yc, yb = min(G, ya + a.yc);
    // warm-up: rows ya-1, ya, ya+1
    load_row(bbase, z, x0, ya - 1);
    load_row(bbase, z, x0, ya);
    load_row(bbase, z, x0, ya + 1);
    asm volatile("cp.async.commit_group;" ::: "memory");
    for (int y = ya; y < yb; ++y) {
      // prefetch the row the next tile adds (its slot last served tile y-2, finished below)
      load_row(bbase, z, x0, y + 2);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 1;" ::: "memory");
      fence_async_smem();
      __syncthreads();
      const int sel = y & 1;
      if (tid == 0) {
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(sel * 32);
#pragma unroll 1
        for (int pz = 0; pz < 3; ++pz) {
#pragma unroll 1
          for (int py = 0; py < 3; ++py) {
            const uint32_t sa = slab_addr(pz, y + py - 1);
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) {
              const int tap = (pz * 3 + py) * 3 + dx;
#pragma unroll
              for (int kc = 0; kc < KSTEP_PER_TAP; ++kc) {
                const uint64_t ad = smem_desc(sa + (uint32_t)(2 * kc * SLAB * 16 + dx * 16), SLAB * 16, 128);
                const int s = tap * KSTEP_PER_TAP + kc;
                const uint64_t bd = smem_desc(w_addr + (uint32_t)(2 * s * N * 16), N * 16, 128);
                umma_bf16(d, ad, bd, IDESC, (pz | py | dx | kc) ? 1u : 0u);
              }
            }
          }
        }
        umma_commit(&mbar[sel]);
      }
      commits[sel]++;
      if (y > ya) {  // epilogue of the previous tile while this tile's MMAs run
        const int ps = sel ^ 1;
        const bool got = mbar_wait_bounded(&mbar[ps], (commits[ps] - 1) & 1, WAIT_BUDGET);
        if (__syncthreads_or(!got)) {  // the give-up decision is the same in every thread
          ok = false;
          break;
        }
        epilogue(bbase, z, y - 1, x0, ps);
      }
      tc_fence_before();
      __syncthreads();
    }
    if (!ok) break;
    // last tile of the unit
    const int ls = (yb - 1) & 1;
    const bool got = mbar_wait_bounded(&mbar[ls], (commits[ls] - 1) & 1, WAIT_BUDGET);
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    epilogue(bbase, z, yb - 1, x0, ls);
    asm volatile("cp.async.wait_all;" ::: "memory");  // the unit's last prefetch (beyond the chunk)
    tc_fence_before();
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
    for (int bb = 0; bb < 2; ++bb)
      if (commits[bb] > 0) mbar_wait_bounded(&mbar[bb], (commits[bb] - 1) & 1, WAIT_BUDGET);
    asm volatile("cp.async.wait_all;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 64);
  }
}

// ---------------------------------------------------------------------------------------
// Input layer on the CUDA cores: x (B, G^3, 2) bf16 -> z0 (bf16), h0 = gelu(z0) (bf16), 32 ch.
// Weights w[n][tap][c] fp32 (27 * 2 * 32) + bias[32].
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) conv_in_kernel(const bf16 *__restrict__ x, const float *__restrict__ w,
                                                      const float *__restrict__ bias, int B, int G,
                                                      bf16 *__restrict__ z0, bf16 *__restrict__ h0) {
  __shared__ float sw[27 * 2 * 32 + 32];
  for (int e = threadIdx.x; e < 27 * 2 * 32; e += blockDim.x) sw[e] = w[e];
  if (threadIdx.x < 32) sw[27 * 64 + threadIdx.x] = bias[threadIdx.x];
  __syncthreads();
  const int64_t nv = (int64_t)B * G * G * G;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = v;
    const int xx = (int)(t % G);
    t /= G;
    const int yy = (int)(t % G);
    t /= G;
    const int zz = (int)(t % G);
    const int64_t b = t / G;
    float in[27][2];
#pragma unroll
    for (int tap = 0; tap < 27; ++tap) {
      const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
      const int z = zz + dz, y = yy + dy, xq = xx + dx;
      if (z >= 0 && z < G && y >= 0 && y < G && xq >= 0 && xq < G) {
        __nv_bfloat162 p = *reinterpret_cast<const __nv_bfloat162 *>(x + (((b * G + z) * G + y) * G + xq) * 2);
        in[tap][0] = __bfloat162float(p.x);
        in[tap][1] = __bfloat162float(p.y);
      } else {
        in[tap][0] = in[tap][1] = 0.f;
      }
    }
    for (int n = 0; n < 32; n += 2) {
      float s0 = sw[27 * 64 + n], s1 = sw[27 * 64 + n + 1];
#pragma unroll
      for (int tap = 0; tap < 27; ++tap) {
        s0 += sw[(n * 27 + tap) * 2] * in[tap][0] + sw[(n * 27 + tap) * 2 + 1] * in[tap][1];
        s1 += sw[((n + 1) * 27 + tap) * 2] * in[tap][0] + sw[((n + 1) * 27 + tap) * 2 + 1] * in[tap][1];
      }
      *reinterpret_cast<__nv_bfloat162 *>(z0 + v * 32 + n) = __floats2bfloat162_rn(s0, s1);
      *reinterpret_cast<__nv_bfloat162 *>(h0 + v * 32 + n) = __floats2bfloat162_rn(gelu_f(s0), gelu_f(s1));
    }
  }
}

// ---------------------------------------------------------------------------------------
// Weight gradient on the CUDA cores: dW[n][tap][c] = sum_v dz[v][n] * h[v + tap][c]
// (zero padding), partial sums per CTA over x rows, reduced in a fixed order afterwards.
// h: (B, G^3, CIN) bf16 ; dz: (B, G^3, N) as bf16 (DZ_F32 = 0) or fp32 (DZ_F32 = 1).
// One thread per (n, c) pair keeps 27 tap sums in registers. Also accumulates the bias
// gradient sum_v dz[v][n] (threads with c == 0).
// ---------------------------------------------------------------------------------------
template <int CIN, int N, int DZ_F32>
__global__ void __launch_bounds__(CIN * N) wgrad_kernel(const bf16 *__restrict__ h, const void *__restrict__ dz,
                                                        int B, int G, int rows_per_cta,
                                                        float *__restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem[];
  float *sh = reinterpret_cast<float *>(smem);            // [9][G + 2][CIN]
  float *sd = sh + (size_t)9 * (G + 2) * CIN;             // [G][N]
  const int tid = threadIdx.x;
  const int n = tid / CIN, c = tid % CIN;
  float acc[27];
#pragma unroll
  for (int t = 0; t < 27; ++t) acc[t] = 0.f;
  float bacc = 0.f;
  const int nrows = B * G * G;
  const int r0 = blockIdx.x * rows_per_cta, r1 = min(nrows, r0 + rows_per_cta);
  for (int row = r0; row < r1; ++row) {
    const int y = row % G, z = (row / G) % G, b = row / (G * G);
    __syncthreads();
    for (int e = tid; e < 9 * (G + 2) * CIN; e += blockDim.x) {
      const int cc = e % CIN, xr = (e / CIN) % (G + 2), p = e / (CIN * (G + 2));
      const int zz = z + p / 3 - 1, yy = y + p % 3 - 1, xx = xr - 1;
      float v = 0.f;
      if (zz >= 0 && zz < G && yy >= 0 && yy < G && xx >= 0 && xx < G)
        v = __bfloat162float(h[((((size_t)b * G + zz) * G + yy) * G + xx) * CIN + cc]);
      sh[e] = v;
    }
    for (int e = tid; e < G * N; e += blockDim.x) {
      const size_t idx = (((size_t)b * G + z) * G + y) * G * N + e;
      sd[e] = DZ_F32 ? reinterpret_cast<const float *>(dz)[idx]
                     : __bfloat162float(reinterpret_cast<const bf16 *>(dz)[idx]);
    }
    __syncthreads();
    for (int x = 0; x < G; ++x) {
      const float g = sd[x * N + n];
      if (c == 0) bacc += g;
#pragma unroll
      for (int p = 0; p < 9; ++p) {
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) acc[p * 3 + dx] += g * sh[(p * (G + 2) + x + dx) * CIN + c];
      }
    }
  }
  float *out = partial + (size_t)blockIdx.x * (N * 27 * CIN + N);
#pragma unroll
  for (int t = 0; t < 27; ++t) out[(n * 27 + t) * CIN + c] = acc[t];
  if (c == 0) out[N * 27 * CIN + n] = bacc;
}

__global__ void reduce_partials_kernel(const float *__restrict__ partial, int nparts, int len,
                                       float *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  float s = 0.f;
  for (int k = 0; k < nparts; ++k) s += partial[(size_t)k * len + e];
  out[e] = s;
}

// ---------------------------------------------------------------------------------------
// Weight preparation: fp32 w[n][tap][c] (n < Nreal, c < Creal) -> bf16 UMMA B operand
// [k/8][N][8] with k = tap * CIN + c (zero padded to CIN x N). flip = 1 builds the data-
// gradient operand: B'[c][k' = tap * Nreal_in + n] = w[n][26 - tap][c] (roles swapped).
// ---------------------------------------------------------------------------------------
__global__ void prep_weights_kernel(const float *__restrict__ w, int Nreal, int Creal, int CIN, int N, int flip,
                                    bf16 *__restrict__ out) {
  const int K = 27 * CIN;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K * N) return;
  const int n = e / K, k = e % K;
  const int tap = k / CIN, c = k % CIN;
  float v = 0.f;
  if (!flip) {
    if (n < Nreal && c < Creal) v = w[(n * 27 + tap) * Creal + c];
  } else {
    // output channel n of the transposed conv is input channel n of the forward conv;
    // reduction channel c is forward output channel c
    if (c < Nreal && n < Creal) v = w[(c * 27 + (26 - tap)) * Creal + n];
  }
  out[((size_t)(k / 8) * N + n) * 8 + (k % 8)] = __float2bfloat16_rn(v);
}

// x (B, G^3, 2) bf16 from the density and potential grids: x0 = log(1 + rho_scale * rho)
// (the density spans four decades in a Plummer core), x1 = phi_scale * phi (phi read from
// lane 3 of the PM force grid).
__global__ void cnn_input_kernel(const float *__restrict__ rho, const float4 *__restrict__ F, int64_t nv,
                                 float rho_scale, float phi_scale, bf16 *__restrict__ x) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  *reinterpret_cast<__nv_bfloat162 *>(x + v * 2) =
      __floats2bfloat162_rn(log1pf(fmaxf(rho_scale * rho[v], 0.f)), phi_scale * F[v].w);
}

// AdamW (decoupled weight decay), fp32 master weights.
__global__ void adamw_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                             float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float wd,
                             float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float mh = mi / bc1, vh = vi / bc2;
  p[i] = p[i] * (1.f - lr * wd) - lr * mh / (sqrtf(vh) + eps);
}

// dL/dfield = CIC scatter of the per-body gradient (transpose of the gather), fp32 atomics.
// field layout float4 [G^3] (lanes 0..2), bodies pos (n, 3), grad (n, 3).
__global__ void gather_transpose_kernel(const float *__restrict__ pos, const float *__restrict__ grad, int64_t n,
                                        int G, float half_ext, float h, float inv_h, float4 *__restrict__ field) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ix, iy, iz;
  float wx, wy, wz;
  cic_axis(pos[i * 3], half_ext, h, ix, wx, inv_h);
  cic_axis(pos[i * 3 + 1], half_ext, h, iy, wy, inv_h);
  cic_axis(pos[i * 3 + 2], half_ext, h, iz, wz, inv_h);
  const float g0 = grad[i * 3], g1 = grad[i * 3 + 1], g2 = grad[i * 3 + 2];
  for (int ox = 0; ox < 2; ++ox)
    for (int oy = 0; oy < 2; ++oy)
      for (int oz = 0; oz < 2; ++oz) {
        const float wt = axis_w(wx, ox) * axis_w(wy, oy) * axis_w(wz, oz);
        const size_t cell = ((size_t)fwrap(iz + oz, G) * G + fwrap(iy + oy, G)) * G + fwrap(ix + ox, G);
        float *f = reinterpret_cast<float *>(field + cell);
        atomicAdd(f, wt * g0);
        atomicAdd(f + 1, wt * g1);
        atomicAdd(f + 2, wt * g2);
      }
}

// (B, G^3) float4 lanes 0..2 -> (B, G^3, 16) bf16 with channels 3..15 zero (input of the
// output layer's data gradient).
__global__ void pack_dout_kernel(const float4 *__restrict__ f, int64_t nv, float scale, bf16 *__restrict__ out) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  float4 a = f[v];
  __align__(16) bf16 o[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) o[c] = __float2bfloat16_rn(0.f);
  o[0] = __float2bfloat16_rn(scale * a.x);
  o[1] = __float2bfloat16_rn(scale * a.y);
  o[2] = __float2bfloat16_rn(scale * a.z);
  uint4 *dst = reinterpret_cast<uint4 *>(out + v * 16);
  dst[0] = reinterpret_cast<uint4 *>(o)[0];
  dst[1] = reinterpret_cast<uint4 *>(o)[1];
}

// dz0 = dh0 * gelu'(z0) for the input layer (no residual): (nv * 32) elements.
__global__ void gelu_bwd_kernel(const float *__restrict__ dh, const bf16 *__restrict__ z, int64_t n,
                                bf16 *__restrict__ dz) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dz[i] = __float2bfloat16_rn(dh[i] * gelu_grad(__bfloat162float(z[i])));
}

}  // namespace augur

using namespace augur;

namespace {

template <int CIN, int N, int EPI>
int launch_conv_tc(const void *in, const void *wB, const float *bias, const void *resid, const void *zprev,
                   void *out0, void *out1, int B, int G, float out_scale, unsigned *err, cudaStream_t st) {
  ConvArgs a;
  a.B = B;
  a.G = G;
  a.xseg = (G + CONV_M - 1) / CONV_M;
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // y chunk: long enough to amortise the 3-row warm-up, short enough to fill every SM
  const int columns = B * G * a.xseg;
  int yc = G;
  while (yc > 8 && (long long)columns * ((G + yc - 1) / yc) < 3LL * nsm) yc = (yc + 1) / 2;
  a.yc = yc;
  a.nyc = (G + yc - 1) / yc;
  a.nunits = columns * a.nyc;
  a.out_scale = out_scale;
  constexpr int WBYTES = 27 * CIN * N * 2;
  constexpr int SLAB_STRIDE = ((((CIN / 8) * SLAB * 16) + 127) / 128) * 128;
  const size_t smem = ((WBYTES + 127) / 128) * 128 + (size_t)3 * RING * SLAB_STRIDE;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(conv_tc_kernel<CIN, N, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  const int grid = std::min(a.nunits, nsm);
  conv_tc_kernel<CIN, N, EPI><<<grid, CONV_THREADS, smem, st>>>(
      (const bf16 *)in, (const bf16 *)wB, bias, resid, (const bf16 *)zprev, out0, (bf16 *)out1, a, err);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

template <int CIN, int N, int DZF>
int launch_wgrad(const void *h, const void *dz, int B, int G, float *partial, int max_parts, float *out,
                 cudaStream_t st) {
  const int nrows = B * G * G;
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int nparts = std::min(max_parts, std::min(nrows, nsm * 4));
  const int rows_per = (nrows + nparts - 1) / nparts;
  nparts = (nrows + rows_per - 1) / rows_per;
  const size_t smem = ((size_t)9 * (G + 2) * CIN + (size_t)G * N) * 4;
  if (smem > 227 * 1024) return AUGUR_EINVAL;
  cudaFuncSetAttribute(wgrad_kernel<CIN, N, DZF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  wgrad_kernel<CIN, N, DZF><<<nparts, CIN * N, smem, st>>>((const bf16 *)h, dz, B, G, rows_per, partial);
  const int len = N * 27 * CIN + N;
  reduce_partials_kernel<<<(len + 255) / 256, 256, 0, st>>>(partial, nparts, len, out);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

}  // namespace

extern "C" {

// layer: 0 = 32 -> 32 residual GELU layer (forward), 1 = output layer 32 -> 3 (added to a
// float4 grid), 2 = data gradient through a 32 -> 32 layer, 3 = data gradient through the
// output layer (input: 16-channel padded output gradient).
int augur_cnn_conv_tc(int layer, const void *in, const void *w_umma, const float *bias, const void *resid,
                      const void *zprev, void *out0, void *out1, int batch, int grid, float out_scale,
                      unsigned *err, void *stream) {
  if (!in || !w_umma || !out0 || batch < 1 || grid < 3 || !err) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  switch (layer) {
    case 0: return launch_conv_tc<32, 32, EPI_FWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, st);
    case 1: return launch_conv_tc<32, 16, EPI_OUT>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, out_scale, err, st);
    case 2: return launch_conv_tc<32, 32, EPI_BWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, st);
    case 3: return launch_conv_tc<16, 32, EPI_BWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, st);
    default: return AUGUR_EINVAL;
  }
}

int augur_cnn_conv_in(const void *x, const float *w, const float *bias, int batch, int grid, void *z0, void *h0,
                      void *stream) {
  if (!x || !w || !bias || !z0 || !h0 || batch < 1 || grid < 3) return AUGUR_EINVAL;
  const int64_t nv = (int64_t)batch * grid * grid * grid;
  const int blocks = (int)std::min<int64_t>((nv + 255) / 256, 152 * 16);
  conv_in_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>((const bf16 *)x, w, bias, batch, grid, (bf16 *)z0,
                                                          (bf16 *)h0);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

// kind: 0 = 32 -> 32 (dz bf16), 1 = output layer 32 -> 3 (dz = output gradient, fp32 float4
// grid), 2 = input layer 2 -> 32 (dz bf16). out: N*27*CIN weight gradients then N bias
// gradients; partial: scratch of max_parts * (N*27*CIN + N) floats.
int augur_cnn_wgrad(int kind, const void *h, const void *dz, int batch, int grid, float *partial, int max_parts,
                    float *out, void *stream) {
  if (!h || !dz || !partial || !out || max_parts < 1) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  switch (kind) {
    case 0: return launch_wgrad<32, 32, 0>(h, dz, batch, grid, partial, max_parts, out, st);
    case 1: return launch_wgrad<32, 4, 1>(h, dz, batch, grid, partial, max_parts, out, st);
    case 2: return launch_wgrad<2, 32, 0>(h, dz, batch, grid, partial, max_parts, out, st);
    default: return AUGUR_EINVAL;
  }
}

int augur_cnn_prep_weights(const float *w, int n_out, int c_in, int cin_pad, int n_pad, int flip, void *out,
                           void *stream) {
  if (!w || !out) return AUGUR_EINVAL;
  const int total = 27 * cin_pad * n_pad;
  prep_weights_kernel<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(w, n_out, c_in, cin_pad, n_pad, flip,
                                                                            (bf16 *)out);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_cnn_input(const float *rho, const float *force4, int64_t nvox, float rho_scale, float phi_scale, void *x,
                    void *stream) {
  if (!rho || !force4 || !x) return AUGUR_EINVAL;
  cnn_input_kernel<<<(unsigned)((nvox + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      rho, (const float4 *)force4, nvox, rho_scale, phi_scale, (bf16 *)x);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_cnn_adamw(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                    float wd, int step, void *stream) {
  if (!p || !g || !m || !v || n < 0 || step < 1) return AUGUR_EINVAL;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  adamw_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, wd, bc1, bc2);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_cnn_gather_transpose(const float *pos, const float *grad, int64_t n, int grid, double extent,
                               float *field4, void *stream) {
  if (!pos || !grad || !field4 || grid < 1) return AUGUR_EINVAL;
  const double h = extent / grid;
  const float h32 = (float)h;
  int ex = 0;
  const float mant = std::frexp(h32, &ex);
  const float inv_h = (mant == 0.5f) ? 1.0f / h32 : 0.0f;
  gather_transpose_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      pos, grad, n, grid, (float)(extent / 2.0), h32, inv_h, (float4 *)field4);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_cnn_pack_dout(const float *field4, int64_t nvox, float scale, void *out16, void *stream) {
  if (!field4 || !out16) return AUGUR_EINVAL;
  pack_dout_kernel<<<(unsigned)((nvox + 255) / 256), 256, 0, (cudaStream_t)stream>>>((const float4 *)field4, nvox,
                                                                                    scale, (bf16 *)out16);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int augur_cnn_gelu_bwd(const float *dh, const void *z, int64_t n, void *dz, void *stream) {
  if (!dh || !z || !dz) return AUGUR_EINVAL;
  gelu_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(dh, (const bf16 *)z, n,
                                                                                (bf16 *)dz);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

}  // extern "C"
