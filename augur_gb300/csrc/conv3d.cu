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

#include <cuda.h>  // CUtensorMap (the encode entry point is resolved through the runtime)
#include <cudaTypedefs.h>

#include <mutex>

#include <atomic>

#include "augur_common.cuh"
#include "tcgen05.cuh"

using bf16 = __nv_bfloat16;

namespace augur {

constexpr int CONV_M = 128;     // voxels per tile (one x segment)
constexpr int SLAB = CONV_M + 2;  // voxel rows of an input slab: x0-1 .. x0+128
constexpr int SLAB_ROWS = 136;    // shared-memory rows per channel block (128-byte aligned TMA boxes)
constexpr int RING = 6;           // input rows (all three z planes) in flight
constexpr int NACC = 4;           // TMEM accumulators: tiles between the MMA warp and the epilogue
// warps 0-7: epilogue (two per TMEM lane quarter, each taking half of the output channels);
// warp 8: MMA issue; warp 9: TMA loads
constexpr int EPI_WARPS = 8;
constexpr int MMA_WARP = EPI_WARPS;
constexpr int TMA_WARP = EPI_WARPS + 1;
constexpr int CONV_THREADS = 32 * (EPI_WARPS + 2);
constexpr uint32_t WAIT_BUDGET = 1u << 20;  // default tries of a pipeline wait (augur_cnn_set_wait_budget)
// Tries of a drain wait: before a CTA exits it waits, with this fixed bound and regardless of the
// pipeline budget, for its own TMA copies and MMAs still in flight, so that nothing writes its
// shared memory or TMEM after it has gone.
constexpr uint32_t DRAIN_BUDGET = 1u << 22;

enum { EPI_FWD = 0, EPI_OUT = 1, EPI_BWD = 2 };

// GELU and its derivative with the erfc of Abramowitz & Stegun 7.1.26 (|erf error| <= 1.5e-7, far
// below the BF16 rounding of the activations; about half the instructions of erff, which matters in
// the epilogues: 32 GELUs per voxel and layer)
__device__ __forceinline__ float gelu_f(float x) { return gelu_as(x); }
__device__ __forceinline__ float gelu_grad(float x) { return gelu_grad_as(x); }

// 5D tiled TMA load (c, x, y, z, b) into shared memory, completing bytes on mbar.
__device__ __forceinline__ void tma_load5(uint32_t dst, const CUtensorMap *map, int c, int x, int y, int z, int b,
                                          uint64_t *mbar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(z), "r"(b), "r"(smem_u32(mbar))
      : "memory");
}

struct ConvArgs {
  int B, G;
  int xseg;          // ceil(G / 128)
  long long rows;    // B * G * xseg * G output rows (b, z, x segment, y), split evenly over the CTAs
  float out_scale;   // EPI_OUT: added field = out_scale * (acc + bias)
  uint32_t budget;   // tries of a pipeline wait before the CTA gives up (AUGUR_ERRBIT_TIMEOUT)
};

struct ConvUnit {
  int b, z, x0, ya, ny;
};
// Work of a CTA: one contiguous range of the flattened output rows (b, z, x segment, y), cut into
// pieces at column ends (a piece is a ConvUnit: consecutive y rows of one (b, z, x segment)).
// Equal ranges keep every SM busy to the end: dealing fixed 32-row units to 152 CTAs gave the
// slowest ones 4 units (136 input rows with halos) against 115 on average at 128^3.
__device__ __forceinline__ long long cta_rows_begin(const ConvArgs &a) {
  return a.rows * (long long)blockIdx.x / gridDim.x;
}
__device__ __forceinline__ long long cta_rows_end(const ConvArgs &a) {
  return a.rows * (long long)(blockIdx.x + 1) / gridDim.x;
}
__device__ __forceinline__ bool next_piece(const ConvArgs &a, long long &f, long long end, ConvUnit &u) {
  if (f >= end) return false;
  const long long col = f / a.G;
  const int y = (int)(f - col * a.G);
  const int ny = (int)min((long long)(a.G - y), end - f);
  int t = (int)col;
  const int xs = t % a.xseg;
  t /= a.xseg;
  u.z = t % a.G;
  u.b = t / a.G;
  u.x0 = xs * CONV_M;
  u.ya = y;
  u.ny = ny;
  f += ny;
  return true;
}


// ---------------------------------------------------------------------------------------
// tcgen05 implicit-GEMM 3x3x3 conv. CIN in {16, 32}, N (output channels) in {16, 32}.
//   EPI_FWD: z = acc + b ; h = h_in + gelu(z)         out0 = h (bf16), out1 = z (bf16, optional)
//   EPI_OUT: y = out_scale * (acc + b)[0..2]          out0 = F (float4 grid, y added to lanes 0..2)
//   EPI_BWD: g = acc + resid (fp32, optional)         out0 = g (fp32), out1 = g * gelu'(zprev) (bf16)
//
// GEMM shape. A 128-voxel input row (x0-1 .. x0+128) of the three planes z-1, z, z+1 is one
// K = 3 * CIN operand; for each dx it multiplies a [3 CIN] x [3 N] weight block whose N axis
// is (dy, output channel). So one input row y' feeds output rows y'+1, y', y'-1 (dy = 0, 1, 2)
// at once, with MMAs of N up to 96 instead of 27 narrow N = 32 ones per output row (a
// 128 x N x 16 MMA costs ~46 cycles for any N <= 64 on this part, 64 at N = 128).
// Output rows accumulate in a ring of RACC TMEM slots ordered so that the three targets of an
// input row are adjacent columns (slot(T) = RACC-1 - T mod RACC for output row T); at the ring's
// wrap, or at a unit's first and last rows, the MMA is split or narrowed to the rows that exist.
// Accumulators start from zero and every MMA accumulates: the epilogue zeroes a slot after
// reading it.
//
// Work: each CTA takes one contiguous range of the output rows (batch, z, x segment, y), in pieces
// of consecutive y rows of one (batch, z, x segment). Warp-specialised pipeline, no block barrier
// per row:
//   TMA warp   loads input row y' of planes z-1, z, z+1 (one 8-channel x 130-voxel box per
//              channel block; the tensor map zero-fills outside the grid) into a ring of RING
//              slots, arming full[slot] with the byte count;
//   MMA warp   per input row: 3 dx x 3 CIN/16 MMAs (or two narrower ones at the wrap), then
//              commits empty[slot] (the row is used once) and slot_full of the output row the
//              row completed;
//   epilogue   per output row: waits for slot_full, reads (tcgen05.ld), zeroes (tcgen05.st) the
//              slot, applies the layer's epilogue, and arrives on slot_empty.
// Every wait is bounded: a stall sets the CTA's abort flag, the roles leave their loops,
// and bit AUGUR_ERRBIT_TIMEOUT is raised in *err.
// ---------------------------------------------------------------------------------------
// output-row accumulator slots in TMEM: 512 / N, which fills the SM's 512 columns (the kernel runs
// one CTA per SM). The deeper ring lets the MMAs run further ahead of the epilogue and halves the
// ring wraps that split an input row's MMAs (32 -> 32 at 128^3: 193 us with 8 slots, 184.5 with
// 16; a probe without the MMA warp's waits ran 169).
template <int N>
constexpr int racc_slots() { return 512 / N; }

template <int CIN, int N, int EPI>
__global__ void __launch_bounds__(CONV_THREADS, 1) conv_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                  const bf16 *__restrict__ wB,
                                                                  const float *__restrict__ bias,
                                                                  const void *__restrict__ resid,
                                                                  const bf16 *__restrict__ zprev,
                                                                  void *__restrict__ out0, bf16 *__restrict__ out1,
                                                                  ConvArgs a, unsigned *__restrict__ err,
                                                                  double *__restrict__ stats) {
  constexpr int CB = CIN / 8;              // 16-byte channel blocks per voxel
  constexpr int KB = 3 * CB;               // K blocks of an input row (three planes)
  constexpr int KSTEPS = KB / 2;           // K = 16 per MMA
  constexpr int NR = 3 * N;                // (dy, output channel)
  constexpr int WBYTES = 27 * CIN * N * 2; // weights [dx][KB][NR][16 B]
  constexpr int WREGION = ((WBYTES + 127) / 128) * 128;
  constexpr int CBLK = SLAB_ROWS * 16;     // one channel block of a slab
  constexpr int SLOT_BYTES = 3 * CB * CBLK;
  constexpr uint32_t ROW_TX = 3u * CB * SLAB * 16;  // bytes the boxes of one ring slot bring
  constexpr int NC = N / 2;
  constexpr int RACC = racc_slots<N>();
  constexpr int TMEM_COLS = RACC * N;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sW = smem;
  unsigned char *sSlab = smem + WREGION;  // [RING][3 planes][CB][SLAB_ROWS][16 B]
  __shared__ __align__(8) uint64_t full[RING], empty[RING], slot_full[RACC], slot_empty[RACC], drained;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = a.G;
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(wB);
    uint4 *dst = reinterpret_cast<uint4 *>(sW);
    for (int e = tid; e < WBYTES / 16; e += CONV_THREADS) dst[e] = src[e];
  }
  if (tid == 0) {
    for (int i = 0; i < RING; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < RACC; ++i) {
      mbar_init(&slot_full[i], 1);
      mbar_init(&slot_empty[i], EPI_WARPS);
    }
    mbar_init(&drained, 1);
    s_abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, TMEM_COLS);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const int q = warp & 3, half = warp >> 2;  // epilogue warps: lane quarter, column half
  if (warp < EPI_WARPS) {  // every accumulator slot starts at zero
    for (int sl = 0; sl < RACC; ++sl) {
      const uint32_t ta = tmem + (uint32_t)(sl * N + half * NC) + ((uint32_t)(q * 32) << 16);
      if constexpr (NC == 16) tmem_zero16(ta);
      else tmem_zero8(ta);
    }
    tmem_wait_st();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t slab0 = smem_u32(sSlab);
  volatile int *abort_flag = &s_abort;
  auto slot_of = [](uint32_t T) -> uint32_t { return RACC - 1 - (T % RACC); };

  // bounded wait; gives up early once another role has given up
  auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
    for (uint32_t i = 0; i < a.budget; ++i) {
      if (mbar_try_wait(bar, parity)) return true;
      if ((i & 255u) == 255u && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
  };

  double s_corr_out = 0.0, s_pm_out = 0.0;  // EPI_OUT with stats: sums over this thread's voxels
  if (warp == TMA_WARP) {
    // ---- producer: rows ya-1 .. ya+ny of every unit, all three planes ----------------------
    uint32_t k = 0;
    if (lane == 0) {
      bool go = true;
      long long fpos = cta_rows_begin(a);
      const long long fend = cta_rows_end(a);
      ConvUnit u;
      while (go && next_piece(a, fpos, fend, u)) {
        for (int j = 0; j < u.ny + 2; ++j, ++k) {
          const uint32_t slot = k % RING, n = k / RING;
          if (n > 0 && !wait(&empty[slot], (n - 1) & 1u)) {
            go = false;
            break;
          }
          mbar_expect_tx(&full[slot], ROW_TX);
          const uint32_t dst0 = slab0 + slot * SLOT_BYTES;
#pragma unroll
          for (int pz = 0; pz < 3; ++pz)
#pragma unroll
            for (int cb = 0; cb < CB; ++cb)
              tma_load5(dst0 + (uint32_t)((pz * CB + cb) * CBLK), &tmap, cb * 8, u.x0 - 1, u.ya - 1 + j, u.z + pz - 1,
                        u.b, &full[slot]);
        }
      }
      // tail: the copies of the last RING fills have landed (no transfer still writes this
      // CTA's shared memory when it exits), waited for even after an abort
      const uint32_t last = k;
      for (uint32_t r = (last > RING ? last - RING : 0); r < last; ++r)
        if (!mbar_wait_bounded(&full[r % RING], (r / RING) & 1u, DRAIN_BUDGET)) *abort_flag = 1;
    }
  } else if (warp == MMA_WARP) {
    // ---- MMA issue, one input row at a time ---------------------------------------------------
    if (lane == 0) {
      const uint32_t w0 = smem_u32(sW);
      uint32_t k0 = 0, T0 = 0;
      bool go = true;
      long long fpos = cta_rows_begin(a);
      const long long fend = cta_rows_end(a);
      ConvUnit u;
      while (go && next_piece(a, fpos, fend, u)) {
        for (int j = 0; j < u.ny + 2 && go; ++j) {
          const uint32_t kr = k0 + j;
          if (!wait(&full[kr % RING], (kr / RING) & 1u)) {
            go = false;
            break;
          }
          if (j <= u.ny - 1) {  // first contribution to output row T0 + j: its slot must be free
            const uint32_t Tn = T0 + j;
            if (Tn >= RACC && !wait(&slot_empty[slot_of(Tn)], ((Tn / RACC) - 1) & 1u)) {
              go = false;
              break;
            }
          }
          tc_fence_after();
          const uint64_t arow = smem_desc(slab0 + (kr % RING) * SLOT_BYTES, CBLK, 128);
          const int dlo = max(0, j - u.ny + 1), dhi = min(2, j);
          // runs of adjacent accumulator slots: split where the ring wraps
          int s0 = dlo;
          for (int dy = dlo; dy <= dhi; ++dy) {
            const uint32_t sl = slot_of(T0 + j - dy);
            if (dy < dhi && sl != RACC - 1) continue;
            const int nrun = dy - s0 + 1;
            const uint32_t d = tmem + slot_of(T0 + j - s0) * N;
            const uint32_t idesc = idesc_bf16_f32(CONV_M, nrun * N);
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) {
#pragma unroll
              for (int kc = 0; kc < KSTEPS; ++kc) {
                const uint64_t ad = arow + (uint64_t)(((2 * kc) * CBLK + dx * 16) >> 4);
                const uint64_t bd = smem_desc(w0 + (uint32_t)(((dx * KB + 2 * kc) * NR + s0 * N) * 16), NR * 16, 128);
                umma_bf16(d, ad, bd, idesc, 1u);
              }
            }
            s0 = dy + 1;
          }
          umma_commit(&empty[kr % RING]);                                     // the input row is used once
          if (j >= 2) umma_commit(&slot_full[slot_of(T0 + j - 2)]);            // output row j - 2 is complete
        }
        k0 += u.ny + 2;
        T0 += u.ny;
      }
      // drain: every MMA this thread issued (and the arrivals its commits make) has completed
      // before the CTA frees TMEM and exits, on the normal path and after an abort alike
      umma_commit(&drained);
      if (!mbar_wait_bounded(&drained, 0u, DRAIN_BUDGET)) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp w reads TMEM lane quarter w % 4 (voxels x0 + 32 (w % 4) + lane) and
    // output channels [NC (w / 4), + NC) of the output row's slot ---------------------------------
    const int c0 = half * NC;
    const bool active = !(EPI == EPI_OUT && half == 1);  // three output channels: first half only
    uint32_t T = 0;
    bool go = true;
    long long fpos = cta_rows_begin(a);
    const long long fend = cta_rows_end(a);
    ConvUnit u;
    while (go && next_piece(a, fpos, fend, u)) {
      const size_t bbase = (size_t)u.b * G * G * G;
      for (int i = 0; i < u.ny; ++i, ++T) {
        const uint32_t sl = slot_of(T);
        const int y = u.ya + i;
        const int x = u.x0 + q * 32 + lane;
        const bool mine = active && x < G;
        const size_t vox = bbase + ((size_t)u.z * G + y) * G + x;
        // the residual / force-grid values this thread adds to are loaded before the wait, so
        // their latency overlaps the row's MMAs
        uint4 hpre[EPI == EPI_FWD ? NC / 8 : 1];
        float4 fpre = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (EPI == EPI_FWD) {
          if (mine) {
#pragma unroll
            for (int n = 0; n < NC; n += 8)
              hpre[n / 8] = *reinterpret_cast<const uint4 *>(reinterpret_cast<const bf16 *>(resid) + vox * N + c0 + n);
          }
        } else if constexpr (EPI == EPI_OUT) {
          if (mine) fpre = reinterpret_cast<const float4 *>(out0)[vox];
        }
        if (!wait(&slot_full[sl], (T / RACC) & 1u)) {
          go = false;
          break;
        }
        tc_fence_after();
        float v[NC];
        const uint32_t taddr = tmem + sl * N + (uint32_t)c0 + ((uint32_t)(q * 32) << 16);
        if constexpr (NC == 16) {
          tmem_ld16(taddr, v);
          tmem_zero16(taddr);
        } else {
          tmem_ld8(taddr, v);
          tmem_zero8(taddr);
        }
        tmem_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&slot_empty[sl]);
        if (mine) {
          if constexpr (EPI == EPI_FWD) {
            bf16 *hout = reinterpret_cast<bf16 *>(out0) + vox * N + c0;
#pragma unroll
            for (int n = 0; n < NC; n += 8) {
              uint4 hv = hpre[n / 8];
              const __nv_bfloat162 *hp = reinterpret_cast<const __nv_bfloat162 *>(&hv);
              __align__(16) __nv_bfloat162 ho[4], zo[4];
#pragma unroll
              for (int q2 = 0; q2 < 4; ++q2) {
                const float z0 = v[n + 2 * q2] + bias[c0 + n + 2 * q2];
                const float z1 = v[n + 2 * q2 + 1] + bias[c0 + n + 2 * q2 + 1];
                ho[q2] = __floats2bfloat162_rn(__bfloat162float(hp[q2].x) + gelu_f(z0),
                                               __bfloat162float(hp[q2].y) + gelu_f(z1));
                zo[q2] = __floats2bfloat162_rn(z0, z1);
              }
              *reinterpret_cast<uint4 *>(hout + n) = *reinterpret_cast<uint4 *>(ho);
              if (out1) *reinterpret_cast<uint4 *>(out1 + vox * N + c0 + n) = *reinterpret_cast<uint4 *>(zo);
            }
          } else if constexpr (EPI == EPI_OUT) {
            float4 f = fpre;
            const float cx = a.out_scale * (v[0] + bias[0]), cy = a.out_scale * (v[1] + bias[1]),
                        cz = a.out_scale * (v[2] + bias[2]);
            if (stats) {  // |correction|^2 and |PM force|^2 of this voxel, summed below
              s_corr_out += (double)(cx * cx + cy * cy + cz * cz);
              s_pm_out += (double)(f.x * f.x + f.y * f.y + f.z * f.z);
            }
            f.x += cx;
            f.y += cy;
            f.z += cz;
            reinterpret_cast<float4 *>(out0)[vox] = f;
          } else {
            const float *rin = reinterpret_cast<const float *>(resid);
            float *gout = reinterpret_cast<float *>(out0) + vox * N + c0;
#pragma unroll
            for (int n = 0; n < NC; n += 4) {
              float4 g = make_float4(v[n], v[n + 1], v[n + 2], v[n + 3]);
              if (rin) {
                const float4 r = *reinterpret_cast<const float4 *>(rin + vox * N + c0 + n);
                g.x += r.x;
                g.y += r.y;
                g.z += r.z;
                g.w += r.w;
              }
              *reinterpret_cast<float4 *>(gout + n) = g;
              if (out1) {
                const bf16 *zp = zprev + vox * N + c0 + n;
                const __nv_bfloat162 z01 = *reinterpret_cast<const __nv_bfloat162 *>(zp);
                const __nv_bfloat162 z23 = *reinterpret_cast<const __nv_bfloat162 *>(zp + 2);
                __align__(8) __nv_bfloat162 o[2];
                o[0] = __floats2bfloat162_rn(g.x * gelu_grad(__bfloat162float(z01.x)),
                                             g.y * gelu_grad(__bfloat162float(z01.y)));
                o[1] = __floats2bfloat162_rn(g.z * gelu_grad(__bfloat162float(z23.x)),
                                             g.w * gelu_grad(__bfloat162float(z23.y)));
                *reinterpret_cast<uint2 *>(out1 + vox * N + c0 + n) = *reinterpret_cast<uint2 *>(o);
              }
            }
          }
        }
      }
    }
  }
  if constexpr (EPI == EPI_OUT) {
    if (stats && warp < EPI_WARPS) {
      double c = s_corr_out, m = s_pm_out;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        m += __shfl_xor_sync(0xffffffffu, m, o);
      }
      if (lane == 0) {
        atomicAdd(&stats[0], c);
        atomicAdd(&stats[1], m);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && *abort_flag) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------------------
// Input layer on tcgen05: x (B, G^3, 2) bf16 -> z0 (optional), h0 = gelu(z0), 32 channels.
// K = 27 taps x 2 channels = 54, padded to 64 (four K = 16 MMAs per tile); the A operand is
// built in shared memory by producer warps (im2col: thread r gathers the 27 neighbours of voxel
// x0 + r, two channels each, into 16-byte K blocks), published to the MMA warp through
// full/empty mbarriers; the epilogue is the forward layers' (eight warps, two per TMEM lane
// quarter). The producers form IN_GROUPS groups of 128 threads that take the tile rows in turn,
// so that as many rows' gathers are in flight at once (one group's loads are a few L2 round trips
// per row, which alone would bound the layer). Weights: augur_cnn_prep_weights(w_in, 32, 2, 2, 32,
// 0) into a zeroed 64 x 32 buffer.
// ---------------------------------------------------------------------------------------
constexpr int IN_PROD_WARPS = 16;                       // producer warps: IN_GROUPS x 128 threads
constexpr int IN_GROUPS = IN_PROD_WARPS / 4;            // rows gathered at once
constexpr int IN_STAGES = 8;                            // A buffers in flight
constexpr int IN_KB = 8;                                // 16-byte K blocks (64 K values)
constexpr int IN_ABYTES = IN_KB * CONV_M * 16;          // 16 KB per A buffer
constexpr int IN_THREADS = 32 * (EPI_WARPS + 1 + IN_PROD_WARPS);

__global__ void __launch_bounds__(IN_THREADS, 1) conv_in_tc_kernel(const bf16 *__restrict__ x,
                                                                   const bf16 *__restrict__ wB,
                                                                   const float *__restrict__ bias,
                                                                   bf16 *__restrict__ z0, bf16 *__restrict__ h0,
                                                                   ConvArgs a, unsigned *__restrict__ err) {
  constexpr int N = 32, NC = 16;
  constexpr uint32_t IDESC = idesc_bf16_f32(CONV_M, N);
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sW = smem;                   // [8 kb][32 n][16 B]
  unsigned char *sA = smem + IN_KB * N * 16;  // [IN_STAGES][8 kb][128 r][16 B]
  __shared__ __align__(8) uint64_t full[IN_STAGES], empty[IN_STAGES], acc_full[NACC], acc_empty[NACC], drained;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = a.G;
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(wB);
    uint4 *dst = reinterpret_cast<uint4 *>(sW);
    for (int e = tid; e < IN_KB * N; e += IN_THREADS) dst[e] = src[e];
    // K block 7 of every A buffer is padding: zero once
    uint4 *A = reinterpret_cast<uint4 *>(sA);
    for (int e = tid; e < IN_STAGES * IN_KB * CONV_M; e += IN_THREADS) A[e] = make_uint4(0u, 0u, 0u, 0u);
  }
  if (tid == 0) {
    for (int i = 0; i < IN_STAGES; ++i) {
      mbar_init(&full[i], CONV_M);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < NACC; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], EPI_WARPS);
    }
    mbar_init(&drained, 1);
    s_abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, NACC * 32);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t a0 = smem_u32(sA);
  volatile int *abort_flag = &s_abort;
  auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
    for (uint32_t i = 0; i < a.budget; ++i) {
      if (mbar_try_wait(bar, parity)) return true;
      if ((i & 255u) == 255u && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
  };

  if (warp > MMA_WARP) {
    // ---- producers: thread r of group grp builds row r of the A operand of tiles t with
    // t % IN_GROUPS == grp (K blocks 0-6; block 7 and tap 27 are padding) ---------------------
    const int pr = tid - 32 * (MMA_WARP + 1);
    const int r = pr & (CONV_M - 1), grp = pr >> 7;
    const uint32_t *x32 = reinterpret_cast<const uint32_t *>(x);  // two bf16 channels per voxel
    uint32_t t = 0;
    bool go = true;
    long long fpos = cta_rows_begin(a);
    const long long fend = cta_rows_end(a);
    ConvUnit u;
    while (go && next_piece(a, fpos, fend, u)) {
      const size_t bbase = (size_t)u.b * G * G * G;
      const int xx = u.x0 + r;
      // the three x neighbours' validity is fixed for the piece; the nine (dz, dy) rows' per row
      bool xin[3];
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) xin[dx] = xx + dx - 1 >= 0 && xx + dx - 1 < G;
      for (int i = 0; i < u.ny; ++i, ++t) {
        if ((int)(t % IN_GROUPS) != grp) continue;
        const uint32_t st = t % IN_STAGES, n = t / IN_STAGES;
        if (n > 0 && !wait(&empty[st], (n - 1) & 1u)) {
          go = false;
          break;
        }
        const int y = u.ya + i;
        uint32_t v[28];
#pragma unroll
        for (int r9 = 0; r9 < 9; ++r9) {
          const int zz = u.z + r9 / 3 - 1, yy = y + r9 % 3 - 1;
          const bool rin = zz >= 0 && zz < G && yy >= 0 && yy < G;
          const uint32_t *row = x32 + bbase + ((size_t)(rin ? zz : 0) * G + (rin ? yy : 0)) * G + xx - 1;
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) v[r9 * 3 + dx] = (rin && xin[dx]) ? __ldg(row + dx) : 0u;
        }
        v[27] = 0u;
        unsigned char *A = sA + (size_t)st * IN_ABYTES;
#pragma unroll
        for (int kb = 0; kb < 7; ++kb)
          *reinterpret_cast<uint4 *>(A + ((size_t)kb * CONV_M + r) * 16) =
              make_uint4(v[4 * kb], v[4 * kb + 1], v[4 * kb + 2], v[4 * kb + 3]);
        fence_async_smem();  // generic-proxy stores -> visible to the tensor core
        mbar_arrive(&full[st]);
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint64_t b_desc0 = smem_desc(smem_u32(sW), N * 16, 128);
      uint32_t t = 0;
      bool go = true;
      long long fpos = cta_rows_begin(a);
      const long long fend = cta_rows_end(a);
      ConvUnit u;
      while (go && next_piece(a, fpos, fend, u)) {
        for (int i = 0; i < u.ny; ++i, ++t) {
          const uint32_t st = t % IN_STAGES, acc = t % NACC;
          if (!wait(&full[st], (t / IN_STAGES) & 1u)) go = false;
          if (go && t >= NACC && !wait(&acc_empty[acc], ((t / NACC) - 1) & 1u)) go = false;
          if (!go) break;
          tc_fence_after();
          const uint64_t ad0 = smem_desc(a0 + st * IN_ABYTES, CONV_M * 16, 128);
#pragma unroll
          for (int kc = 0; kc < 4; ++kc)
            umma_bf16(tmem + acc * 32, ad0 + (uint64_t)((2 * kc * CONV_M * 16) >> 4),
                      b_desc0 + (uint64_t)((2 * kc * N * 16) >> 4), IDESC, kc ? 1u : 0u);
          umma_commit(&acc_full[acc]);
          umma_commit(&empty[st]);
        }
      }
      // drain: every MMA issued here (and its commits' arrivals) has completed before the CTA
      // frees TMEM and exits, also after an abort
      umma_commit(&drained);
      if (!mbar_wait_bounded(&drained, 0u, DRAIN_BUDGET)) *abort_flag = 1;
    }
  } else {
    // ---- epilogue ------------------------------------------------------------------------------
    const int q = warp & 3, half = warp >> 2;
    const int c0 = half * NC;
    uint32_t t = 0;
    bool go = true;
    long long fpos = cta_rows_begin(a);
    const long long fend = cta_rows_end(a);
    ConvUnit u;
    while (go && next_piece(a, fpos, fend, u)) {
      const size_t bbase = (size_t)u.b * G * G * G;
      for (int i = 0; i < u.ny; ++i, ++t) {
        const uint32_t acc = t % NACC;
        if (!wait(&acc_full[acc], (t / NACC) & 1u)) {
          go = false;
          break;
        }
        tc_fence_after();
        float v[NC];
        tmem_ld16(tmem + acc * 32 + (uint32_t)c0 + ((uint32_t)(q * 32) << 16), v);
        const int xq = u.x0 + q * 32 + lane;
        if (xq < G) {
          const size_t vox = bbase + ((size_t)u.z * G + u.ya + i) * G + xq;
#pragma unroll
          for (int nn = 0; nn < NC; nn += 8) {
            __align__(16) __nv_bfloat162 ho[4], zo[4];
#pragma unroll
            for (int q2 = 0; q2 < 4; ++q2) {
              const float za = v[nn + 2 * q2] + bias[c0 + nn + 2 * q2];
              const float zb = v[nn + 2 * q2 + 1] + bias[c0 + nn + 2 * q2 + 1];
              ho[q2] = __floats2bfloat162_rn(gelu_f(za), gelu_f(zb));
              zo[q2] = __floats2bfloat162_rn(za, zb);
            }
            *reinterpret_cast<uint4 *>(h0 + vox * N + c0 + nn) = *reinterpret_cast<uint4 *>(ho);
            if (z0) *reinterpret_cast<uint4 *>(z0 + vox * N + c0 + nn) = *reinterpret_cast<uint4 *>(zo);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[acc]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && *abort_flag) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, NACC * 32);
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
// One thread per (n, c, x range): XS threads share an (n, c) pair, each keeping 27 tap sums
// over a contiguous range of x in registers (a sliding window loads each input value once);
// the XS partial sums are added in a fixed order at the end. Also accumulates the bias
// gradient sum_v dz[v][n] (threads with c == 0).
// ---------------------------------------------------------------------------------------
template <int CIN, int N, int DZ_F32, int XS, int NB>
__global__ void __launch_bounds__(CIN * (N / NB) * XS) wgrad_kernel(const bf16 *__restrict__ h,
                                                                    const void *__restrict__ dz, int B, int G,
                                                                    int rows_per_cta, float *__restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem[];
  float *sh = reinterpret_cast<float *>(smem);            // [9][G + 2][CIN]
  float *sd = sh + (size_t)9 * (G + 2) * CIN;             // [G][N]
  constexpr int NP = CIN * (N / NB);                      // (output-channel group, c) pairs
  constexpr int NT = NP * XS;
  const int tid = threadIdx.x;
  const int pair = tid % NP, xs = tid / NP;
  const int n0 = (pair / CIN) * NB, c = pair % CIN;
  const int xa = (G * xs) / XS, xb = (G * (xs + 1)) / XS;
  float acc[NB][27];
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int t = 0; t < 27; ++t) acc[i][t] = 0.f;
  float bacc[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) bacc[i] = 0.f;
  const int nrows = B * G * G;
  const int r0 = blockIdx.x * rows_per_cta, r1 = min(nrows, r0 + rows_per_cta);
  for (int row = r0; row < r1; ++row) {
    const int y = row % G, z = (row / G) % G, b = row / (G * G);
    __syncthreads();
    for (int e = tid; e < 9 * (G + 2) * CIN; e += NT) {
      const int cc = e % CIN, xr = (e / CIN) % (G + 2), p = e / (CIN * (G + 2));
      const int zz = z + p / 3 - 1, yy = y + p % 3 - 1, xx = xr - 1;
      float v = 0.f;
      if (zz >= 0 && zz < G && yy >= 0 && yy < G && xx >= 0 && xx < G)
        v = __bfloat162float(h[((((size_t)b * G + zz) * G + yy) * G + xx) * CIN + cc]);
      sh[e] = v;
    }
    for (int e = tid; e < G * N; e += NT) {
      const size_t idx = (((size_t)b * G + z) * G + y) * G * N + e;
      sd[e] = DZ_F32 ? reinterpret_cast<const float *>(dz)[idx]
                     : __bfloat162float(reinterpret_cast<const bf16 *>(dz)[idx]);
    }
    __syncthreads();
    // sliding window: voxel x + dx of plane-row p is loaded once (at x' = x + 2) and reused for
    // the three dx taps and the NB output channels that read it
    float win[9][3];
#pragma unroll
    for (int p = 0; p < 9; ++p) {
      win[p][0] = sh[(p * (G + 2) + xa) * CIN + c];
      win[p][1] = sh[(p * (G + 2) + xa + 1) * CIN + c];
    }
    for (int x = xa; x < xb; ++x) {
      float g[NB];
#pragma unroll
      for (int i = 0; i < NB; ++i) g[i] = sd[x * N + n0 + i];
      if (c == 0)
#pragma unroll
        for (int i = 0; i < NB; ++i) bacc[i] += g[i];
#pragma unroll
      for (int p = 0; p < 9; ++p) {
        win[p][2] = sh[(p * (G + 2) + x + 2) * CIN + c];
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
          for (int i = 0; i < NB; ++i) acc[i][p * 3 + dx] += g[i] * win[p][dx];
        win[p][0] = win[p][1];
        win[p][1] = win[p][2];
      }
    }
  }
  float *out = partial + (size_t)blockIdx.x * (N * 27 * CIN + N);
  if constexpr (XS == 1) {
#pragma unroll
    for (int i = 0; i < NB; ++i) {
#pragma unroll
      for (int t = 0; t < 27; ++t) out[((n0 + i) * 27 + t) * CIN + c] = acc[i][t];
      if (c == 0) out[N * 27 * CIN + n0 + i] = bacc[i];
    }
  } else {
    static_assert(NB == 1, "x ranges are only used with one output channel per thread");
    // fixed-order sum of the XS ranges through shared memory (reusing the row buffers)
    __syncthreads();
    float *red = sh;  // [XS][CIN * N][28]
#pragma unroll
    for (int t = 0; t < 27; ++t) red[((size_t)xs * NP + pair) * 28 + t] = acc[0][t];
    red[((size_t)xs * NP + pair) * 28 + 27] = bacc[0];
    __syncthreads();
    for (int e = tid; e < NP * 28; e += NT) {
      const int pr = e / 28, t = e % 28;
      float v = 0.f;
      for (int k = 0; k < XS; ++k) v += red[((size_t)k * NP + pr) * 28 + t];
      const int nn = pr / CIN, cc = pr % CIN;
      if (t < 27) out[(nn * 27 + t) * CIN + cc] = v;
      else if (cc == 0) out[N * 27 * CIN + nn] = v;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Weight gradient on tcgen05: dW[n][tap][c] = sum_v dz[v][n] * h[v + tap][c] (zero padding) and
// the bias gradient sum_v dz[v][n], for 32 input channels and NP = 16 or 32 gradient channels.
//
// GEMM: D[(plane, c)][n] += A[(plane, c)][x] * B[x][n] over K = the 128 voxels x of one dz row
// (b, z, y, x0 .. x0+127), with A = the input rows of the nine (dz, dy) neighbour planes and B =
// the dz row. Both operands sit in shared memory exactly as the TMA boxes land, channels-last
// [8-channel block][voxel row][16 B], which for K = voxels is the MN-major no-swizzle layout: a
// core matrix is 8 voxel rows of 8 channels (128 contiguous bytes); in this mode the descriptor's
// leading byte offset is the distance between K-adjacent core matrices (128 B) and its stride
// byte offset the distance between MN-adjacent ones (CBLK). The nine planes and a constant plane
// of ones are stored back to back (plane stride 4 CBLK), so four consecutive planes x 32
// channels are one M = 128 operand with a uniform channel-block stride, and the dx taps are
// the same operand started 16 B (one voxel row) later. Per 16 voxels: 3 dx x 3 M tiles
// (planes 0-3, 4-7, 6-9; planes 6 and 7 of the last tile repeat the second tile's and are
// not read back) into nine TMEM accumulators of NP columns. The ones plane gives the bias
// gradient (its rows are sum_x dz[x][n] for every c).
//
// Each CTA takes a contiguous range of dz rows (consecutive y, so the h rows are re-read
// from L2), accumulates in TMEM for its whole range, and writes one partial of
// NOUT * 27 * 32 + NOUT floats; partials are added in a fixed order afterwards.
// Roles: warps 0-3 epilogue (TMEM lane quarters), warp 4 MMA issue, warp 5 TMA.
// ---------------------------------------------------------------------------------------
constexpr int WG_PLANES = 10;                    // nine (dz, dy) planes + the ones plane
constexpr int WG_CBLK = SLAB_ROWS * 16;          // one 8-channel block of an input row
constexpr int WG_PLANE = 4 * WG_CBLK;            // 32 channels
constexpr int WG_DBLK = CONV_M * 16;             // one 8-channel block of the dz row
constexpr int WG_STAGES = 2;
constexpr int WG_THREADS = 6 * 32;
constexpr int WG_TMEM_COLS = 512;

struct WgArgs {
  int B, G, xseg, nunits;
  uint32_t budget;
};

template <int NP>
constexpr int wg_stage_bytes() {
  return WG_PLANES * WG_PLANE + (NP / 8) * WG_DBLK;
}

template <int NP, int NOUT>
__global__ void __launch_bounds__(WG_THREADS, 1) wgrad_tc_kernel(const __grid_constant__ CUtensorMap hmap,
                                                                 const __grid_constant__ CUtensorMap dmap, WgArgs a,
                                                                 float *__restrict__ partial,
                                                                 unsigned *__restrict__ err) {
  constexpr int STAGE = wg_stage_bytes<NP>();
  constexpr uint32_t TX = 9u * 4u * SLAB * 16u + (uint32_t)(NP / 8) * CONV_M * 16u;
  constexpr uint32_t IDESC = idesc_bf16_f32(CONV_M, NP) | (1u << 15) | (1u << 16);  // A and B MN-major
  constexpr int LEN = NOUT * 27 * 32 + NOUT;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[WG_STAGES], empty[WG_STAGES], done;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = a.G;
  // this CTA's contiguous range of dz rows (units), y fastest
  const int u0 = (int)(((long long)a.nunits * blockIdx.x) / gridDim.x);
  const int u1 = (int)(((long long)a.nunits * (blockIdx.x + 1)) / gridDim.x);
  {  // the ones plane of every stage (bf16 1.0), never overwritten
    const uint4 one = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    for (int e = tid; e < WG_STAGES * (WG_PLANE / 16); e += WG_THREADS) {
      const int st = e / (WG_PLANE / 16), r = e % (WG_PLANE / 16);
      reinterpret_cast<uint4 *>(smem + (size_t)st * STAGE + 9 * WG_PLANE)[r] = one;
    }
  }
  if (tid == 0) {
    for (int i = 0; i < WG_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&done, 1);
    s_abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, WG_TMEM_COLS);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t base0 = smem_u32(smem);
  volatile int *abort_flag = &s_abort;
  auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
    for (uint32_t i = 0; i < a.budget; ++i) {
      if (mbar_try_wait(bar, parity)) return true;
      if ((i & 255u) == 255u && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
  };
  auto unit_coords = [&](int u, int &b, int &z, int &y, int &x0) {
    const int xs = u % a.xseg;
    int t = u / a.xseg;
    y = t % G;
    t /= G;
    z = t % G;
    b = t / G;
    x0 = xs * CONV_M;
  };

  if (warp == 5) {
    // ---- TMA: the nine neighbour rows (130 voxels from x0 - 1) and the dz row (128 voxels) ----
    if (lane == 0) {
      uint32_t issued = 0;
      for (int u = u0; u < u1; ++u) {
        const uint32_t i = (uint32_t)(u - u0), slot = i % WG_STAGES, n = i / WG_STAGES;
        if (n > 0 && !wait(&empty[slot], (n - 1) & 1u)) break;
        int b, z, y, x0;
        unit_coords(u, b, z, y, x0);
        const uint32_t dst = base0 + slot * STAGE;
        mbar_expect_tx(&full[slot], TX);
        for (int p = 0; p < 9; ++p)
#pragma unroll
          for (int cb = 0; cb < 4; ++cb)
            tma_load5(dst + (uint32_t)(p * WG_PLANE + cb * WG_CBLK), &hmap, cb * 8, x0 - 1, y + p % 3 - 1,
                      z + p / 3 - 1, b, &full[slot]);
#pragma unroll
        for (int nb = 0; nb < NP / 8; ++nb)
          tma_load5(dst + (uint32_t)(WG_PLANES * WG_PLANE + nb * WG_DBLK), &dmap, nb * 8, x0, y, z, b, &full[slot]);
        issued = i + 1;
      }
      // tail: the last copies have landed before the CTA can exit (also after an abort)
      for (uint32_t r = (issued > WG_STAGES ? issued - WG_STAGES : 0); r < issued; ++r)
        if (!mbar_wait_bounded(&full[r % WG_STAGES], (r / WG_STAGES) & 1u, DRAIN_BUDGET)) *abort_flag = 1;
    }
  } else if (warp == 4) {
    // ---- MMA issue ---------------------------------------------------------------------------
    if (lane == 0) {
      bool first = true;
      for (int u = u0; u < u1; ++u) {
        const uint32_t i = (uint32_t)(u - u0), slot = i % WG_STAGES;
        if (!wait(&full[slot], (i / WG_STAGES) & 1u)) break;
        tc_fence_after();
        int b, z, y, x0;
        unit_coords(u, b, z, y, x0);
        const int ks_n = (min(CONV_M, G - x0) + 15) / 16;
        const uint32_t sb = base0 + slot * STAGE;
        for (int ks = 0; ks < ks_n; ++ks) {
          const uint64_t bd = smem_desc(sb + (uint32_t)(WG_PLANES * WG_PLANE + ks * 256), 128, WG_DBLK);
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int t = 0; t < 3; ++t) {
              const int p0 = t == 0 ? 0 : (t == 1 ? 4 : 6);
              const uint64_t ad = smem_desc(sb + (uint32_t)(p0 * WG_PLANE + (ks * 16 + dx) * 16), 128, WG_CBLK);
              umma_bf16(tmem + (uint32_t)((t * 3 + dx) * NP), ad, bd, IDESC, first ? 0u : 1u);
            }
          first = false;
        }
        umma_commit(&empty[slot]);
      }
      // every MMA (and every commit's arrival) completes before the epilogue reads TMEM and
      // before the CTA exits, also after an abort
      umma_commit(&done);
      if (!mbar_wait_bounded(&done, 0u, DRAIN_BUDGET)) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp q reads TMEM lanes 32q .. 32q + 31 = plane p0 + q, channel = lane ----------
    const int q = warp;
    const bool ok = wait(&done, 0u);
    tc_fence_after();
    float *out = partial + (size_t)blockIdx.x * LEN;
    const bool any = u1 > u0 && ok;  // accumulators hold this CTA's sums (else write zeros)
    for (int t = 0; t < 3; ++t) {
      const int p = (t == 0 ? 0 : (t == 1 ? 4 : 6)) + q;
      if (t == 2 && q < 2) continue;  // planes 6 and 7 again
      for (int dx = 0; dx < 3; ++dx) {
        if (p == 9 && dx != 1) continue;
        float v[NP];
        const uint32_t ta = tmem + (uint32_t)((t * 3 + dx) * NP) + ((uint32_t)(q * 32) << 16);
        if (any) {
          if constexpr (NP == 32) tmem_ld32(ta, v);
          else tmem_ld16(ta, v);
        }
        if (p == 9) {
          if (lane == 0)
#pragma unroll
            for (int n = 0; n < NOUT; ++n) out[NOUT * 27 * 32 + n] = any ? v[n] : 0.f;
        } else {
          const int tap = (p / 3) * 9 + (p % 3) * 3 + dx;
#pragma unroll
          for (int n = 0; n < NOUT; ++n) out[(n * 27 + tap) * 32 + lane] = any ? v[n] : 0.f;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && *abort_flag) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, WG_TMEM_COLS);
  }
}

__global__ void reduce_partials_kernel(const float *__restrict__ partial, int nparts, int len,
                                       float *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  float s = 0.f;
  for (int k = 0; k < nparts; ++k) s += partial[(size_t)k * len + e];
  out[e] = s;
}

// fp32 w[n][tap][c] -> bf16 tensor-core B operand. 3-channel-padded layers (CIN >= 16) use the
// row layout of conv_tc_kernel: for each dx a K x NR block, K = (dz, c) = 3 CIN, NR = (dy, n) =
// 3 N, stored [dx][K / 8][NR][8]. The input layer (CIN = 2) uses the flat layout K = (tap, c)
// of conv_in_tc_kernel, [K / 8][N][8]. flip builds the data-gradient operand (taps mirrored,
// input and output channels exchanged).
__global__ void prep_weights_kernel(const float *__restrict__ w, int Nreal, int Creal, int CIN, int N, int flip,
                                    bf16 *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 27 * CIN * N) return;
  int tap, c, n;
  size_t idx;
  if (CIN < 8) {  // flat K = tap * CIN + c
    const int K = 27 * CIN;
    n = e / K;
    const int k = e % K;
    tap = k / CIN;
    c = k % CIN;
    idx = ((size_t)(k / 8) * N + n) * 8 + (k % 8);
  } else {  // rows: e = ((dx * K) + k) * NR + nr
    const int K = 3 * CIN, NR = 3 * N;
    const int dx = e / (K * NR);
    const int rem = e % (K * NR);
    const int k = rem / NR, nr = rem % NR;
    const int dz = k / CIN, dy = nr / N;
    c = k % CIN;
    n = nr % N;
    tap = (dz * 3 + dy) * 3 + dx;
    idx = (((size_t)dx * (K / 8) + k / 8) * NR + nr) * 8 + (k % 8);
  }
  float v = 0.f;
  if (!flip) {
    if (n < Nreal && c < Creal) v = w[(n * 27 + tap) * Creal + c];
  } else {
    // output channel n of the transposed conv is input channel n of the forward conv;
    // reduction channel c is forward output channel c
    if (c < Nreal && n < Creal) v = w[(c * 27 + (26 - tap)) * Creal + n];
  }
  out[idx] = __float2bfloat16_rn(v);
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

// tries of a pipeline wait in the tensor-core kernels (augur_cnn_set_wait_budget)
std::atomic<uint32_t> g_wait_budget{WAIT_BUDGET};

// cuTensorMapEncodeTiled through the runtime's driver entry-point query (no link against
// libcuda); resolved once.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  });
  return fn;
}

template <int CIN>
int make_act_map(CUtensorMap *map, const void *in, int B, int G) {
  auto fn = encode_fn();
  if (!fn || (reinterpret_cast<uintptr_t>(in) & 15) != 0) return AUGUR_EINVAL;
  const cuuint64_t dim[5] = {(cuuint64_t)CIN, (cuuint64_t)G, (cuuint64_t)G, (cuuint64_t)G, (cuuint64_t)B};
  const cuuint64_t stride[4] = {(cuuint64_t)CIN * 2, (cuuint64_t)G * CIN * 2, (cuuint64_t)G * G * CIN * 2,
                                (cuuint64_t)G * G * G * CIN * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)SLAB, 1, 1, 1};
  const cuuint32_t estride[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(in), dim, stride, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? AUGUR_OK : AUGUR_EINVAL;
}

template <int CIN, int N, int EPI>
int launch_conv_tc(const void *in, const void *wB, const float *bias, const void *resid, const void *zprev,
                   void *out0, void *out1, int B, int G, float out_scale, unsigned *err, double *stats,
                   cudaStream_t st) {
  ConvArgs a;
  a.B = B;
  a.G = G;
  a.xseg = (G + CONV_M - 1) / CONV_M;
  const int nsm = current_sm_count();
  a.rows = (long long)B * G * a.xseg * G;
  a.out_scale = out_scale;
  a.budget = g_wait_budget.load();
  // input activations [B][G][G][G][CIN] bf16 as a 5D tensor (c, x, y, z, b); box = 8 channels x
  // SLAB voxels of one row; outside the grid the box reads zeros (the convolution's padding)
  CUtensorMap map;
  if (make_act_map<CIN>(&map, in, B, G) != AUGUR_OK) return AUGUR_ECUDA;
  constexpr int WBYTES = 27 * CIN * N * 2;
  const size_t smem = ((WBYTES + 127) / 128) * 128 + (size_t)RING * 3 * (CIN / 8) * SLAB_ROWS * 16;
  if (raise_dyn_smem((const void *)conv_tc_kernel<CIN, N, EPI>, smem)) return AUGUR_ECUDA;
  const int grid = (int)std::min<long long>(a.rows, nsm);
  conv_tc_kernel<CIN, N, EPI><<<grid, CONV_THREADS, smem, st>>>(map, (const bf16 *)wB, bias, resid,
                                                                (const bf16 *)zprev, out0, (bf16 *)out1, a, err, stats);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

int launch_conv_in_tc(const void *x, const void *wB, const float *bias, void *z0, void *h0, int B, int G,
                      unsigned *err, cudaStream_t st) {
  ConvArgs a;
  a.B = B;
  a.G = G;
  a.xseg = (G + CONV_M - 1) / CONV_M;
  const int nsm = current_sm_count();
  a.rows = (long long)B * G * a.xseg * G;
  a.out_scale = 1.f;
  a.budget = g_wait_budget.load();
  const size_t smem = (size_t)IN_KB * 32 * 16 + (size_t)IN_STAGES * IN_ABYTES;
  if (raise_dyn_smem((const void *)conv_in_tc_kernel, smem)) return AUGUR_ECUDA;
  const int grid = (int)std::min<long long>(a.rows, nsm);
  conv_in_tc_kernel<<<grid, IN_THREADS, smem, st>>>((const bf16 *)x, (const bf16 *)wB, bias, (bf16 *)z0, (bf16 *)h0,
                                                    a, err);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

// (B, G, G, G, C) bf16 channels-last as a 5D tensor (c, x, y, z, b) with a box of 8 channels x
// boxx voxels of one row; out-of-range boxes read zeros.
int make_rows_map(CUtensorMap *map, const void *ptr, int C, int B, int G, int boxx) {
  auto fn = encode_fn();
  if (!fn || (reinterpret_cast<uintptr_t>(ptr) & 15) != 0 || C % 8 != 0) return AUGUR_EINVAL;
  const cuuint64_t dim[5] = {(cuuint64_t)C, (cuuint64_t)G, (cuuint64_t)G, (cuuint64_t)G, (cuuint64_t)B};
  const cuuint64_t stride[4] = {(cuuint64_t)C * 2, (cuuint64_t)G * C * 2, (cuuint64_t)G * G * C * 2,
                                (cuuint64_t)G * G * G * C * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)boxx, 1, 1, 1};
  const cuuint32_t estride[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(ptr), dim, stride, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? AUGUR_OK : AUGUR_EINVAL;
}

// weight gradient on tcgen05: h (B, G^3, 32) bf16, dz (B, G^3, NP) bf16; NOUT gradient channels
// are written (out: NOUT * 27 * 32 weights, then NOUT biases)
template <int NP, int NOUT>
int launch_wgrad_tc(const void *h, const void *dz, int B, int G, float *partial, int max_parts, float *out,
                    unsigned *err, cudaStream_t st) {
  if (G < 3 || !err) return AUGUR_EINVAL;
  WgArgs a;
  a.B = B;
  a.G = G;
  a.xseg = (G + CONV_M - 1) / CONV_M;
  a.nunits = B * G * G * a.xseg;
  a.budget = g_wait_budget.load();
  CUtensorMap hmap, dmap;
  if (make_rows_map(&hmap, h, 32, B, G, SLAB) != AUGUR_OK || make_rows_map(&dmap, dz, NP, B, G, CONV_M) != AUGUR_OK)
    return AUGUR_EINVAL;
  const int nparts = std::min(std::min(max_parts, current_sm_count()), a.nunits);
  const size_t smem = (size_t)WG_STAGES * wg_stage_bytes<NP>();
  if (raise_dyn_smem((const void *)wgrad_tc_kernel<NP, NOUT>, smem)) return AUGUR_ECUDA;
  wgrad_tc_kernel<NP, NOUT><<<nparts, WG_THREADS, smem, st>>>(hmap, dmap, a, partial, err);
  const int len = NOUT * 27 * 32 + NOUT;
  reduce_partials_kernel<<<(len + 255) / 256, 256, 0, st>>>(partial, nparts, len, out);
  return cudaGetLastError() == cudaSuccess ? AUGUR_OK : AUGUR_ECUDA;
}

template <int CIN, int N, int DZF>
int launch_wgrad(const void *h, const void *dz, int B, int G, float *partial, int max_parts, float *out,
                 cudaStream_t st) {
  const int nrows = B * G * G;
  const int nsm = current_sm_count();
  int nparts = std::min(max_parts, std::min(nrows, nsm * 4));
  const int rows_per = (nrows + nparts - 1) / nparts;
  nparts = (nrows + rows_per - 1) / rows_per;
  // narrower layers get x ranges so that a CTA has 1024 threads (ranges may be short or empty
  // for small G); measured on GB300, two output channels per thread (NB = 2, 512 threads) is
  // slower for the 32 x 32 layers (21.9 -> 24.9 ms at batch 4, 128^3)
  constexpr int NB = 1;
  constexpr int XS = (CIN * N >= 1024) ? 1 : 1024 / (CIN * N);
  const size_t smem = std::max(((size_t)9 * (G + 2) * CIN + (size_t)G * N) * 4,
                               XS > 1 ? (size_t)XS * CIN * N * 28 * 4 : 0);
  if (smem > 227 * 1024) return AUGUR_EINVAL;
  if (raise_dyn_smem((const void *)wgrad_kernel<CIN, N, DZF, XS, NB>, smem)) return AUGUR_ECUDA;
  wgrad_kernel<CIN, N, DZF, XS, NB><<<nparts, CIN * (N / NB) * XS, smem, st>>>((const bf16 *)h, dz, B, G, rows_per,
                                                                              partial);
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
                      unsigned *err, double *stats, void *stream) {
  if (!in || !w_umma || !out0 || batch < 1 || grid < 3 || !err) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  switch (layer) {
    case 0: return launch_conv_tc<32, 32, EPI_FWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, nullptr, st);
    case 1: return launch_conv_tc<32, 16, EPI_OUT>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, out_scale, err, stats, st);
    case 2: return launch_conv_tc<32, 32, EPI_BWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, nullptr, st);
    case 3: return launch_conv_tc<16, 32, EPI_BWD>(in, w_umma, bias, resid, zprev, out0, out1, batch, grid, 1.f, err, nullptr, st);
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

int augur_cnn_conv_in_tc(const void *x, const void *w_umma, const float *bias, int batch, int grid, void *z0,
                         void *h0, unsigned *err, void *stream) {
  if (!x || !w_umma || !bias || !h0 || !err || batch < 1 || grid < 3) return AUGUR_EINVAL;
  if ((reinterpret_cast<uintptr_t>(x) & 3) != 0) return AUGUR_EINVAL;
  return launch_conv_in_tc(x, w_umma, bias, z0, h0, batch, grid, err, (cudaStream_t)stream);
}

// kind: 0 = 32 -> 32 (dz bf16, tcgen05), 1 = output layer 32 -> 3 (dz = output gradient, fp32
// float4 grid, CUDA cores), 2 = input layer 2 -> 32 (dz bf16, CUDA cores), 3 = output layer from
// the 16-channel bf16 gradient of augur_cnn_pack_dout (tcgen05), 4 = 32 -> 32 on the CUDA cores.
// out: N*27*CIN weight gradients then N bias gradients (N = 4 for the output layer); partial:
// scratch of max_parts * (N*27*CIN + N) floats. err: the error word of the tcgen05 kinds.
int augur_cnn_wgrad(int kind, const void *h, const void *dz, int batch, int grid, float *partial, int max_parts,
                    float *out, unsigned *err, void *stream) {
  if (!h || !dz || !partial || !out || max_parts < 1 || batch < 1 || grid < 3) return AUGUR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  switch (kind) {
    case 0: return launch_wgrad_tc<32, 32>(h, dz, batch, grid, partial, max_parts, out, err, st);
    case 1: return launch_wgrad<32, 4, 1>(h, dz, batch, grid, partial, max_parts, out, st);
    case 2: return launch_wgrad<2, 32, 0>(h, dz, batch, grid, partial, max_parts, out, st);
    case 3: return launch_wgrad_tc<16, 4>(h, dz, batch, grid, partial, max_parts, out, err, st);
    case 4: return launch_wgrad<32, 32, 0>(h, dz, batch, grid, partial, max_parts, out, st);
    default: return AUGUR_EINVAL;
  }
}

unsigned augur_cnn_set_wait_budget(unsigned tries) { return g_wait_budget.exchange(tries); }

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
