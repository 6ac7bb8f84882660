// pm_kernels.cuh — device kernels of the PM gravity step (sm_103a).
//
// Data layout in HBM (x fastest everywhere):
//   sorted body state  pos4[i] = (x, y, z, m*mask), vel4[i] = (vx, vy, vz, bits(id | maskbit))
//   row histogram      one counter per grid row (3D periodic: row = z*G + y of the CIC base
//                      cell; 2D isolated: row = y0+1, plus one discard bucket)
//   half spectrum      spec[kx][row]  (kx = 0..L/2), complex64 — rows contiguous, so the
//                      y transform reads contiguous lines and the z transform reads
//                      128-byte column strips
//   force grid         F4[cell] = (a_x, a_y, a_z, phi) float4, so the gather is one 128-bit
//                      load per CIC corner
#pragma once
#include <type_traits>

#include "augur_common.cuh"
#include "tcgen05.cuh"

namespace augur {

constexpr int SCAN_TILE = 4096;  // rows per local scan tile (1024 threads x 4)
// tries of a bounded mbarrier wait in the TMA-fed kernels, and of the wait for a CTA's own copies
// in flight before it exits after giving up
constexpr uint32_t PM_WAIT_BUDGET = 1u << 20;
constexpr uint32_t PM_DRAIN_BUDGET = 1u << 22;

// The dynamic shared memory of the TMA-fed kernels, rounded up to a 128-byte boundary in the shared
// window (their launches request 128 bytes more than they use).
__device__ __forceinline__ unsigned char *smem_align128(unsigned char *p) {
  const uint32_t a = smem_u32(p);
  return p + (((a + 127u) & ~127u) - a);
}
// Checks a copy's addresses before it is issued: the shared destination or source 128-byte aligned
// (16 for plain bulk copies), the global address and byte count 16-byte aligned. A copy that fails
// is not issued; the caller raises AUGUR_ERRBIT_RANGE and gives up (its waits would never end).
__device__ __forceinline__ bool copy_ok(uint32_t s_addr, uint32_t s_align, const void *g, uint32_t bytes) {
  return (s_addr & (s_align - 1u)) == 0u && (reinterpret_cast<uintptr_t>(g) & 15u) == 0u && (bytes & 15u) == 0u;
}
constexpr int MAXSEG = 64;

struct GridParams {
  int G;          // cells per side
  int D;          // 2 or 3
  int periodic;   // 1 periodic, 0 isolated (out-of-grid corners dropped)
  int nrow;       // histogram buckets
  float h;        // fp32(extent / G)
  float half_ext; // fp32(extent / 2)
  float ext;      // fp32(extent)
  float inv_hD;   // fp32(1 / h^D) (density scale of ScatterField.scatter, in_scale = 1)
  float inv_h;    // 1/h when h is a power of two (exact), else 0 (use the IEEE division)
};

// fixed-point scale of the deposit, derived on the device from max(m*mask)
struct QScale {
  float qs1, qs2;   // contribution * qs1 * qs2 = contribution * 2^S (both exact)
  float outscale;   // 2^-S / h^D
};

__device__ __forceinline__ QScale qscale_from_mmax(const unsigned *mmax_bits, float inv_hD) {
  float mmax = __uint_as_float(*mmax_bits);
  int e = 0;
  if (mmax > 0.f) frexpf(mmax, &e);  // mmax = f * 2^e, f in [0.5, 1)
  // every contribution c <= mmax < 2^e, so c * 2^(26-e) < 2^26 and the sum of one warp's
  // 32 quanta fits a 32-bit reduction
  int S = 26 - e;
  int S1 = S / 2, S2 = S - S1;
  QScale q;
  q.qs1 = ldexpf(1.f, S1);
  q.qs2 = ldexpf(1.f, S2);
  q.outscale = ldexpf(inv_hD, -S);
  return q;
}

__device__ __forceinline__ uint32_t row_begin(const uint32_t *start, const uint32_t *tile_off, uint32_t r) {
  return tile_off[r / SCAN_TILE] + start[r];
}

// Base-cell row key. 3D periodic: wrap(iz)*G + wrap(iy). 2D isolated: iy+1 in [0, G]
// when some corner lands on the grid, else the discard bucket G+1.
__device__ __forceinline__ uint32_t row_key(const GridParams &g, int ix, int iy, int iz) {
  if (g.D == 3) {
    return (uint32_t)(fwrap(iz, g.G) * g.G + fwrap(iy, g.G));
  }
  if (g.periodic) return (uint32_t)fwrap(iy, g.G);
  bool on = (ix >= -1) && (ix < g.G) && (iy >= -1) && (iy < g.G);
  return on ? (uint32_t)(iy + 1) : (uint32_t)(g.G + 1);
}

// Warp-aggregated slot within a row: one atomicAdd per distinct key per warp (in sorted order
// the lanes of a warp share a few row keys even after a drift has moved some of them; adding per
// run of equal adjacent keys instead measured 80 -> 128 us for the gather at 3M bodies, from the
// extra adds on the same hot row counters).
// All 32 lanes must call this together.
__device__ __forceinline__ uint32_t warp_slot(uint32_t *row_count, uint32_t key, bool valid) {
  const int lane = threadIdx.x & 31;
  unsigned peers = __match_any_sync(0xffffffffu, valid ? key : 0xffffffffu);
  uint32_t base = 0;
  if (valid) {
    int leader = __ffs(peers) - 1;
    if (lane == leader) base = atomicAdd(&row_count[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    base += __popc(peers & ((1u << lane) - 1u));
  }
  return base;
}

// ---------------------------------------------------------------------------------
// K1: keys + histogram from caller (AoS) arrays. Optional velocity-Verlet drift
// pos += dt*vel + (dt^2/2)*acc in the reference's fp32 order (scripts/scatter_field.py:685),
// written back in place (periodic mode wraps into the box).
// Also reduces max(m*mask) for the deposit's fixed-point scale.
// ---------------------------------------------------------------------------------
template <int D, bool DRIFT>
__global__ void __launch_bounds__(256) keys_hist_aos_kernel(float *__restrict__ pos, const float *__restrict__ vel,
                                                            const float *__restrict__ acc, const float *__restrict__ mass,
                                                            const float *__restrict__ mask, int64_t n, GridParams g,
                                                            float dt, float hdt2, uint32_t *__restrict__ key,
                                                            uint32_t *__restrict__ slot, uint32_t *__restrict__ row_count,
                                                            unsigned *__restrict__ mmax_bits, unsigned *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  uint32_t k = 0;
  float mm = 0.f;
  if (valid) {
    float x[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d) x[d] = pos[i * D + d];
    if (DRIFT) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        float t = __fadd_rn(x[d], __fmul_rn(dt, vel[i * D + d]));
        t = __fadd_rn(t, __fmul_rn(hdt2, acc[i * D + d]));
        if (g.periodic) {
          if (t >= g.half_ext) t = __fsub_rn(t, g.ext);
          else if (t < -g.half_ext) t = __fadd_rn(t, g.ext);
        }
        x[d] = t;
        pos[i * D + d] = t;
      }
    }
    int i0[3] = {0, 0, 0};
    float w;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < D; ++d) ok &= cic_axis(x[d], g.half_ext, g.h, i0[d], w, g.inv_h);
    if (!ok) set_err(err, AUGUR_ERRBIT_NONFINITE);
    k = row_key(g, i0[0], i0[1], i0[2]);
    mm = __fmul_rn(mass[i], mask[i]);
  }
  uint32_t s = warp_slot(row_count, k, valid);
  if (valid) {
    key[i] = k;
    slot[i] = s;
  }
  // block max of m*mask (non-negative floats order like their bit patterns)
  unsigned b = valid ? __float_as_uint(fmaxf(mm, 0.f)) : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  if ((threadIdx.x & 31) == 0 && b) atomicMax(mmax_bits, b);
}

// ---------------------------------------------------------------------------------
// Scan of the row histogram: local exclusive scan per 4096-row tile (and the
// counters are cleared for the next histogram), then one block scans the tile totals.
// row_begin(r) = tile_off[r / 4096] + start[r] for any r <= nrow.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void scan_local_kernel_body(uint32_t *__restrict__ count, uint32_t *__restrict__ start,
                                                          uint32_t *__restrict__ tile_sum, int nrow, const int bx) {
  __shared__ uint32_t wsum[32];
  const int tile = bx;
  const int base = tile * SCAN_TILE + threadIdx.x * 4;
  uint32_t v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int r = base + q;
    v[q] = (r < nrow) ? count[r] : 0u;
    if (r < nrow) count[r] = 0u;
  }
  uint32_t local = v[0] + v[1] + v[2] + v[3];
  // warp inclusive scan
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = wsum[lane];
    uint32_t si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    wsum[lane] = si - s;  // exclusive
    if (lane == 31) tile_sum[tile] = si;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + inc - local;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    start[base + q] = run;  // start is sized (ntiles + 1) * 4096, zero beyond nrow
    run += v[q];
  }
}

__global__ void __launch_bounds__(1024) scan_local_kernel(uint32_t *__restrict__ count, uint32_t *__restrict__ start,
                                                          uint32_t *__restrict__ tile_sum, int nrow) {
  scan_local_kernel_body(count, start, tile_sum, nrow, (int)blockIdx.x);
}

__device__ __forceinline__ void scan_tiles_kernel_body(const uint32_t *__restrict__ tile_sum,
                                                          uint32_t *__restrict__ tile_off, int ntiles, const int bx) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b0 = 0; b0 < ntiles; b0 += 1024) {
    int t = b0 + threadIdx.x;
    uint32_t v = t < ntiles ? tile_sum[t] : 0u;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = wsum[lane], si = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, si, o);
        if (lane >= o) si += u;
      }
      wsum[lane] = si - s;
    }
    __syncthreads();
    uint32_t c = carry;
    if (t < ntiles) tile_off[t] = c + wsum[warp] + inc - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + wsum[warp] + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_off[ntiles] = carry;
}

__global__ void __launch_bounds__(1024) scan_tiles_kernel(const uint32_t *__restrict__ tile_sum,
                                                          uint32_t *__restrict__ tile_off, int ntiles) {
  scan_tiles_kernel_body(tile_sum, tile_off, ntiles, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------------
// Scatter bodies to their sorted slot. From caller AoS arrays (FROM_AOS) or from the
// previous sorted state (run loop).
// ---------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) scatter_aos_kernel(const float *__restrict__ pos, const float *__restrict__ vel,
                                                          const float *__restrict__ mass, const float *__restrict__ mask,
                                                          int64_t n, const uint32_t *__restrict__ key,
                                                          const uint32_t *__restrict__ slot,
                                                          const uint32_t *__restrict__ start,
                                                          const uint32_t *__restrict__ tile_off, float4 *__restrict__ pos4,
                                                          float4 *__restrict__ vel4) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t dst = row_begin(start, tile_off, key[i]) + slot[i];
  float mk = mask[i];
  float4 p = make_float4(pos[i * D], pos[i * D + 1], D == 3 ? pos[i * D + 2] : 0.f, __fmul_rn(mass[i], mk));
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (vel) {
    v.x = vel[i * D];
    v.y = vel[i * D + 1];
    if (D == 3) v.z = vel[i * D + 2];
  }
  uint32_t id = (uint32_t)i | (mk == 0.f ? 0x80000000u : 0u);
  v.w = __uint_as_float(id);
  pos4[dst] = p;
  vel4[dst] = v;
}

__device__ __forceinline__ void scatter_sorted_kernel_body(const float4 *__restrict__ pos_in,
                                                             const float4 *__restrict__ vel_in, int64_t n,
                                                             const uint32_t *__restrict__ key,
                                                             const uint32_t *__restrict__ slot,
                                                             const uint32_t *__restrict__ start,
                                                             const uint32_t *__restrict__ tile_off,
                                                             float4 *__restrict__ pos_out, float4 *__restrict__ vel_out, const int bx) {
  const int64_t i = (int64_t)bx * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t dst = row_begin(start, tile_off, key[i]) + slot[i];
  pos_out[dst] = pos_in[i];
  vel_out[dst] = vel_in[i];
}

__global__ void __launch_bounds__(256) scatter_sorted_kernel(const float4 *__restrict__ pos_in,
                                                             const float4 *__restrict__ vel_in, int64_t n,
                                                             const uint32_t *__restrict__ key,
                                                             const uint32_t *__restrict__ slot,
                                                             const uint32_t *__restrict__ start,
                                                             const uint32_t *__restrict__ tile_off,
                                                             float4 *__restrict__ pos_out, float4 *__restrict__ vel_out) {
  scatter_sorted_kernel_body(pos_in, vel_in, n, key, slot, start, tile_off, pos_out, vel_out, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------------
// Deposit geometry: row blocks of RY x RZ grid rows and their work items.
// ---------------------------------------------------------------------------------
struct DepositArgs {
  GridParams g;
  int RY, RZ;
  FftShape fsh;   // complex length M = G/2 (MODE 1)
  int twmul;      // table stride for the length-M transform
  int Lt;         // twiddle table length
  int nblk;       // row blocks
  uint32_t chunk; // bodies per work item
  FastDiv fdG, fdRR, fdRY;
};

// Calls f(first, last, first_row_key) for every contiguous run of sorted bodies that can touch row
// block b: base rows [y0-1, y0+RY-1] x [z0-1, z0+RZ-1] (periodic wrap), or base rows
// y0-1 .. y0+RY-1 <-> keys y0 .. y0+RY for the isolated 2D grid.
template <int D, class F>
__device__ __forceinline__ void block_segments(const DepositArgs &a, int b, const uint32_t *start,
                                               const uint32_t *tile_off, F f) {
  const int G = a.g.G, RY = a.RY, RZ = a.RZ;
  const int nyb = G / RY;
  const int y0 = (b % nyb) * RY;
  const int z0 = (D == 3) ? (b / nyb) * RZ : 0;
  auto add = [&](uint32_t r0, uint32_t r1) {
    uint32_t lo = row_begin(start, tile_off, r0), hi = row_begin(start, tile_off, r1);
    if (hi > lo) f(lo, hi, r0);
  };
  auto ylist = [&](uint32_t rb) {
    if (RY < G) {
      int yh = wrap_idx(y0 - 1, G);
      add(rb + yh, rb + yh + 1);
      add(rb + y0, rb + y0 + RY);
    } else {
      add(rb, rb + G);
    }
  };
  if (D == 3) {
    const int nz = (RZ < G) ? RZ + 1 : G;
    const int zs = (RZ < G) ? z0 - 1 : 0;
    for (int t = 0; t < nz; ++t) ylist((uint32_t)wrap_idx(zs + t, G) * G);
  } else if (a.g.periodic) {
    ylist(0);
  } else {
    add(y0, y0 + RY + 1);
  }
}

// Work items: every row block gets max(1, ceil(bodies / chunk)) items. One CTA records each
// block's body segments (seg_tab[b] = {first body, prefix count} pairs), scans the per-block
// item counts into item_off (nblk + 1 entries) and slot_off (the 64-bit accumulator tile of each
// block split over more than one item), and lists the block of every item in item_blk.
constexpr int MAXSEGB = 32;  // segments per row block: 2 * (RZ + 1) with RZ <= 15
// Bodies per deposit work item at most: a work item adds each contribution q < 2^26 to a cell
// as two 13-bit halves in 32-bit shared accumulators, which cannot overflow for fewer than 2^19
// contributions per cell (one per body visit).
constexpr int64_t DEP_ITEM_MAX = (int64_t)1 << 19;

// One thread per row block (many CTAs): the block's body segments and its item count.
template <int D>
__device__ __forceinline__ void deposit_count_kernel_body(const uint32_t *__restrict__ start,
                                                            const uint32_t *__restrict__ tile_off, DepositArgs a,
                                                            uint32_t *__restrict__ nch, uint4 *__restrict__ seg_tab,
                                                            unsigned *__restrict__ err, const int bx) {
  const int b = bx * blockDim.x + threadIdx.x;
  if (b >= a.nblk) return;
  uint32_t cnt = 0;
  int ns = 0;
  uint4 *tab = seg_tab + (size_t)b * (MAXSEGB + 1);
  block_segments<D>(a, b, start, tile_off, [&](uint32_t lo, uint32_t hi, uint32_t row0) {
    if (ns < MAXSEGB) {
      tab[1 + ns] = make_uint4(lo, cnt, row0, 0u);
      ++ns;
      cnt += hi - lo;
    } else {
      set_err(err, AUGUR_ERRBIT_RANGE);
    }
  });
  tab[0] = make_uint4((uint32_t)ns, cnt, 0u, 0u);
  nch[b] = cnt == 0 ? 1u : (cnt + a.chunk - 1) / a.chunk;
}

template <int D>
__global__ void __launch_bounds__(256) deposit_count_kernel(const uint32_t *__restrict__ start,
                                                            const uint32_t *__restrict__ tile_off, DepositArgs a,
                                                            uint32_t *__restrict__ nch, uint4 *__restrict__ seg_tab,
                                                            unsigned *__restrict__ err) {
  deposit_count_kernel_body<D>(start, tile_off, a, nch, seg_tab, err, (int)blockIdx.x);
}

// One CTA: scan of the item counts into item_off and slot_off, and the block of every item.
template <int D>
__device__ __forceinline__ void deposit_plan_kernel_body(const uint32_t *__restrict__ start,
                                                            const uint32_t *__restrict__ tile_off, DepositArgs a,
                                                            uint32_t *__restrict__ nch, uint32_t *__restrict__ item_off,
                                                            uint32_t *__restrict__ slot_off,
                                                            uint4 *__restrict__ seg_tab, uint32_t *__restrict__ item_blk,
                                                            unsigned *__restrict__ err, const int bx) {
  __shared__ uint32_t wsum[2][32];
  const int nb = a.nblk, tid = threadIdx.x, nt = blockDim.x;
  const int per = (nb + nt - 1) / nt;
  const int b0 = min(nb, tid * per), b1 = min(nb, b0 + per);
  uint32_t si = 0, ss = 0;
  for (int b = b0; b < b1; ++b) {
    uint32_t c = nch[b];
    si += c;
    ss += c > 1 ? 1u : 0u;
  }
  const int lane = tid & 31, warp = tid >> 5;
  uint32_t ii = si, is = ss;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t u = __shfl_up_sync(0xffffffffu, ii, o), v = __shfl_up_sync(0xffffffffu, is, o);
    if (lane >= o) {
      ii += u;
      is += v;
    }
  }
  if (lane == 31) {
    wsum[0][warp] = ii;
    wsum[1][warp] = is;
  }
  __syncthreads();
  if (warp == 0) {
    uint32_t x = lane < (nt >> 5) ? wsum[0][lane] : 0u, y = lane < (nt >> 5) ? wsum[1][lane] : 0u;
    uint32_t xi = x, yi = y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, xi, o), v = __shfl_up_sync(0xffffffffu, yi, o);
      if (lane >= o) {
        xi += u;
        yi += v;
      }
    }
    wsum[0][lane] = xi - x;
    wsum[1][lane] = yi - y;
  }
  __syncthreads();
  uint32_t ri = wsum[0][warp] + ii - si, rs = wsum[1][warp] + is - ss;
  for (int b = b0; b < b1; ++b) {
    uint32_t c = nch[b];
    item_off[b] = ri;
    slot_off[b] = rs;
    for (uint32_t j = 0; j < c; ++j) item_blk[ri + j] = (uint32_t)b;
    ri += c;
    rs += c > 1 ? 1u : 0u;
  }
  if (tid == nt - 1) item_off[nb] = ri;
}

template <int D>
__global__ void __launch_bounds__(1024) deposit_plan_kernel(const uint32_t *__restrict__ start,
                                                            const uint32_t *__restrict__ tile_off, DepositArgs a,
                                                            uint32_t *__restrict__ nch, uint32_t *__restrict__ item_off,
                                                            uint32_t *__restrict__ slot_off,
                                                            uint4 *__restrict__ seg_tab, uint32_t *__restrict__ item_blk,
                                                            unsigned *__restrict__ err) {
  deposit_plan_kernel_body<D>(start, tile_off, a, nch, item_off, slot_off, seg_tab, item_blk, err, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------------
// K2 (+K3a): deterministic CIC deposit of one block of grid rows in fixed point (integer
// sums are associative, so the result is independent of body order and scheduling), then
// either written as float32 density rows (MODE 0) or transformed along x in shared
// memory (R2C, MODE 1) and written to the half spectrum spec[kx][row] (MODE 2: both).
//
// Block = RY consecutive y rows x RZ consecutive z planes (2D: RZ = 1). Bodies that
// touch the block are those whose base row lies in [y0-1, y0+RY-1] x [z0-1, z0+RZ-1];
// with the state sorted by base row they form at most 2*(RZ+1) contiguous segments.
// Each contribution q < 2^26 is added to its cell as two 13-bit halves (q & 8191, q >> 13)
// with 32-bit shared-memory reductions: on this part a 32-bit shared atomic add issues many
// times faster than a 64-bit one, and the halves cannot overflow (at most DEP_ITEM_MAX
// contributions per cell per work item); the cell's sum is hi * 2^13 + lo.
// A block with more than `chunk` bodies is split over several CTAs (work items); each
// adds its nonzero sums into the block's 64-bit tile in global memory (L2 reductions), and
// the CTA that finishes last (counter + threadfence, no waiting) reads the tile, clears it
// for the next call, and converts.
// ---------------------------------------------------------------------------------
// R2C post-process of a row block's M-point transforms Z (row stride MS) into the half spectrum:
// X_k = (Z_k + conj Z_{M-k})/2 - i/2 W^k (Z_k - conj Z_{M-k}), k = 0..M, at spec[kx][row].
template <int D>
__device__ __forceinline__ void deposit_r2c_post(const float2 *Z, int MS, int M, int RR, int G, int RY, int z0, int y0,
                                                 const DepositArgs &a, const float2 *tw, float2 *__restrict__ spec_out) {
  const int tstep = a.Lt / G;
  const size_t plane = (size_t)(D == 3 ? G : 1) * G;  // rows per kx plane
  auto post = [&](int kx, int rr) -> float2 {
    float2 zk = Z[rr * MS + (kx == M ? 0 : kx)];
    float2 zc = cconj(Z[rr * MS + (kx == 0 ? 0 : M - kx)]);
    float2 ev = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
    float2 od = make_float2(0.5f * (zk.x - zc.x), 0.5f * (zk.y - zc.y));
    float2 w = tw[kx * tstep];
    float2 t = cmul(w, od);
    return make_float2(ev.x + t.y, ev.y - t.x);  // ev - i*t
  };
  auto row_of = [&](int rr) -> size_t {
    const int zz = (int)fdiv(rr, a.fdRY), yy = rr - zz * RY;
    return (size_t)(z0 + zz) * G + (y0 + yy);
  };
  const int nt = blockDim.x;
  if (nt % RR == 0) {  // each thread keeps one row: kx = tid / RR, + nt / RR, ...
    const int rr = threadIdx.x % RR;
    float2 *dst = spec_out + row_of(rr);
    for (int kx = threadIdx.x / RR; kx <= M; kx += nt / RR) dst[(size_t)kx * plane] = post(kx, rr);
  } else {
    for (int e = threadIdx.x; e < (M + 1) * RR; e += nt) {
      const int kx = (int)fdiv(e, a.fdRR), rr = e - kx * RR;
      spec_out[(size_t)kx * plane + row_of(rr)] = post(kx, rr);
    }
  }
}

// adds q < 2^31 to cell c of the split accumulators (lo gets the low 13 bits, hi the rest)
__device__ __forceinline__ void dep_add(uint32_t *lo, uint32_t *hi, int c, uint32_t q) {
  if (q & 8191u) atomicAdd(&lo[c], q & 8191u);
  if (q >> 13) atomicAdd(&hi[c], q >> 13);
}

template <int D, int MODE, bool AGG>
__device__ __forceinline__ void deposit_kernel_body(const float4 *__restrict__ pos4,
                                                      const unsigned *__restrict__ mmax_bits, DepositArgs a,
                                                      const float2 *__restrict__ twg, float *__restrict__ rho_out,
                                                      float2 *__restrict__ spec_out, unsigned *__restrict__ err,
                                                      const uint32_t *__restrict__ item_off,
                                                      const uint32_t *__restrict__ slot_off,
                                                      const uint4 *__restrict__ seg_tab,
                                                      const uint32_t *__restrict__ item_blk,
                                                      unsigned long long *__restrict__ scratch,
                                                      unsigned *__restrict__ counters, const int bx) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ long long s_beg[MAXSEGB];
  __shared__ long long s_pre[MAXSEGB + 1];
  __shared__ uint32_t s_row[MAXSEGB];
  __shared__ int s_nseg, s_last;

  const GridParams &g = a.g;
  const int G = g.G, RY = a.RY, RZ = a.RZ, RR = RY * RZ;
  const int tid = threadIdx.x, nt = blockDim.x;
  const uint32_t item = bx;
  if (item >= item_off[a.nblk]) return;  // uniform across the CTA
  const int blk = (int)item_blk[item];
  const uint32_t part = item - item_off[blk];
  const uint32_t nparts = item_off[blk + 1] - item_off[blk];
  const int nyb = G / RY;
  const int y0 = (blk % nyb) * RY;
  const int z0 = (D == 3) ? (blk / nyb) * RZ : 0;
  const int RS = G + 2;                       // fp32 row stride (complex rows 8-byte aligned and padded)
  const int PS = fft_row_stride(G / 2);       // padded transform rows
  const size_t region = (size_t)RR * 2 * PS * 8;  // >= RR * G * 8: accumulator, then transform scratch

  // [accumulator halves lo, hi / transform scratch: region][fp32 rows: RR*RS*4][twiddles]
  uint32_t *acc_lo = reinterpret_cast<uint32_t *>(smem);
  uint32_t *acc_hi = acc_lo + (size_t)RR * G;
  float *rows = reinterpret_cast<float *>(smem + region);
  float2 *tw = reinterpret_cast<float2 *>(smem + region + (size_t)RR * RS * 4);

  const uint4 *tab = seg_tab + (size_t)blk * (MAXSEGB + 1);
  if (tid <= MAXSEGB) {
    uint4 t = tab[tid];
    if (tid == 0) {
      s_nseg = (int)t.x;
      s_pre[t.x] = t.y;  // total
    } else if (tid - 1 < (int)tab[0].x) {
      s_beg[tid - 1] = t.x;
      s_pre[tid - 1] = t.y;
      s_row[tid - 1] = t.z;
    }
  }
  for (int e = tid; e < RR * G / 2; e += nt) reinterpret_cast<uint4 *>(acc_lo)[e] = make_uint4(0u, 0u, 0u, 0u);
  if (MODE != 0)
    for (int e = tid; e < a.Lt; e += nt) tw[e] = twg[e];
  __syncthreads();

  const QScale qs = qscale_from_mmax(mmax_bits, g.inv_hD);
  const int nseg = s_nseg;
  const long long f_lo = (long long)part * a.chunk;
  const long long f_hi = min(s_pre[nseg], f_lo + (long long)a.chunk);
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;

  // One segment at a time: a segment is one base z row (one key range of sorted bodies), so
  // which z corners of its bodies fall inside the block is the same for the whole segment.
  // (the body loop is compiled twice, with the cell-index division resolved either way; the
  // choice made per body inside the loop cost 5 us at 3M bodies, 32-bit indices another 2-3 us)
  auto segments = [&](auto pow2) {
  constexpr bool POW2 = decltype(pow2)::value;
  for (int sg = 0; sg < nseg; ++sg) {
    const long long s0 = max(f_lo, s_pre[sg]), s1 = min(f_hi, s_pre[sg + 1]);
    if (s0 >= s1) continue;
    const long long bias = s_beg[sg] - s_pre[sg];  // sorted body index = bias + f
    int lzc[2] = {0, 0};
    bool zin[2] = {true, false};
    if (D == 3) {
      const int bz = (int)(s_row[sg] / (uint32_t)G);
#pragma unroll
      for (int oz = 0; oz < 2; ++oz) {
        int cz = bz + oz;
        if (cz == G) cz = 0;
        int lz = cz - z0;
        if (lz < 0) lz += G;
        lzc[oz] = lz;
        zin[oz] = lz < RZ;
      }
    }
    // body indices are below 2^31 (32-bit loop arithmetic)
    const int s1i = (int)s1;
    const float4 *pb = pos4 + bias;
    for (int f0 = (int)s0 + warp * 32; f0 < s1i; f0 += nwarp * 32) {
      const int f = f0 + lane;
      const bool valid = f < s1i;
      float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
      if (valid) p = pb[f];
      int ix = 0, iy = 0, iz = 0;
      float wx = 0.f, wy = 0.f, wz = 0.f;
      bool ok = cic_axis_t<POW2>(p.x, g.half_ext, g.h, g.inv_h, ix, wx) &
                cic_axis_t<POW2>(p.y, g.half_ext, g.h, g.inv_h, iy, wy);
      if (D == 3) ok &= cic_axis_t<POW2>(p.z, g.half_ext, g.h, g.inv_h, iz, wz);
      if (valid && !ok) set_err(err, AUGUR_ERRBIT_NONFINITE);
      const bool live = valid && ok && p.w > 0.f;
      // x corners: cells bx and bx1 of a row (periodic wrap or grid bounds)
      int bx = ix, bx1 = ix + 1;
      bool inx0 = true, inx1 = true;
      if (g.periodic) {
        bx = fwrap(ix, G);
        bx1 = (bx + 1 == G) ? 0 : bx + 1;
      } else {
        inx0 = (ix >= 0) && (ix < G);
        inx1 = (ix + 1 >= 0) && (ix + 1 < G);
      }
      // y corners: local rows of the block
      int lyc[2];
      bool yin[2];
      if (g.periodic) {
        const int by = fwrap(iy, G);
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
          int cy = by + oy;
          if (cy == G) cy = 0;
          int ly = cy - y0;
          if (ly < 0) ly += G;
          lyc[oy] = ly;
          yin[oy] = ly < RY;
        }
      } else {
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
          const int ly = iy + oy - y0;
          lyc[oy] = ly;
          yin[oy] = (ly >= 0) && (ly < RY) && (inx0 || inx1);
        }
      }
      const float wx0 = axis_w(wx, 0), wx1 = axis_w(wx, 1);
#pragma unroll
      for (int oz = 0; oz < (D == 3 ? 2 : 1); ++oz) {
        if (!zin[oz]) continue;  // uniform across the warp
        const float wzt = axis_w(wz, oz);
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
          // key identifies the (row, x pair) of this (y, z) corner pair; both x corners share it
          unsigned key = 0xffffffffu;
          uint32_t q0 = 0, q1 = 0;
          const int rowbase = (lzc[oz] * RY + lyc[oy]) * G;
          if (live && yin[oy]) {
            key = g.periodic ? (unsigned)(rowbase + bx) : (unsigned)(lyc[oy] * (G + 1) + ix + 1);
            // weight order of the reference: ((w_x * w_y) * w_z) * m
            const float wyt = axis_w(wy, oy);
            float w0 = __fmul_rn(wx0, wyt), w1 = __fmul_rn(wx1, wyt);
            if (D == 3) {
              w0 = __fmul_rn(w0, wzt);
              w1 = __fmul_rn(w1, wzt);
            }
            if (inx0) q0 = __float2uint_rz(__fmul_rn(__fmul_rn(__fmul_rn(w0, p.w), qs.qs1), qs.qs2));
            if (inx1) q1 = __float2uint_rz(__fmul_rn(__fmul_rn(__fmul_rn(w1, p.w), qs.qs1), qs.qs2));
          }
          const int c0 = g.periodic ? rowbase + bx : rowbase + ix;
          const int c1 = g.periodic ? rowbase + bx1 : rowbase + ix + 1;
          // AGG: warp aggregation when neighbouring lanes share a key (pays off only for cells
          // dense enough that many lanes of a warp hit the same one; otherwise the shared-memory
          // atomics resolve the few collisions faster than the vote and match)
          bool agg = false;
          if constexpr (AGG) {
            const unsigned prev = __shfl_up_sync(0xffffffffu, key, 1);
            const bool dup = (lane > 0) && (key != 0xffffffffu) && (prev == key);
            agg = __any_sync(0xffffffffu, dup);
          }
          if (agg) {
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            if (key != 0xffffffffu) {
              const uint32_t s0q = __reduce_add_sync(peers, q0);  // < 32 * 2^26
              const uint32_t s1q = __reduce_add_sync(peers, q1);
              if (lane == __ffs(peers) - 1) {
                dep_add(acc_lo, acc_hi, c0, s0q);
                dep_add(acc_lo, acc_hi, c1, s1q);
              }
            }
          } else if (key != 0xffffffffu) {
            dep_add(acc_lo, acc_hi, c0, q0);
            dep_add(acc_lo, acc_hi, c1, q1);
          }
        }
      }
    }
  }
  };
  if (g.inv_h != 0.f) segments(std::true_type{});
  else segments(std::false_type{});

  __syncthreads();

  unsigned long long *gtile = nullptr;
  if (nparts > 1) {
    // add this part's sums into the block's 64-bit tile; the last part to arrive converts it
    gtile = scratch + (size_t)slot_off[blk] * ((size_t)RR * G);
    for (int e = tid; e < RR * G; e += nt) {
      const unsigned long long v = ((unsigned long long)acc_hi[e] << 13) + acc_lo[e];
      if (v) atomicAdd(&gtile[e], v);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(&counters[blk], 1u) == nparts - 1) ? 1 : 0;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (tid == 0) counters[blk] = 0u;
  }

  // fixed point -> float32 density rows (MODE 0: to HBM, 1: to shared memory, 2: both), two
  // adjacent cells per thread and iteration (G is even: 64-bit shared loads and stores)
  // u64 -> f32 rounds correctly either way; the 32-bit conversion is a fast FP32-pipe instruction,
  // the 64-bit one is not on this part and is only needed for sums >= 2^32
  auto to_f32 = [&](unsigned long long q) {
    const float fq = (q >> 32) ? __ull2float_rn(q) : __uint2float_rn((unsigned)q);
    return __fmul_rn(fq, qs.outscale);
  };
  for (int e = 2 * tid; e < RR * G; e += 2 * nt) {
    int rr = (int)fdiv(e, a.fdG), x = e - rr * G;
    unsigned long long q0, q1;
    if (gtile) {  // the split block's total, and the tile cleared for the next call
      q0 = __ldcg(&gtile[e]);
      q1 = __ldcg(&gtile[e + 1]);
      gtile[e] = 0ull;
      gtile[e + 1] = 0ull;
    } else {
      const uint2 lo = *reinterpret_cast<const uint2 *>(&acc_lo[e]);
      const uint2 hi = *reinterpret_cast<const uint2 *>(&acc_hi[e]);
      q0 = ((unsigned long long)hi.x << 13) + lo.x;
      q1 = ((unsigned long long)hi.y << 13) + lo.y;
    }
    const float2 v = make_float2(to_f32(q0), to_f32(q1));
    if (MODE != 1) {
      int zz = (int)fdiv(rr, a.fdRY), yy = rr - zz * RY;
      size_t row = (size_t)(z0 + zz) * G + (y0 + yy);
      float *dst = &rho_out[row * G + x];
      if ((reinterpret_cast<uintptr_t>(rho_out) & 7) == 0) {  // a caller's array may be 4-byte aligned
        *reinterpret_cast<float2 *>(dst) = v;
      } else {
        dst[0] = v.x;
        dst[1] = v.y;
      }
    }
    if (MODE != 0) *reinterpret_cast<float2 *>(&rows[rr * RS + x]) = v;
  }
  if (MODE == 0) return;
  __syncthreads();

  // R2C along x: rows viewed as M = G/2 complex values, stride RS/2 = M+1; the transform
  // reads them, ping-pongs through the (now free) accumulator area and lands back on them
  const int M = G / 2, MS = M + 1;
  float2 *Z = reinterpret_cast<float2 *>(rows);
  float2 *TA = reinterpret_cast<float2 *>(smem);
  float2 *TB = TA + (size_t)RR * PS;
  {
    const float2 *src = Z;
    auto ld = [&](int b, int e) -> float2 { return src[b * MS + e]; };
    auto st = [&](int b, int e, float2 v) { Z[b * MS + e] = v; };
    AUGUR_FFT_IO(M, 0, RR, ld, st, TA, TB, PS, tw, a.twmul, false);
  }
  deposit_r2c_post<D>(Z, MS, M, RR, G, RY, z0, y0, a, tw, spec_out);
}

template <int D, int MODE, bool AGG>
__global__ void __launch_bounds__(256, 4) deposit_kernel(const float4 *__restrict__ pos4,
                                                      const unsigned *__restrict__ mmax_bits, DepositArgs a,
                                                      const float2 *__restrict__ twg, float *__restrict__ rho_out,
                                                      float2 *__restrict__ spec_out, unsigned *__restrict__ err,
                                                      const uint32_t *__restrict__ item_off,
                                                      const uint32_t *__restrict__ slot_off,
                                                      const uint4 *__restrict__ seg_tab,
                                                      const uint32_t *__restrict__ item_blk,
                                                      unsigned long long *__restrict__ scratch,
                                                      unsigned *__restrict__ counters) {
  deposit_kernel_body<D, MODE, AGG>(pos4, mmax_bits, a, twg, rho_out, spec_out, err, item_off, slot_off, seg_tab, item_blk, scratch, counters, (int)blockIdx.x);
}

// ---------------------------------------------------------------------------------
// Generic R2C of real rows (zero padded from Lin to L, rows >= nin are zero):
// out[kx * nout + r], kx = 0..L/2. Used for the Poisson solve from a given density
// grid and for the 2D isolated (2G zero-padded) transform.
// ---------------------------------------------------------------------------------
struct RowsArgs {
  int L, Lin, nin, nout, RB, Lt;
  FftShape fsh;  // complex length L/2
  int twmul;     // for the length L/2 transform
  FastDiv fdL, fdRB;
};

__global__ void __launch_bounds__(256) r2c_rows_kernel(const float *__restrict__ in, RowsArgs a,
                                                       const float2 *__restrict__ twg, float2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int L = a.L, M = L / 2, MS = M + 1, RB = a.RB, PS = fft_row_stride(M);
  float2 *A = reinterpret_cast<float2 *>(smem);
  float2 *B = A + (size_t)RB * MS;
  float2 *C = B + (size_t)RB * PS;
  float2 *tw = C + (size_t)RB * PS;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int r0 = blockIdx.x * RB;
  for (int e = tid; e < a.Lt; e += nt) tw[e] = twg[e];
  float *Af = reinterpret_cast<float *>(A);
  for (int e = tid; e < RB * L; e += nt) {
    int rr = (int)fdiv(e, a.fdL), x = e - rr * L;
    int r = r0 + rr;
    float v = 0.f;
    if (r < a.nin && x < a.Lin) v = in[(size_t)r * a.Lin + x];
    Af[rr * 2 * MS + x] = v;
  }
  __syncthreads();
  float2 *Z = A;
  {
    auto ld = [&](int b, int e) -> float2 { return A[b * MS + e]; };
    auto st = [&](int b, int e, float2 v) { Z[b * MS + e] = v; };
    AUGUR_FFT_IO(M, 0, RB, ld, st, B, C, PS, tw, a.twmul, false);
  }
  const int tstep = a.Lt / L;
  for (int e = tid; e < (M + 1) * RB; e += nt) {
    int kx = (int)fdiv(e, a.fdRB), rr = e - kx * RB;
    int r = r0 + rr;
    if (r >= a.nout) continue;
    float2 zk = Z[rr * MS + (kx == M ? 0 : kx)];
    float2 zc = cconj(Z[rr * MS + (kx == 0 ? 0 : M - kx)]);
    float2 ev = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
    float2 od = make_float2(0.5f * (zk.x - zc.x), 0.5f * (zk.y - zc.y));
    float2 t = cmul(tw[kx * tstep], od);
    out[(size_t)kx * a.nout + r] = make_float2(ev.x + t.y, ev.y - t.x);
  }
}

// In-place FFT of contiguous complex rows of length L (rows = lines along y): the first
// stage reads HBM, the last writes HBM, the stages between go through shared memory.
__device__ __forceinline__ void fft_rows_kernel_body(float2 *__restrict__ data, int64_t nrows, int RB, int L,
                                                       FastDiv fdL, int twmul, int Lt,
                                                       const float2 *__restrict__ twg, int inverse, const int bx) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int LS = fft_row_stride(L);
  float2 *A = reinterpret_cast<float2 *>(smem);
  float2 *B = A + (size_t)RB * LS;
  float2 *tw = B + (size_t)RB * LS;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int64_t r0 = (int64_t)bx * RB;
  const int nr = (int)min((int64_t)RB, nrows - r0);
  for (int e = tid; e < Lt; e += nt) tw[e] = twg[e];
  float2 *base = data + r0 * L;
  if (L <= 16) {  // single-stage lengths: stage through shared memory (in place)
    for (int e = tid; e < nr * L; e += nt) {
      int rr = (int)fdiv(e, fdL), x = e - rr * L;
      B[rr * LS + x] = base[(size_t)rr * L + x];
    }
    __syncthreads();
    auto ld = [&](int b, int e) -> float2 { return B[b * LS + e]; };
    auto st = [&](int b, int e, float2 v) { base[(size_t)b * L + e] = v; };
    AUGUR_FFT_IO(L, 0, nr, ld, st, A, A, LS, tw, twmul, inverse != 0);
    return;
  }
  __syncthreads();
  auto ld = [&](int b, int e) -> float2 { return base[(size_t)b * L + e]; };
  auto st = [&](int b, int e, float2 v) { base[(size_t)b * L + e] = v; };
  AUGUR_FFT_IO(L, 0, nr, ld, st, A, B, LS, tw, twmul, inverse != 0);
}

__global__ void __launch_bounds__(256) fft_rows_kernel(float2 *__restrict__ data, int64_t nrows, int RB, int L,
                                                       FastDiv fdL, int twmul, int Lt,
                                                       const float2 *__restrict__ twg, int inverse) {
  fft_rows_kernel_body(data, nrows, RB, L, fdL, twmul, Lt, twg, inverse, (int)blockIdx.x);
}

// Row transforms (fft_rows_kernel) as a persistent kernel fed by bulk copies: the CTA takes row
// batches blockIdx.x, + gridDim.x, ...; thread 0 keeps two batches' rows (contiguous, RB * L
// complex) in flight into a two-slot ring, the first stage reads them from the slot, the last
// stage writes the transformed rows back to global memory in place. Needs a multi-stage length
// (L >= 32). Bounded waits as c2r_tma_kernel.
constexpr int ROWST_STAGES = 2;
__global__ void __launch_bounds__(256, 2) rows_tma_kernel(float2 *__restrict__ data, int64_t nrows, int RB, int L,
                                                          int twmul, int Lt, const float2 *__restrict__ twg,
                                                          int inverse, unsigned *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_align128(smem_raw);
  __shared__ __align__(8) uint64_t full[ROWST_STAGES];
  __shared__ int s_issued, s_bad;  // copies thread 0 has issued; a copy that failed copy_ok()
  const int LS = fft_row_stride(L);
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t slot_elems = (size_t)RB * L;
  float2 *ring = reinterpret_cast<float2 *>(smem);
  float2 *A = ring + ROWST_STAGES * slot_elems;  // transforms of two stages only use B
  float2 *B = A + (fft_nstages(L) > 2 ? (size_t)RB * LS : 0);
  float2 *tw = B + (size_t)RB * LS;
  const int64_t nbatch = (nrows + RB - 1) / RB;
  const int nmine = (int64_t)blockIdx.x < nbatch ? (int)((nbatch - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto rows_of = [&](int i, int64_t &r0) {
    r0 = ((int64_t)blockIdx.x + (int64_t)i * gridDim.x) * RB;
    return (int)min((int64_t)RB, nrows - r0);
  };
  auto issue = [&](int i) {  // thread 0: batch i into its slot, unless its addresses fail the check
    int64_t r0;
    const int nr = rows_of(i, r0);
    const int slot = i % ROWST_STAGES;
    const uint32_t bytes = (uint32_t)nr * L * 8u;
    const uint32_t dst = smem_u32(ring + slot * slot_elems);
    if (!copy_ok(dst, 16u, data + r0 * L, bytes)) {
      s_bad = 1;
      return;
    }
    mbar_expect_tx(&full[slot], bytes);
    bulk_load(dst, data + r0 * L, bytes, &full[slot]);
    s_issued = i + 1;
  };
  if (tid == 0) {
    for (int i = 0; i < ROWST_STAGES; ++i) mbar_init(&full[i], 1);
    s_issued = 0;
    s_bad = 0;
    mbar_fence_init();
    for (int i = 0; i < min(nmine, ROWST_STAGES) && !s_bad; ++i) issue(i);
  }
  for (int e = tid; e < Lt; e += nt) tw[e] = twg[e];
  __syncthreads();
  int i = 0;
  bool abort = false;
  for (; i < nmine; ++i) {
    const int slot = i % ROWST_STAGES;
    int64_t r0;
    const int nr = rows_of(i, r0);
    const bool ok = i < s_issued && mbar_wait_bounded(&full[slot], (uint32_t)(i / ROWST_STAGES) & 1u, PM_WAIT_BUDGET);
    if (__syncthreads_or(!ok)) {
      abort = true;
      break;
    }
    const float2 *S = ring + slot * slot_elems;
    float2 *base = data + r0 * L;
    auto ld = [&](int b, int e) -> float2 { return S[(size_t)b * L + e]; };
    auto st = [&](int b, int e, float2 v) { base[(size_t)b * L + e] = v; };
    AUGUR_FFT_IO(L, 0, nr, ld, st, A, B, LS, tw, twmul, inverse != 0);
    // the slot was read by the first stage (a barrier ago): hand it to the copy engine again
    fence_async_smem();
    __syncthreads();
    if (tid == 0 && i + ROWST_STAGES < nmine && !s_bad) issue(i + ROWST_STAGES);
  }
  if (tid == 0) {
    for (int r = i; r < s_issued; ++r)  // every copy issued lands before the CTA exits
      if (!mbar_wait_bounded(&full[r % ROWST_STAGES], (uint32_t)(r / ROWST_STAGES) & 1u, PM_DRAIN_BUDGET))
        abort = true;
    if (s_bad) atomicOr(err, AUGUR_ERRBIT_RANGE);
    else if (abort) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
  }
}

// 2D isolated, kpad = "ext" (scripts/scatter_field.py:286-288): the central difference reads the
// potential's wrapped neighbours, E = phi at rows/columns -1 .. G of the 2G transform.
__global__ void fd_grad2d_ext_kernel(const float *__restrict__ E, int G, float two_h, float4 *__restrict__ F4) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G * G) return;
  int y = e / G, x = e - y * G;
  const int W = G + 2;
  const float *c = E + (size_t)(y + 1) * W + (x + 1);
  float gx = __fdiv_rn(__fsub_rn(c[1], c[-1]), two_h);
  float gy = __fdiv_rn(__fsub_rn(c[W], c[-W]), two_h);
  F4[e] = make_float4(-gx, -gy, 0.f, c[0]);
}

// Learned radial kernel on the 2G x 2G minimum-image lattice (ScatterField._kernel_fft,
// scripts/scatter_field.py:263-272): K = kmlp(features(r)), kmlp = Linear(ncol, 64), GELU,
// Linear(64, 64), GELU, Linear(64, 1) (torch layouts, exact erf GELU); features [r, log(r + h)]
// or in cell units [r/h, log(r/h + 1), log(0.5/h)] (:141-151), then the constant extras; prior
// K = -(1 + K)/sqrt(r^2 + eps^2); split K *= 1 - (1 - min(r/rs, 1)^2)^2.
constexpr int KMLP_H = 64;
constexpr int KMLP_MAXCOL = 8;
struct KmlpArgs {
  int L, ncol, nbase, flags;
  float h, split_r, eps2;
  float extra[KMLP_MAXCOL];
};
__global__ void __launch_bounds__(256) kmlp_lattice_kernel(const float *__restrict__ params, KmlpArgs a,
                                                           float *__restrict__ K) {
  extern __shared__ float sp[];  // W1 (64 x ncol), b1, W2 (64 x 64), b2, W3 (64), b3
  const int np = KMLP_H * a.ncol + KMLP_H + KMLP_H * KMLP_H + KMLP_H + KMLP_H + 1;
  for (int i = threadIdx.x; i < np; i += blockDim.x) sp[i] = params[i];
  __syncthreads();
  const float *W1 = sp, *b1 = W1 + KMLP_H * a.ncol, *W2 = b1 + KMLP_H, *b2 = W2 + KMLP_H * KMLP_H;
  const float *W3 = b2 + KMLP_H, *b3 = W3 + KMLP_H;
  const int L = a.L;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= L * L) return;
  const int iy = e / L, ix = e - iy * L;
  const float dy = (float)min(iy, L - iy) * a.h, dx = (float)min(ix, L - ix) * a.h;
  const float r = sqrtf(dy * dy + dx * dx);
  float f[KMLP_MAXCOL];
  if (a.flags & 1) {  // cell units
    f[0] = r / a.h;
    f[1] = logf(r / a.h + 1.0f);
    f[2] = logf(0.5f / a.h);
  } else {
    f[0] = r;
    f[1] = logf(r + a.h);
  }
  for (int j = a.nbase; j < a.ncol; ++j) f[j] = a.extra[j - a.nbase];
  float h1[KMLP_H];
#pragma unroll 4
  for (int o = 0; o < KMLP_H; ++o) {
    float t = b1[o];
    for (int j = 0; j < a.ncol; ++j) t += W1[o * a.ncol + j] * f[j];
    h1[o] = 0.5f * t * (1.f + erff(t * 0.70710678118654752440f));
  }
  float out = b3[0];
  for (int o = 0; o < KMLP_H; ++o) {
    float t = b2[o];
#pragma unroll 8
    for (int j = 0; j < KMLP_H; ++j) t += W2[o * KMLP_H + j] * h1[j];
    out += W3[o] * (0.5f * t * (1.f + erff(t * 0.70710678118654752440f)));
  }
  float k = out;
  if (a.flags & 2) k = -(1.f + k) / sqrtf(r * r + a.eps2);
  if (a.flags & 4) {
    const float u = fminf(r / a.split_r, 1.f);
    const float w = 1.f - u * u;
    k *= 1.f - w * w;
  }
  K[e] = k;
}

// ---------------------------------------------------------------------------------
// Pair term of the isolated 2D model (ScatterField.pp_acc, scripts/scatter_field.py:291-300,
// 324-364, 500-521). The reference sorts bodies with mask > 0 into cells of side ppe and takes
// each body's knn nearest among the 3 x 3 cells around it; a pair's weight is exactly zero once
// r / ppe rounds to 1, so the knn nearest within ppe decide the sum. Here the cells are finer
// (side ppe / m, clamped into C x C as in _cell_keys) and a body searches rings of cells outwards
// from its own, skipping every cell that cannot hold a candidate nearer than its current knn-th;
// candidates are ranked by (|d|^2 + 1e-8, index), which fixes the selection and the summation
// order whatever the order of the bodies in memory.
// ---------------------------------------------------------------------------------
struct PairArgs {
  int C, W, knn, ncol, nbase, flags;
  float half_ext, cs, inv_ppe, thr0, eps2, h, slack;
  float extra[KMLP_MAXCOL];
};
constexpr int PAIR_CMAX = 2048;
constexpr int PAIR_KMAX = 32;

__device__ __forceinline__ int pair_cell(float x, const PairArgs &a) {
  const float c = floorf(__fdiv_rn(__fadd_rn(x, a.half_ext), a.cs));
  return (int)fminf(fmaxf(c, 0.f), (float)(a.C - 1));
}

// key (cell, or C*C for mask <= 0) and rank of the body within its cell
__global__ void pair_keys_kernel(const float *__restrict__ pos, const float *__restrict__ mask, int64_t n, PairArgs a,
                                 uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                                 uint32_t *__restrict__ counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t k = (uint32_t)(a.C * a.C);
  if (mask[i] > 0.f) k = (uint32_t)(pair_cell(pos[2 * i + 1], a) * a.C + pair_cell(pos[2 * i], a));
  key[i] = k;
  rank[i] = atomicAdd(&counts[k], 1u);
}

// sorted[slot] = (x, y, 0, index bits); slot = cell start (two-level scan) + rank
__global__ void pair_scatter_kernel(const float *__restrict__ pos, const uint32_t *__restrict__ key,
                                    const uint32_t *__restrict__ rank, int64_t n, const uint32_t *__restrict__ start,
                                    const uint32_t *__restrict__ tile_off, float4 *__restrict__ sorted) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = key[i];
  const uint32_t s = tile_off[k / SCAN_TILE] + start[k] + rank[i];
  sorted[s] = make_float4(pos[2 * i], pos[2 * i + 1], 0.f, __uint_as_float((uint32_t)i));
}

// GELU for the pair MLP, evaluated 128 times per pair: 0.5 x erfc(-x / sqrt 2) with erfc from
// the pair MLP's GELU: gelu_as (erfc after Abramowitz & Stegun 7.1.26, |erf error| <= 1.5e-7)
__device__ __forceinline__ float pair_gelu_as(float x) { return gelu_as(x); }

// lower bound of the distance from coordinate x to cell c's extent along one axis (edge cells
// extend to infinity: they hold the clamped bodies)
__device__ __forceinline__ float pair_gap(float x, int c, const PairArgs &a) {
  float g = 0.f;
  if (c > 0) g = fmaxf(g, ((float)c * a.cs - a.half_ext) - x);
  if (c < a.C - 1) g = fmaxf(g, x - ((float)(c + 1) * a.cs - a.half_ext));
  return fmaxf(g - a.slack, 0.f);
}

// Search: one thread per sorted slot; writes the slot's neighbour list (index, |d|^2 + 1e-8) in
// ascending (|d|^2 + 1e-8, index) order to nb_j / nb_q[slot * KP ..], unused entries j = ~0u.
__global__ void __launch_bounds__(128) pair_search_kernel(const float4 *__restrict__ sorted, int64_t n,
                                                          const uint32_t *__restrict__ start,
                                                          const uint32_t *__restrict__ tile_off, PairArgs a, int KP,
                                                          uint32_t *__restrict__ nb_j, float *__restrict__ nb_q) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float4 me = sorted[t];
  const uint32_t i = __float_as_uint(me.w);
  const uint32_t excl = (uint32_t)a.C * a.C;
  auto begin = [&](uint32_t c) { return tile_off[c / SCAN_TILE] + start[c]; };
  float qk[PAIR_KMAX];
  uint32_t jk[PAIR_KMAX];
  int cnt = 0;
  if ((uint32_t)t < begin(excl)) {
    const float xi = me.x, yi = me.y;
    const int cx = pair_cell(xi, a), cy = pair_cell(yi, a);
    const int K = a.knn;
    float thr = a.thr0;  // candidates at or beyond thr0 have exactly zero weight
    for (int d = 0; d <= a.W; ++d) {
      if (d >= 2) {
        const float lb = fmaxf((float)(d - 1) * a.cs - a.slack, 0.f);
        if (lb * lb > thr) break;
      }
      for (int oy = -d; oy <= d; ++oy) {
        const int yy = cy + oy;
        if (yy < 0 || yy >= a.C) continue;
        const float gy = pair_gap(yi, yy, a);
        if (gy * gy > thr) continue;
        const int step = (d == 0 || oy == -d || oy == d) ? 1 : 2 * d;
        for (int ox = -d; ox <= d; ox += step) {
          const int xx = cx + ox;
          if (xx < 0 || xx >= a.C) continue;
          const float gx = pair_gap(xi, xx, a);
          if (gx * gx + gy * gy > thr) continue;
          const uint32_t c = (uint32_t)(yy * a.C + xx);
          const uint32_t s1 = begin(c + 1);
          for (uint32_t s = begin(c); s < s1; ++s) {
            const float4 v = sorted[s];
            const uint32_t j = __float_as_uint(v.w);
            const float dx = v.x - xi, dy = v.y - yi;
            const float q = dx * dx + dy * dy + 1e-8f;
            if (!(q < thr || (q == thr && cnt == K && j < jk[K - 1])) || j == i) continue;
            int p = cnt < K ? cnt : K - 1;
            while (p > 0 && (qk[p - 1] > q || (qk[p - 1] == q && jk[p - 1] > j))) {
              qk[p] = qk[p - 1];
              jk[p] = jk[p - 1];
              --p;
            }
            qk[p] = q;
            jk[p] = j;
            if (cnt < K) ++cnt;
            if (cnt == K) thr = qk[K - 1];
          }
        }
      }
    }
  }
  for (int q = 0; q < KP; ++q) {
    nb_j[t * KP + q] = q < cnt ? jk[q] : ~0u;
    nb_q[t * KP + q] = q < cnt ? qk[q] : 0.f;
  }
}

// Weights: KP lanes (a power of two) per sorted slot, one neighbour each, reduced over the lanes
// by a fixed butterfly; lane 0 writes the body's acceleration (0 for mask <= 0).
__global__ void __launch_bounds__(128) pair_weight_kernel(const float4 *__restrict__ sorted, const float *__restrict__ pos,
                                                          const float *__restrict__ mass,
                                                          const float *__restrict__ mask, int64_t n, int KP,
                                                          const uint32_t *__restrict__ nb_j,
                                                          const float *__restrict__ nb_q,
                                                          const float *__restrict__ params, PairArgs a,
                                                          float *__restrict__ acc) {
  extern __shared__ __align__(16) float sp[];  // ppmlp: W1 (64 x ncol), b1, W2 (64 x 64), b2, W3 (64), b3
  const bool mlp = params != nullptr;
  if (mlp) {
    const int np = KMLP_H * a.ncol + KMLP_H + KMLP_H * KMLP_H + KMLP_H + KMLP_H + 1;
    for (int e = threadIdx.x; e < np; e += blockDim.x) sp[e] = params[e];
    __syncthreads();
  }
  const int64_t g_id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t t = g_id / KP;  // KP divides 32: a slot's lanes share a warp
  const bool live = t < n;      // every lane stays for the shuffles below
  const uint32_t j = live ? nb_j[g_id] : ~0u;
  float cx = 0.f, cy = 0.f;
  const float4 me = live ? sorted[t] : make_float4(0.f, 0.f, 0.f, 0.f);
  if (j != ~0u) {
    const float r = sqrtf(nb_q[g_id]);
    const float dx = pos[2 * j] - me.x, dy = pos[2 * j + 1] - me.y;
    const float u0 = fminf(r * a.inv_ppe, 1.f), u = u0 * u0;
    const float win = (1.f - u) * (1.f - u);
    float w = 0.f;
    if (mlp && win > 0.f) {
      const float *W1 = sp, *b1 = W1 + KMLP_H * a.ncol, *W2 = b1 + KMLP_H, *b2 = W2 + KMLP_H * KMLP_H;
      const float *W3 = b2 + KMLP_H, *b3 = W3 + KMLP_H;
      float f[KMLP_MAXCOL];
      if (a.flags & 1) {
        f[0] = r / a.h;
        f[1] = logf(r / a.h + 0.1f);
        f[2] = logf(0.5f / a.h);
      } else {
        f[0] = r;
        f[1] = logf(r + 0.05f);
      }
#pragma unroll
      for (int e = 2; e < KMLP_MAXCOL; ++e)
        if (e >= a.nbase) f[e] = e < a.ncol ? a.extra[e - a.nbase] : 0.f;
      float h1[KMLP_H];
#pragma unroll
      for (int o = 0; o < KMLP_H; ++o) {
        float z = b1[o];
#pragma unroll
        for (int e = 0; e < KMLP_MAXCOL; ++e)
          if (e < a.ncol) z += W1[o * a.ncol + e] * f[e];
        h1[o] = pair_gelu_as(z);
      }
      float gsum = b3[0];
#pragma unroll 1
      for (int o = 0; o < KMLP_H; ++o) {
        const float4 *w4 = reinterpret_cast<const float4 *>(W2 + o * KMLP_H);
        float z = b2[o];
#pragma unroll
        for (int e = 0; e < KMLP_H / 4; ++e) {
          const float4 wv = w4[e];
          z += wv.x * h1[4 * e];
          z += wv.y * h1[4 * e + 1];
          z += wv.z * h1[4 * e + 2];
          z += wv.w * h1[4 * e + 3];
        }
        gsum += W3[o] * pair_gelu_as(z);
      }
      w = gsum * win;
    }
    if (a.flags & 2) {
      const float qd = sqrtf(r * r + a.eps2);
      const float q3 = qd * qd * qd;
      const float a_mesh = -4.f * (1.f - u) * r * a.inv_ppe * a.inv_ppe / qd + (1.f - win) * r / q3;
      w += r / q3 - a_mesh;
    }
    w *= mass[j] * mask[j];
    cx = w * dx / r;
    cy = w * dy / r;
  }
  for (int o = KP >> 1; o > 0; o >>= 1) {
    cx += __shfl_xor_sync(0xffffffffu, cx, o);
    cy += __shfl_xor_sync(0xffffffffu, cy, o);
  }
  if (live && (g_id & (KP - 1)) == 0) {
    const uint32_t i = __float_as_uint(me.w);
    acc[2 * (int64_t)i] = cx;
    acc[2 * (int64_t)i + 1] = cy;
  }
}

// Pair weights with the MLP's 64 x 64 layer on the tensor cores. A CTA of 128 threads takes
// tiles of 128 (body, neighbour) rows: each thread builds its row's layer-1 activations h1
// (fp32, exact GELU) and stores them split as h1 = hi + lo, two BF16 numbers; the layer is
// D = hi W2hi^T + hi W2lo^T + lo W2hi^T (tcgen05.mma kind::f16, M = 128, N = 64, K = 64, fp32
// accumulation in TMEM), which keeps about 16 bits of every product (the dropped lo x lo term
// is 2^-16 relative). The epilogue reads its row back with tcgen05.ld and finishes as
// pair_weight_kernel does. Operands are K-major without swizzle: element (row, k) of a
// [rows x 64] operand lives at byte (k / 8) * rows * 16 + row * 16 + (k % 8) * 2.
constexpr int PTC_M = 128, PTC_N = 64, PTC_K = 64;
constexpr uint32_t PTC_WAIT = 1u << 20;
constexpr size_t PTC_A_BYTES = (size_t)PTC_M * PTC_K * 2, PTC_B_BYTES = (size_t)PTC_N * PTC_K * 2;
constexpr size_t PTC_SMEM = 2 * PTC_A_BYTES + 2 * PTC_B_BYTES + sizeof(float) * (4 * KMLP_H + 2 * KMLP_H + 4);

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

__global__ void __launch_bounds__(PTC_M) pair_weight_tc_kernel(const float4 *__restrict__ sorted,
                                                               const float *__restrict__ pos,
                                                               const float *__restrict__ mass,
                                                               const float *__restrict__ mask, int64_t n, int KP,
                                                               const uint32_t *__restrict__ nb_j,
                                                               const float *__restrict__ nb_q,
                                                               const float *__restrict__ params, PairArgs a,
                                                               float *__restrict__ acc, unsigned *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sAhi = smem, *sAlo = smem + PTC_A_BYTES;
  unsigned char *sBhi = smem + 2 * PTC_A_BYTES, *sBlo = sBhi + PTC_B_BYTES;
  // per layer-1 output o: {W1[o][0], W1[o][1], b1[o] + the constant features' terms, 0};
  // per layer-2 output o: {b2[o], W3[o]}; then b3
  float4 *L1 = reinterpret_cast<float4 *>(sBlo + PTC_B_BYTES);
  float2 *L2 = reinterpret_cast<float2 *>(L1 + KMLP_H);
  float *b3 = reinterpret_cast<float *>(L2 + KMLP_H);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ncol = a.ncol;
  {
    const float *gW1 = params, *gb1 = gW1 + KMLP_H * ncol, *gW2 = gb1 + KMLP_H, *gb2 = gW2 + KMLP_H * KMLP_H;
    const float *gW3 = gb2 + KMLP_H, *gb3 = gW3 + KMLP_H;
    // features 0 and 1 depend on r; the rest (log(0.5/h) in cell units, the extras) are constant
    float fc[KMLP_MAXCOL];
#pragma unroll
    for (int e = 0; e < KMLP_MAXCOL; ++e) fc[e] = 0.f;
    if (a.flags & 1) fc[2] = logf(0.5f / a.h);
#pragma unroll
    for (int e = 2; e < KMLP_MAXCOL; ++e)
      if (e >= a.nbase && e < a.ncol) fc[e] = a.extra[e - a.nbase];
    for (int o = tid; o < KMLP_H; o += PTC_M) {
      float bc = gb1[o];
      for (int e = 2; e < ncol; ++e) bc += gW1[o * ncol + e] * fc[e];
      L1[o] = make_float4(gW1[o * ncol], gW1[o * ncol + 1], bc, 0.f);
      L2[o] = make_float2(gb2[o], gW3[o]);
    }
    if (tid == 0) b3[0] = gb3[0];
    // B = W2 (n = output, k = input; torch's [out][in] is already K-major), split hi + lo
    for (int e = tid; e < PTC_N * PTC_K / 2; e += PTC_M) {
      const int nn = e / (PTC_K / 2), k = 2 * (e % (PTC_K / 2));
      const float w0 = gW2[nn * PTC_K + k], w1 = gW2[nn * PTC_K + k + 1];
      const __nv_bfloat16 h0 = __float2bfloat16_rn(w0), h1 = __float2bfloat16_rn(w1);
      const __nv_bfloat16 l0 = __float2bfloat16_rn(w0 - __bfloat162float(h0));
      const __nv_bfloat16 l1 = __float2bfloat16_rn(w1 - __bfloat162float(h1));
      const size_t off = (size_t)(k / 8) * PTC_N * 16 + (size_t)nn * 16 + (k % 8) * 2;
      *reinterpret_cast<uint32_t *>(sBhi + off) = bf16x2_bits(h0, h1);
      *reinterpret_cast<uint32_t *>(sBlo + off) = bf16x2_bits(l0, l1);
    }
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_abort = 0;
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, PTC_N);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = idesc_bf16_f32(PTC_M, PTC_N);
  const uint64_t adh = smem_desc(smem_u32(sAhi), PTC_M * 16, 128), adl = smem_desc(smem_u32(sAlo), PTC_M * 16, 128);
  const uint64_t bdh = smem_desc(smem_u32(sBhi), PTC_N * 16, 128), bdl = smem_desc(smem_u32(sBlo), PTC_N * 16, 128);
  const int64_t rows = n * KP, ntiles = (rows + PTC_M - 1) / PTC_M;
  uint32_t phase = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t g_id = tile * PTC_M + tid;
    const int64_t t = g_id / KP;
    const bool live = g_id < rows;
    const uint32_t j = live ? nb_j[g_id] : ~0u;
    const float4 me = live ? sorted[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    float r = 1.f, u = 1.f, win = 0.f, dx = 0.f, dy = 0.f;
    if (j != ~0u) {
      r = sqrtf(nb_q[g_id]);
      dx = pos[2 * j] - me.x;
      dy = pos[2 * j + 1] - me.y;
      const float u0 = fminf(r * a.inv_ppe, 1.f);
      u = u0 * u0;
      win = (1.f - u) * (1.f - u);
    }
    // layer 1 + GELU for this row, split into hi / lo BF16 rows of A (zero for empty rows)
    {
      const float f0 = (a.flags & 1) ? r / a.h : r;
      const float f1 = (a.flags & 1) ? logf(r / a.h + 0.1f) : logf(r + 0.05f);
      const bool use = j != ~0u && win > 0.f;
#pragma unroll
      for (int kb = 0; kb < PTC_K / 8; ++kb) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) {
          float hv[2];
#pragma unroll
          for (int s2 = 0; s2 < 2; ++s2) {
            const float4 l1 = L1[kb * 8 + q2 * 2 + s2];
            const float z = fmaf(l1.y, f1, fmaf(l1.x, f0, l1.z));
            hv[s2] = use ? pair_gelu_as(z) : 0.f;
          }
          const __nv_bfloat16 h0 = __float2bfloat16_rn(hv[0]), h1 = __float2bfloat16_rn(hv[1]);
          hi[q2] = bf16x2_bits(h0, h1);
          lo[q2] = bf16x2_bits(__float2bfloat16_rn(hv[0] - __bfloat162float(h0)),
                               __float2bfloat16_rn(hv[1] - __bfloat162float(h1)));
        }
        const size_t off = (size_t)kb * PTC_M * 16 + (size_t)tid * 16;
        *reinterpret_cast<uint4 *>(sAhi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4 *>(sAlo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    fence_async_smem();  // generic-proxy stores -> visible to the tensor core
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint64_t ad[3] = {adh, adh, adl}, bd[3] = {bdh, bdl, bdh};
#pragma unroll
      for (int pss = 0; pss < 3; ++pss)
#pragma unroll
        for (int kc = 0; kc < PTC_K / 16; ++kc)
          umma_bf16(tmem, ad[pss] + (uint64_t)((2 * kc * PTC_M * 16) >> 4),
                    bd[pss] + (uint64_t)((2 * kc * PTC_N * 16) >> 4), idesc, (pss | kc) ? 1u : 0u);
      umma_commit(&bar);
    }
    bool ok = false;
    for (uint32_t i = 0; i < PTC_WAIT && !ok; ++i) ok = mbar_try_wait(&bar, phase);
    phase ^= 1u;
    if (!ok) s_abort = 1;
    tc_fence_after();
    // layer 2's bias and GELU, then layer 3, 32 TMEM columns at a time (whole warps load)
    float g = b3[0];
#pragma unroll
    for (int hh = 0; hh < PTC_N / 32; ++hh) {
      float d[32];
      tmem_ld32(tmem + (uint32_t)(32 * hh) + ((uint32_t)(warp * 32) << 16), d);
#pragma unroll
      for (int o = 0; o < 32; ++o) {
        const float2 l2 = L2[32 * hh + o];
        g = fmaf(l2.y, pair_gelu_as(d[o] + l2.x), g);
      }
    }
    float cx = 0.f, cy = 0.f;
    if (j != ~0u) {
      float w = 0.f;
      if (win > 0.f) w = g * win;
      if (a.flags & 2) {
        const float qd = sqrtf(r * r + a.eps2);
        const float q3 = qd * qd * qd;
        const float a_mesh = -4.f * (1.f - u) * r * a.inv_ppe * a.inv_ppe / qd + (1.f - win) * r / q3;
        w += r / q3 - a_mesh;
      }
      w *= mass[j] * mask[j];
      cx = w * dx / r;
      cy = w * dy / r;
    }
    for (int o = KP >> 1; o > 0; o >>= 1) {
      cx += __shfl_xor_sync(0xffffffffu, cx, o);
      cy += __shfl_xor_sync(0xffffffffu, cy, o);
    }
    if (live && (g_id & (KP - 1)) == 0) {
      const uint32_t i = __float_as_uint(me.w);
      acc[2 * (int64_t)i] = cx;
      acc[2 * (int64_t)i + 1] = cy;
    }
    tc_fence_before();
    __syncthreads();  // TMEM and the A rows are reused by the next tile
    if (s_abort) break;
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_abort) atomicOr(err, AUGUR_ERRBIT_TIMEOUT);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, PTC_N);
  }
  (void)lane;
}

// ---------------------------------------------------------------------------------
// K3b: z transform + Green's function + spectral gradient + inverse z transform, for
// one kx plane and a strip of TY ky columns, all z. spec is [kx][z][ky] (after the
// forward y transform). Writes ncomp outputs out[c][kx][z][ky]: the three components of
// a_k = -i k phi_k (Nyquist of the differentiated axis -> 0) and, if ncomp == 4, phi_k.
// phi_k = -4 pi G rho_k / k^2 (k = 0 -> 0) with the 1/G^3 of the inverse transform folded in.
// ---------------------------------------------------------------------------------
struct GreenArgs {
  int G, TY, ncomp, Lt;
  int nbuf;        // transform scratch buffers: 1 for two-stage lengths (the stages meet in one), else 2
  FftShape fsh;    // length G
  float kfund;     // 2 pi / box
  float gfac;      // -4 pi G_newton / G^3
};

template <int TY>
__device__ __forceinline__ void fft_z_green_kernel_body(const float2 *__restrict__ spec, GreenArgs a,
                                                          const float2 *__restrict__ twg,
                                                          float2 *__restrict__ out, const int bx) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = a.G, M = G / 2;
  const int nyt = G / TY;
  const int kx = bx / nyt;
  const int y0 = (bx % nyt) * TY;
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t plane = (size_t)G * G;
  const size_t cstride = (size_t)(M + 1) * plane;
  float2 *P = reinterpret_cast<float2 *>(smem);
  float2 *B = P + (size_t)G * TY;
  float2 *C = B + (size_t)(a.nbuf - 1) * G * TY;
  float2 *tw = C + (size_t)G * TY;
  for (int e = tid; e < a.Lt; e += nt) tw[e] = twg[e];
  __syncthreads();
  const float2 *src = spec + (size_t)kx * plane + y0;
  const float mx = (float)kx;
  // forward z transform from HBM; the last stage applies the Green's function on its way to P
  {
    auto ld = [&](int b, int e) -> float2 { return src[(size_t)e * G + b]; };
    auto st = [&](int b, int e, float2 v) {
      const int ky = y0 + b;
      const float my = (float)(ky < M ? ky : ky - G);
      const float mz = (float)(e < M ? e : e - G);
      const float m2 = mx * mx + my * my + mz * mz;
      const float f = (m2 > 0.f) ? a.gfac / (a.kfund * a.kfund * m2) : 0.f;
      P[e * TY + b] = make_float2(v.x * f, v.y * f);
    };
    AUGUR_FFT_IO(G, TY, TY, ld, st, B, C, 0, tw, 1, false);
  }
  for (int c = 0; c < a.ncomp; ++c) {
    float2 *dst = out + c * cstride + (size_t)kx * plane + y0;
    // inverse z transform of -i k_c phi_k (or phi_k for c == 3), the derivative applied on load
    auto ld = [&](int b, int e) -> float2 {
      const float2 ph = P[e * TY + b];
      if (c == 3) return ph;
      const int idx = (c == 0) ? kx : (c == 1 ? y0 + b : e);
      float m;
      if (c == 0) m = (idx == M) ? 0.f : (float)idx;
      else m = (idx == M) ? 0.f : (float)(idx < M ? idx : idx - G);
      const float k = a.kfund * m;
      return make_float2(k * ph.y, -k * ph.x);  // -i k phi
    };
    auto st = [&](int b, int e, float2 v) { dst[(size_t)e * G + b] = v; };
    AUGUR_FFT_IO(G, TY, TY, ld, st, B, C, 0, tw, 1, true);
  }
}

// Threads of fft_z_green_kernel: one per (column, butterfly) of a radix-16 stage, at least 16 TY,
// at most 512 (256 at G = 128 and 256: 101 -> 92 us at 256^3 against 512; 512 for longer columns,
// whose stages have more butterflies: 8.0 ms at 1024^3 against 12.6 with 256)
__host__ __device__ inline int green_threads(int G, int TY) {
  const int t = TY * G / 16;
  return t < 16 * TY ? 16 * TY : (t > 512 ? 512 : t);
}

template <int TY>
__global__ void __launch_bounds__(512) fft_z_green_kernel(const float2 *__restrict__ spec, GreenArgs a,
                                                          const float2 *__restrict__ twg,
                                                          float2 *__restrict__ out) {
  fft_z_green_kernel_body<TY>(spec, a, twg, out, (int)blockIdx.x);
}

// 2D isolated: pointwise product with the kernel spectrum (complex), spec[kx][ky].
__global__ void kmul_kernel(float2 *__restrict__ spec, const float2 *__restrict__ khat, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) spec[i] = cmul(spec[i], khat[i]);
}

// ---------------------------------------------------------------------------------
// K3c: C2R along x. in[c][kx][r] (kx = 0..L/2, r < nrows). Each block transforms RB rows
// of every component. OUT4: writes F4[r][x] = (c0, c1, c2, c3 or 0) for x < L.
// Otherwise writes component 0 as real rows out[r][x] for r < nkeep, x < Lkeep (times scale).
// ---------------------------------------------------------------------------------
// The C2R input block X: for M <= 128 (a warp's first-stage lanes span several rows) stored
// [kx][row] with RB + 2 float2 per kx, so consecutive rows of one kx land on consecutive banks for
// the copies and the first stage's reads of X_k and X_{M-k} spread over the banks; for longer rows
// (a warp within one row) stored [row][kx] with rows of fft_row_stride(M), loaded through
// registers (the kx-major form with cp.async measured 17.3 ms at 1024^3 against 15.4). For
// transforms of three or more stages X is also the second scratch buffer, rows of
// fft_row_stride(M).
__host__ __device__ inline int c2r_x_elems(int M, int RB) {
  const int a = (M + 1) * (RB + 2), b = RB * fft_row_stride(M);
  return a > b ? a : b;
}
// Shared memory of c2r_rows_kernel: nbx input blocks, the scratch rows, nres result planes, twiddles.
__host__ __device__ inline size_t c2r_smem_bytes(int M, int RB, int L, int nres, int nbx, int Lt) {
  return ((size_t)nbx * c2r_x_elems(M, RB) + (size_t)RB * fft_row_stride(M)) * 8 + (size_t)nres * RB * L * 4 +
         (size_t)Lt * 8;
}
struct C2RArgs {
  int L, nrows, RB, ncomp, Lt;
  int nkeep, Lkeep;
  float scale;
  FftShape fsh;  // complex length L/2
  int twmul;
  FastDiv fdRB, fdM, fdL;
  int ext;  // single component: keep rows/columns 0..Lkeep and L-1 into a (Lkeep+2)^2 array, index +1 (L-1 -> 0)
  int nbx;  // input blocks: 2 = the next component is copied in while this one is transformed (0 or 1: one)
};

// KXM (M <= 128): input block [kx][row], the next component copied in with cp.async during this
// one's transform (two blocks when a.nbx == 2). Otherwise: rows [row][kx] loaded through
// registers, C2R_LU loads per thread in flight, one block.
constexpr int C2R_LU = 5;
template <bool OUT4, bool KXM>
__device__ __forceinline__ void c2r_rows_kernel_body(const float2 *__restrict__ in, C2RArgs a,
                                                       const float2 *__restrict__ twg, float *__restrict__ out, const int bx) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int L = a.L, M = L / 2, RB = a.RB;
  const int MS = fft_row_stride(M);  // scratch row stride
  const int XP = RB + 2;             // X[kx * XP + row] (KXM) or X[row * MS + kx]
  auto xi = [&](int kx, int rr) { return KXM ? kx * XP + rr : rr * MS + kx; };
  const int XE = c2r_x_elems(M, RB);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int r0 = bx * RB;
  const int nc = OUT4 ? a.ncomp : 1;
  const int nbx = (KXM && a.nbx == 2 && nc > 1) ? 2 : 1;
  float2 *X0 = reinterpret_cast<float2 *>(smem);
  float2 *Y = X0 + (size_t)nbx * XE;
  float *res = reinterpret_cast<float *>(Y + (size_t)RB * MS);  // [nc][RB][L]
  float2 *tw = reinterpret_cast<float2 *>(res + (size_t)nc * RB * L);
  for (int e = tid; e < a.Lt; e += nt) tw[e] = twg[e];
  const size_t cstride = (size_t)(M + 1) * a.nrows;
  const int tstep = a.Lt / L;
  auto xbuf = [&](int c) { return X0 + (size_t)(nbx == 2 ? (c & 1) : 0) * XE; };
  // component c into its input block by asynchronous 8-byte copies (rows past nrows read as zero);
  // the reads, 128-byte row pieces spread over M + 1 kx planes, are latency-bound, so with two
  // blocks the next component's copies run during this one's transform
  auto issue = [&](int c) {
    const float2 *src = in + c * cstride;
    float2 *Xb = xbuf(c);
    for (int e = tid; e < (M + 1) * RB; e += nt) {
      const int kx = (int)fdiv(e, a.fdRB), rr = e - kx * RB;
      const bool inr = r0 + rr < a.nrows;
      cp_async8(smem_u32(&Xb[xi(kx, rr)]), inr ? &src[(size_t)kx * a.nrows + r0 + rr] : src, inr ? 8u : 0u);
    }
    cp_async_commit();
  };
  // component c through registers (C2R_LU loads per thread in flight before any is stored)
  auto load_regs = [&](int c) {
    const float2 *src = in + c * cstride;
    for (int e0 = tid; e0 < (M + 1) * RB; e0 += nt * C2R_LU) {
      float2 v[C2R_LU];
#pragma unroll
      for (int u = 0; u < C2R_LU; ++u) {
        const int e = e0 + u * nt;
        v[u] = make_float2(0.f, 0.f);
        if (e < (M + 1) * RB) {
          const int kx = (int)fdiv(e, a.fdRB), rr = e - kx * RB;
          if (r0 + rr < a.nrows) v[u] = __ldcs(&src[(size_t)kx * a.nrows + r0 + rr]);
        }
      }
#pragma unroll
      for (int u = 0; u < C2R_LU; ++u) {
        const int e = e0 + u * nt;
        if (e < (M + 1) * RB) {
          const int kx = (int)fdiv(e, a.fdRB), rr = e - kx * RB;
          X0[xi(kx, rr)] = v[u];
        }
      }
    }
  };
  if (KXM) issue(0);
  for (int c = 0; c < nc; ++c) {
    if (KXM) {
      if (nbx == 2 && c + 1 < nc) {
        issue(c + 1);  // its block was last read by the transform of component c - 1
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
    } else {
      load_regs(c);
    }
    __syncthreads();
    const float2 *X = xbuf(c);
    // inverse transform whose first stage computes the pre-process on load:
    // E_k = X_k + conj X_{M-k} ; O_k = (X_k - conj X_{M-k}) W^{-k} ; Z_k = E_k + i O_k
    // (the imaginary parts of X_0 and X_M, DC and Nyquist, are ignored)
    float *dst = res + (size_t)c * RB * L;
    auto ld = [&](int b, int k) -> float2 {
      float2 xk = X[xi(k, b)];
      float2 xc = cconj(X[xi(M - k, b)]);
      if (k == 0) {
        xk.y = 0.f;
        xc.y = 0.f;
      }
      float2 E = cadd(xk, xc);
      float2 O = cmul(csub(xk, xc), cconj(tw[k * tstep]));
      return make_float2(E.x - O.y, E.y + O.x);
    };
    auto st = [&](int b, int k, float2 v) {
      *reinterpret_cast<float2 *>(&dst[b * L + 2 * k]) = make_float2(v.x * a.scale, v.y * a.scale);
    };
    // (three-stage lengths use the input block as their second scratch buffer)
    AUGUR_FFT_IO(M, 0, RB, ld, st, const_cast<float2 *>(X), Y, MS, tw, a.twmul, true);
    if (KXM && nbx == 1 && c + 1 < nc) issue(c + 1);
  }
  if (OUT4) {
    float4 *o4 = reinterpret_cast<float4 *>(out);
    for (int e = tid; e < RB * L; e += nt) {
      int rr = (int)fdiv(e, a.fdL), x = e - rr * L;
      int r = r0 + rr;
      if (r >= a.nrows) continue;
      float4 v;
      v.x = res[(size_t)0 * RB * L + rr * L + x];
      v.y = res[(size_t)1 * RB * L + rr * L + x];
      v.z = (a.ncomp > 2) ? res[(size_t)2 * RB * L + rr * L + x] : 0.f;
      v.w = (a.ncomp > 3) ? res[(size_t)3 * RB * L + rr * L + x] : 0.f;
      o4[(size_t)r * L + x] = v;
    }
  } else if (a.ext) {
    // rows and columns -1 .. Lkeep of the zero-padded transform (index -1 is L - 1)
    const int W = a.Lkeep + 2;
    for (int e = tid; e < RB * L; e += nt) {
      int rr = (int)fdiv(e, a.fdL), x = e - rr * L;
      int r = r0 + rr;
      if (r >= a.nrows) continue;
      const int er = (r == L - 1) ? 0 : r + 1, ex = (x == L - 1) ? 0 : x + 1;
      if (er > a.Lkeep + 1 || ex > a.Lkeep + 1) continue;
      out[(size_t)er * W + ex] = res[rr * L + x];
    }
  } else {
    for (int e = tid; e < RB * L; e += nt) {
      int rr = (int)fdiv(e, a.fdL), x = e - rr * L;
      int r = r0 + rr;
      if (r >= a.nkeep || x >= a.Lkeep) continue;
      out[(size_t)r * a.Lkeep + x] = res[rr * L + x];
    }
  }
}

template <bool OUT4>
__global__ void __launch_bounds__(512, 2) c2r_rows_kernel(const float2 *__restrict__ in, C2RArgs a,
                                                       const float2 *__restrict__ twg, float *__restrict__ out) {
  if (a.L <= 256)
    c2r_rows_kernel_body<OUT4, true>(in, a, twg, out, (int)blockIdx.x);
  else
    c2r_rows_kernel_body<OUT4, false>(in, a, twg, out, (int)blockIdx.x);
}

// 2D isolated: F4 grid from the potential by the reference's zero-padded central
// difference (scripts/scatter_field.py:551-555): a_x = -((phi[y][x+1] - phi[y][x-1]) / (2h)).
__global__ void fd_grad2d_kernel(const float *__restrict__ phi, int G, float two_h, float4 *__restrict__ F4) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G * G) return;
  int y = e / G, x = e - y * G;
  float xp = (x + 1 < G) ? phi[e + 1] : 0.f, xm = (x > 0) ? phi[e - 1] : 0.f;
  float yp = (y + 1 < G) ? phi[e + G] : 0.f, ym = (y > 0) ? phi[e - G] : 0.f;
  float gx = __fdiv_rn(__fsub_rn(xp, xm), two_h);
  float gy = __fdiv_rn(__fsub_rn(yp, ym), two_h);
  F4[e] = make_float4(-gx, -gy, 0.f, phi[e]);
}

// 2D isolated: kernel lattice K = -1/sqrt(d_y^2 + d_x^2 + eps^2) on the 2G min-image
// lattice (scripts/pm_baseline_force_error.py:70-73), fp32.
__global__ void kernel_lattice_kernel(float *__restrict__ K, int G2, float h, float eps2) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G2 * G2) return;
  int y = e / G2, x = e - y * G2;
  float dy = __fmul_rn((float)min(y, G2 - y), h), dx = __fmul_rn((float)min(x, G2 - x), h);
  float s = __fadd_rn(__fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dx, dx)), eps2);
  K[e] = __fdiv_rn(-1.0f, __fsqrt_rn(s));
}

// ---------------------------------------------------------------------------------
// K4: CIC gather of F4 at the sorted bodies, fused with the integrator.
//   MODE_FORCE : acc4s[i] = (a * mask, phi * mask) in sorted order (float4, coalesced); the
//                caller's arrays are written by accel_to_caller_kernel
//   MODE_KD    : v += kick * a ; if drift: x += dt * v, wrap, new row key + slot (run loop)
// Corner order and fp32 operation order follow ScatterField.gather (:252-261).
// ---------------------------------------------------------------------------------
enum { MODE_FORCE = 0, MODE_KD = 1 };

struct GatherArgs {
  GridParams g;
  float kick, dt;
  int drift;
  float esync;    // energy tap: kinetic energy at v + esync * a (the synchronised velocity)
  double *epart;  // energy tap: per-block (kinetic, potential) partial sums, or null
};

template <int D, int MODE>
__device__ __forceinline__ void gather_kernel_body(const float4 *__restrict__ F4, float4 *__restrict__ pos4,
                                                     float4 *__restrict__ vel4, int64_t n, GatherArgs a,
                                                     float *__restrict__ acc_out, float *__restrict__ phi_out,
                                                     float *__restrict__ vel_out, uint32_t *__restrict__ key,
                                                     uint32_t *__restrict__ slot, uint32_t *__restrict__ row_count,
                                                     unsigned *__restrict__ err, const int bx) {
  const GridParams &g = a.g;
  const int G = g.G;
  const int64_t i = (int64_t)bx * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f), v = p;
  if (valid) {
    p = pos4[i];
    v = vel4[i];
  }
  int ix = 0, iy = 0, iz = 0;
  float wx = 0.f, wy = 0.f, wz = 0.f;
  bool ok = cic_axis(p.x, g.half_ext, g.h, ix, wx, g.inv_h) & cic_axis(p.y, g.half_ext, g.h, iy, wy, g.inv_h);
  if (D == 3) ok &= cic_axis(p.z, g.half_ext, g.h, iz, wz, g.inv_h);
  if (valid && !ok) set_err(err, AUGUR_ERRBIT_NONFINITE);
  float ax = 0.f, ay = 0.f, az = 0.f, ph = 0.f;
  if (valid && ok) {
    int cxs[2], cys[2], czs[2] = {0, 0};
    bool inx[2] = {true, true}, iny[2] = {true, true};
    if (g.periodic) {
      cxs[0] = fwrap(ix, G);
      cxs[1] = cxs[0] + 1 == G ? 0 : cxs[0] + 1;
      cys[0] = fwrap(iy, G);
      cys[1] = cys[0] + 1 == G ? 0 : cys[0] + 1;
      if (D == 3) {
        czs[0] = fwrap(iz, G);
        czs[1] = czs[0] + 1 == G ? 0 : czs[0] + 1;
      }
    } else {
#pragma unroll
      for (int o = 0; o < 2; ++o) {
        inx[o] = (ix + o >= 0) && (ix + o < G);
        iny[o] = (iy + o >= 0) && (iy + o < G);
        cxs[o] = min(max(ix + o, 0), G - 1);
        cys[o] = min(max(iy + o, 0), G - 1);
      }
    }
#pragma unroll
    for (int ox = 0; ox < 2; ++ox) {
#pragma unroll
      for (int oy = 0; oy < 2; ++oy) {
#pragma unroll
        for (int oz = 0; oz < (D == 3 ? 2 : 1); ++oz) {
          float wt = __fmul_rn(axis_w(wx, ox), axis_w(wy, oy));
          if (D == 3) wt = __fmul_rn(wt, axis_w(wz, oz));
          if (!(inx[ox] && iny[oy])) wt = 0.f;
          size_t cell = (D == 3) ? ((size_t)czs[oz] * G + cys[oy]) * G + cxs[ox] : (size_t)cys[oy] * G + cxs[ox];
          float4 f = __ldg(&F4[cell]);
          ax = __fadd_rn(ax, __fmul_rn(f.x, wt));
          ay = __fadd_rn(ay, __fmul_rn(f.y, wt));
          if (D == 3) az = __fadd_rn(az, __fmul_rn(f.z, wt));
          ph = __fadd_rn(ph, __fmul_rn(f.w, wt));
        }
      }
    }
  }
  const uint32_t idw = __float_as_uint(v.w);
  const uint32_t id = idw & 0x7fffffffu;
  const float mk = (idw & 0x80000000u) ? 0.f : 1.f;
  if (MODE == MODE_FORCE) {
    if (valid)
      reinterpret_cast<float4 *>(acc_out)[i] =
          make_float4(__fmul_rn(ax, mk), __fmul_rn(ay, mk), __fmul_rn(az, mk), __fmul_rn(ph, mk));
  } else {  // MODE_KD on the sorted state
    uint32_t k = 0;
    if (valid) {
      ax = __fmul_rn(ax, mk);
      ay = __fmul_rn(ay, mk);
      az = __fmul_rn(az, mk);
    }
    if (a.epart) {  // energy at the synchronised time (uniform branch: every thread takes part)
      double ek = 0.0, ep = 0.0;
      if (valid) {
        const float vx = v.x + a.esync * ax, vy = v.y + a.esync * ay, vz = v.z + a.esync * az;
        ek = 0.5 * (double)p.w * (double)(vx * vx + vy * vy + vz * vz);
        ep = 0.5 * (double)p.w * (double)(ph * mk);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ek += __shfl_xor_sync(0xffffffffu, ek, o);
        ep += __shfl_xor_sync(0xffffffffu, ep, o);
      }
      __shared__ double sred[2][8];
      const int w = threadIdx.x >> 5;
      if ((threadIdx.x & 31) == 0) {
        sred[0][w] = ek;
        sred[1][w] = ep;
      }
      __syncthreads();
      if (threadIdx.x < 2) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sred[threadIdx.x][q];
        a.epart[(size_t)bx * 2 + threadIdx.x] = t;
      }
    }
    if (valid) {
      v.x = __fadd_rn(v.x, __fmul_rn(a.kick, ax));
      v.y = __fadd_rn(v.y, __fmul_rn(a.kick, ay));
      if (D == 3) v.z = __fadd_rn(v.z, __fmul_rn(a.kick, az));
      if (a.drift) {
        float xs[3] = {p.x, p.y, p.z};
        const float vs[3] = {v.x, v.y, v.z};
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float t = __fadd_rn(xs[d], __fmul_rn(a.dt, vs[d]));
          if (t >= g.half_ext) t = __fsub_rn(t, g.ext);
          else if (t < -g.half_ext) t = __fadd_rn(t, g.ext);
          xs[d] = t;
        }
        p.x = xs[0];
        p.y = xs[1];
        p.z = xs[2];
        int jx = 0, jy = 0, jz = 0;
        float u;
        bool ok2 = cic_axis(p.x, g.half_ext, g.h, jx, u, g.inv_h) & cic_axis(p.y, g.half_ext, g.h, jy, u, g.inv_h);
        if (D == 3) ok2 &= cic_axis(p.z, g.half_ext, g.h, jz, u, g.inv_h);
        if (!ok2) set_err(err, AUGUR_ERRBIT_NONFINITE);
        k = row_key(g, jx, jy, jz);
      }
      pos4[i] = p;
      vel4[i] = v;
      if (acc_out) {
        acc_out[(size_t)id * D] = ax;
        acc_out[(size_t)id * D + 1] = ay;
        if (D == 3) acc_out[(size_t)id * D + 2] = az;
      }
    }
    if (a.drift) {
      uint32_t s = warp_slot(row_count, k, valid);
      if (valid) {
        key[i] = k;
        slot[i] = s;
      }
    }
  }
}

// six CTAs per SM (40 registers): the corner loads are latency-bound, and more resident warps hide
// them (80 -> 74 us at 3M bodies against five CTAs at 48 registers; eight spilled and ran 86 us)
template <int D, int MODE>
__global__ void __launch_bounds__(256, 6) gather_kernel(const float4 *__restrict__ F4, float4 *__restrict__ pos4,
                                                     float4 *__restrict__ vel4, int64_t n, GatherArgs a,
                                                     float *__restrict__ acc_out, float *__restrict__ phi_out,
                                                     float *__restrict__ vel_out, uint32_t *__restrict__ key,
                                                     uint32_t *__restrict__ slot, uint32_t *__restrict__ row_count,
                                                     unsigned *__restrict__ err) {
  gather_kernel_body<D, MODE>(F4, pos4, vel4, n, a, acc_out, phi_out, vel_out, key, slot, row_count, err, (int)blockIdx.x);
}

// Caller-order pass after a MODE_FORCE gather. Body j of the caller's arrays sits at sorted slot
// row_begin(key[j]) + slot[j] (where scatter_aos put it), so its acceleration is read there (the
// sorted float4s and the row starts stay in L2) while the caller's arrays are read and written in
// their own order, coalesced, instead of one scattered read-modify-write per body.
//   VV = false: acc[j] = a ; phi[j] = phi (when given)
//   VV = true : velocity-Verlet kick vel[j] += kick * (acc[j] + a) ; acc[j] = a
//               (scripts/scatter_field.py:686-688)
template <int D, bool VV>
__global__ void __launch_bounds__(256) accel_to_caller_kernel(const float4 *__restrict__ acc4s, int64_t n,
                                                              const uint32_t *__restrict__ key,
                                                              const uint32_t *__restrict__ slot,
                                                              const uint32_t *__restrict__ start,
                                                              const uint32_t *__restrict__ tile_off, float kick,
                                                              float *__restrict__ acc, float *__restrict__ phi,
                                                              float *__restrict__ vel) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float4 a = acc4s[row_begin(start, tile_off, key[j]) + slot[j]];
  const float an[3] = {a.x, a.y, a.z};
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (VV) {
      const float dv = __fmul_rn(kick, __fadd_rn(acc[(size_t)j * D + d], an[d]));
      vel[(size_t)j * D + d] = __fadd_rn(vel[(size_t)j * D + d], dv);
    }
    acc[(size_t)j * D + d] = an[d];
  }
  if (phi) phi[j] = a.w;
}

// Fixed-order sum of the gather's per-block energy partials: out[0] kinetic, out[1] potential.
// Fixed-order fold of the per-block energy partials: thread t sums a contiguous chunk
// (compensated), then a shared-memory tree in a fixed pattern -- deterministic, and parallel
// (a serial FP64 chain over ~10^4 partials takes milliseconds on this part).
constexpr int FOLD_THREADS = 1024;
__global__ void __launch_bounds__(FOLD_THREADS) energy_fold_kernel(const double *__restrict__ epart, int nblk,
                                                                   double *__restrict__ out) {
  __shared__ double sh[2][FOLD_THREADS];
  const int t = threadIdx.x;
  const int per = (nblk + FOLD_THREADS - 1) / FOLD_THREADS;
  const int b0 = min(nblk, t * per), b1 = min(nblk, b0 + per);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    double s = 0.0, c = 0.0;
    for (int b = b0; b < b1; ++b) {
      const double v = epart[(size_t)b * 2 + q];
      const double u = s + v;
      c += (fabs(s) >= fabs(v)) ? (s - u) + v : (v - u) + s;
      s = u;
    }
    sh[q][t] = s + c;
  }
  __syncthreads();
  for (int w = FOLD_THREADS / 2; w > 0; w >>= 1) {
    if (t < w) {
      sh[0][t] += sh[0][t + w];
      sh[1][t] += sh[1][t + w];
    }
    __syncthreads();
  }
  if (t < 2) out[t] = sh[t][0];
}

// Write the sorted state back to the caller's order (end of a run).
template <int D>
__global__ void unsort_kernel(const float4 *__restrict__ pos4, const float4 *__restrict__ vel4, int64_t n,
                              float *__restrict__ pos, float *__restrict__ vel) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pos4[i], v = vel4[i];
  uint32_t id = __float_as_uint(v.w) & 0x7fffffffu;
  pos[(size_t)id * D] = p.x;
  pos[(size_t)id * D + 1] = p.y;
  vel[(size_t)id * D] = v.x;
  vel[(size_t)id * D + 1] = v.y;
  if (D == 3) {
    pos[(size_t)id * D + 2] = p.z;
    vel[(size_t)id * D + 2] = v.z;
  }
}

// Cell index output (bit-exact with ScatterField._corners).
template <int D>
__global__ void cell_index_kernel(const float *__restrict__ pos, int64_t n, GridParams g, int32_t *__restrict__ i0,
                                  float *__restrict__ w, unsigned *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    int c;
    float f;
    if (!cic_axis(pos[i * D + d], g.half_ext, g.h, c, f, g.inv_h)) set_err(err, AUGUR_ERRBIT_NONFINITE);
    i0[i * D + d] = c;
    w[i * D + d] = f;
  }
}

// ---------------------------------------------------------------------------------
// Multi-scene launches: one grid covers the blocks of every scene of a batch for one stage of
// the run loop. Scene s owns blocks [boff[s], boff[s+1]) of the grid; its block runs the
// single-scene kernel body with the scene's arguments (a pack in device memory) and its local
// block index, so every scene computes exactly what its own launch would.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int scene_of(const int *__restrict__ boff, int ns, int b) {
  int lo = 0, hi = ns;  // boff[lo] <= b < boff[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&boff[mid]) <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

struct ScanPack {
  uint32_t *count, *start, *tile_sum, *tile_off;
  int nrow, ntiles;
};
struct ScatterPack {
  const float4 *pos_in, *vel_in;
  int64_t n;
  const uint32_t *key, *slot, *start, *tile_off;
  float4 *pos_out, *vel_out;
};
struct DepPlanPack {
  const uint32_t *start, *tile_off;
  DepositArgs a;
  uint32_t *nch, *item_off, *slot_off, *item_blk;
  uint4 *seg_tab;
  unsigned *err;
};
struct DepPack {
  const float4 *pos4;
  const unsigned *mmax;
  DepositArgs a;
  const float2 *tw;
  float2 *spec;
  unsigned *err;
  const uint32_t *item_off, *slot_off, *item_blk;
  const uint4 *seg_tab;
  unsigned long long *scratch;
  unsigned *counters;
};
struct RowsPack {
  float2 *data;
  int64_t nrows;
  int RB, L, twmul, Lt, inverse;
  FastDiv fdL;
  const float2 *tw;
};
struct GreenPack {
  const float2 *spec;
  GreenArgs a;
  const float2 *tw;
  float2 *out;
};
struct C2RPack {
  const float2 *in;
  C2RArgs a;
  const float2 *tw;
  float *out;
};
struct GatherPack {
  const float4 *F4;
  float4 *pos4, *vel4;
  int64_t n;
  GatherArgs a;
  uint32_t *key, *slot, *row_count;
  unsigned *err;
};

__global__ void __launch_bounds__(1024) scan_local_multi(const ScanPack *__restrict__ pk, const int *__restrict__ boff,
                                                         int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const ScanPack q = pk[s];
  scan_local_kernel_body(q.count, q.start, q.tile_sum, q.nrow, (int)blockIdx.x - boff[s]);
}
// one block per scene
__global__ void __launch_bounds__(1024) scan_tiles_multi(const ScanPack *__restrict__ pk) {
  const ScanPack q = pk[blockIdx.x];
  scan_tiles_kernel_body(q.tile_sum, q.tile_off, q.ntiles, 0);
}
__global__ void __launch_bounds__(256) scatter_sorted_multi(const ScatterPack *__restrict__ pk,
                                                            const int *__restrict__ boff, int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const ScatterPack q = pk[s];
  scatter_sorted_kernel_body(q.pos_in, q.vel_in, q.n, q.key, q.slot, q.start, q.tile_off, q.pos_out, q.vel_out,
                             (int)blockIdx.x - boff[s]);
}
__global__ void __launch_bounds__(256) deposit_count_multi(const DepPlanPack *__restrict__ pk,
                                                           const int *__restrict__ boff, int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const DepPlanPack &q = pk[s];
  deposit_count_kernel_body<3>(q.start, q.tile_off, q.a, q.nch, q.seg_tab, q.err, (int)blockIdx.x - boff[s]);
}
// one block per scene
__global__ void __launch_bounds__(1024) deposit_plan_multi(const DepPlanPack *__restrict__ pk) {
  const DepPlanPack &q = pk[blockIdx.x];
  deposit_plan_kernel_body<3>(q.start, q.tile_off, q.a, q.nch, q.item_off, q.slot_off, q.seg_tab, q.item_blk, q.err, 0);
}
template <bool AGG>
__global__ void __launch_bounds__(256, 4) deposit_multi(const DepPack *__restrict__ pk, const int *__restrict__ boff,
                                                        int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const DepPack &q = pk[s];
  deposit_kernel_body<3, 1, AGG>(q.pos4, q.mmax, q.a, q.tw, nullptr, q.spec, q.err, q.item_off, q.slot_off, q.seg_tab,
                                 q.item_blk, q.scratch, q.counters, (int)blockIdx.x - boff[s]);
}
__global__ void __launch_bounds__(256) fft_rows_multi(const RowsPack *__restrict__ pk, const int *__restrict__ boff,
                                                      int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const RowsPack &q = pk[s];
  fft_rows_kernel_body(q.data, q.nrows, q.RB, q.L, q.fdL, q.twmul, q.Lt, q.tw, q.inverse, (int)blockIdx.x - boff[s]);
}
template <int TY>
__global__ void __launch_bounds__(512) green_multi(const GreenPack *__restrict__ pk, const int *__restrict__ boff,
                                                   int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const GreenPack &q = pk[s];
  fft_z_green_kernel_body<TY>(q.spec, q.a, q.tw, q.out, (int)blockIdx.x - boff[s]);
}
__global__ void __launch_bounds__(512, 2) c2r_multi(const C2RPack *__restrict__ pk, const int *__restrict__ boff,
                                                    int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const C2RPack &q = pk[s];
  if (q.a.L <= 256)
    c2r_rows_kernel_body<true, true>(q.in, q.a, q.tw, q.out, (int)blockIdx.x - boff[s]);
  else
    c2r_rows_kernel_body<true, false>(q.in, q.a, q.tw, q.out, (int)blockIdx.x - boff[s]);
}
__global__ void __launch_bounds__(256) gather_multi(const GatherPack *__restrict__ pk, const int *__restrict__ boff,
                                                    int ns) {
  const int s = scene_of(boff, ns, blockIdx.x);
  const GatherPack &q = pk[s];
  gather_kernel_body<3, MODE_KD>(q.F4, q.pos4, q.vel4, q.n, q.a, nullptr, nullptr, nullptr, q.key, q.slot,
                                 q.row_count, q.err, (int)blockIdx.x - boff[s]);
}

}  // namespace augur
