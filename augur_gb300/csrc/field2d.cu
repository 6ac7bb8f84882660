// field2d.cu — the reference's production 2D scatter-field model around the PM plan:
// three-channel CIC scatter, the 5-level U-Net grid net with the recurrent potential input,
// potential gradient + learned kernel acceleration, momentum fix and the velocity-Verlet
// pieces (ScatterField with net="unet", potential=True, kernel=True, pp>0, verlet=True;
// scripts/scatter_field.py:28-67, 221-261, 551-555, 561-688).
//
// The U-Net runs in fp32 on the CUDA cores, as the reference's default path does: a 3x3
// convolution kernel whose input loader also performs avg_pool2d(2) of the previous level,
// or nearest upsampling by 2 concatenated with the skip tensor, so pooling, upsampling and
// concatenation never materialise. Layout: channels-first (C, H, W) per scene, as torch's
// NCHW with B = 1.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "augur_common.cuh"
#include "augur_field2d.h"

namespace {

cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }
unsigned nblocks(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

#define F2_LAUNCH_CHECK()                                                                                  \
  do {                                                                                                     \
    cudaError_t _e = cudaGetLastError();                                                                   \
    if (_e != cudaSuccess) {                                                                               \
      fprintf(stderr, "augur: launch failed: %s (%s:%d)\n", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return AUGUR_ECUDA;                                                                                  \
    }                                                                                                      \
  } while (0)

__device__ __forceinline__ float gelu_erf(float t) { return 0.5f * t * (1.f + erff(t * 0.70710678118654752440f)); }

// ---------------------------------------------------------------------------------
// Three-channel scatter [m, m vx, m vy] * in_scale / h^2 (ScatterField.scatter,
// scripts/scatter_field.py:237-250), out-of-grid corners dropped (:208). Deterministic:
// each corner's fp32 contribution is rounded to a per-channel fixed point 2^-e_c and summed
// with 64-bit integer atomics, where e_c keeps n * max|value_c| below 2^61.
// ---------------------------------------------------------------------------------
struct ScatterArgs {
  int G;
  float E, h, scale;  // scale = in_scale / h^2
};

__device__ __forceinline__ void cic2(float x, float y, const ScatterArgs &a, int &ix, int &iy, float &wx, float &wy) {
  // ScatterField._corners: u = (x + E/2) / h - 0.5, i0 = floor(u), w = u - i0 (fp32)
  const float ux = __fsub_rn(__fdiv_rn(__fadd_rn(x, 0.5f * a.E), a.h), 0.5f);
  const float uy = __fsub_rn(__fdiv_rn(__fadd_rn(y, 0.5f * a.E), a.h), 0.5f);
  const float fx = floorf(ux), fy = floorf(uy);
  ix = (int)fx;
  iy = (int)fy;
  wx = __fsub_rn(ux, fx);
  wy = __fsub_rn(uy, fy);
}

__global__ void f2_absmax_kernel(const float *__restrict__ vel, const float *__restrict__ mass,
                                 const float *__restrict__ mask, int64_t n, float scale, unsigned *__restrict__ mx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float m0 = 0.f, m1 = 0.f, m2 = 0.f;
  if (i < n) {
    const float mm = mass[i] * mask[i];
    const float v0 = mm * scale, v1 = mm * vel[2 * i] * scale, v2 = mm * vel[2 * i + 1] * scale;
    m0 = fabsf(v0);
    m1 = fabsf(v1);
    m2 = fabsf(v2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  if ((threadIdx.x & 31) == 0) {  // non-negative floats order as their bit patterns
    atomicMax(&mx[0], __float_as_uint(m0));
    atomicMax(&mx[1], __float_as_uint(m1));
    atomicMax(&mx[2], __float_as_uint(m2));
  }
}

__device__ __forceinline__ int fix_exp(unsigned mbits, int64_t n) {
  const float m = __uint_as_float(mbits);
  if (!(m > 0.f) || !isfinite(m)) return 0;
  int ex;
  frexpf(m, &ex);  // m < 2^ex
  int ln = 0;
  while ((1ll << ln) < n) ++ln;  // n <= 2^ln
  return 61 - ex - ln;
}

__global__ void f2_scatter_kernel(const float *__restrict__ pos, const float *__restrict__ vel,
                                  const float *__restrict__ mass, const float *__restrict__ mask, int64_t n,
                                  ScatterArgs a, const unsigned *__restrict__ mx,
                                  unsigned long long *__restrict__ acc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float mm = mass[i] * mask[i];
  const float val[3] = {mm * a.scale, mm * vel[2 * i] * a.scale, mm * vel[2 * i + 1] * a.scale};
  float sc[3];  // 2^e, exact in fp32 (fix_exp keeps e within +-126 for finite values)
#pragma unroll
  for (int c = 0; c < 3; ++c) sc[c] = __int_as_float((127 + max(-120, min(120, fix_exp(mx[c], n)))) << 23);
  int ix, iy;
  float wx, wy;
  cic2(pos[2 * i], pos[2 * i + 1], a, ix, iy, wx, wy);
  const int G = a.G;
#pragma unroll
  for (int oy = 0; oy < 2; ++oy) {
#pragma unroll
    for (int ox = 0; ox < 2; ++ox) {
      const int x = ix + ox, y = iy + oy;
      if (x < 0 || x >= G || y < 0 || y >= G) continue;
      const float w = (ox ? wx : 1.f - wx) * (oy ? wy : 1.f - wy);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long q = __float2ll_rn(__fmul_rn(val[c] * w, sc[c]));
        atomicAdd(&acc[((size_t)c * G + y) * G + x], (unsigned long long)q);
      }
    }
  }
}

__global__ void f2_convert_kernel(const unsigned long long *__restrict__ acc, const unsigned *__restrict__ mx, int64_t n,
                                  int G, float *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3ll * G * G) return;
  const int c = (int)(e / ((int64_t)G * G));
  const long long q = (long long)acc[e];
  out[e] = (float)ldexp((double)q, -max(-120, min(120, fix_exp(mx[c], n))));
}

// ---------------------------------------------------------------------------------
// Input stack channels 3.. : kernel acceleration (a_x, a_y lanes of the plan's force grid)
// then the recurrent field (ScatterField._grid_force concatenation order, :633-640).
// ---------------------------------------------------------------------------------
__global__ void f2_inputs_kernel(const float4 *__restrict__ F4k, const float *__restrict__ field, int cf, int G,
                                 float *__restrict__ x) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int GG = G * G;
  if (e >= GG) return;
  const float4 f = F4k[e];
  x[3 * GG + e] = f.x;
  x[4 * GG + e] = f.y;
  for (int c = 0; c < cf; ++c) x[(5 + c) * GG + e] = field ? field[c * GG + e] : 0.f;
}

// ---------------------------------------------------------------------------------
// 3x3 convolution, zero padding 1, fp32. One CTA = an 8 x 8 output tile x all output
// channels (<= 32): thread (pixel, group of 8 output channels). The CTA stages the layer's
// whole weight block (prepared layout [in][tap][32 outputs], float4 copies) and its input tile
// with halo for every input channel in shared memory, all loads in flight at once, then
// accumulates without further barriers. The input loader applies the source mode:
//   A_SAME: srcA at the output resolution; A_POOL: 2x2 average of srcA at twice the
//   resolution (avg_pool2d(2)); A_UP: srcA at half the resolution, nearest (interpolate x2).
// Channels [CA, CA + CB) come from srcB at the output resolution (the U-Net's skip).
// ---------------------------------------------------------------------------------
enum { A_SAME = 0, A_POOL = 1, A_UP = 2 };
constexpr int CT = 8;   // output tile side
constexpr int CTH = CT + 2;
constexpr int CO = 32;  // output channels per CTA (max); prepared weights are padded to it
constexpr int CIN_MAX = 64;

struct ConvSrc {
  const float *a;
  const float *b;
  int ca, cb, mode;
};

size_t conv_smem(int cin) { return (size_t)cin * 9 * CO * sizeof(float) + (size_t)cin * CTH * CTH * sizeof(float); }

// KS threads share one (pixel, 8 outputs): each sums a contiguous range of the input channels,
// then the partial sums are added in ks order through shared memory (deterministic).
template <int MODE, int KS>
__global__ void __launch_bounds__(256 * KS) f2_conv3_kernel(ConvSrc src, const float *__restrict__ Wp, int cout,
                                                            int H, int act, float *__restrict__ out) {
  extern __shared__ __align__(16) float smem[];
  const int cin = src.ca + src.cb;
  float *sw = smem;                         // [cin][9][CO]
  float *sx = smem + (size_t)cin * 9 * CO;  // [cin][CTH][CTH]
  const int tid = threadIdx.x;
  constexpr int NT = 256 * KS;
  {  // scene blockIdx.z of a batch: channels-first tensors one after another
    const size_t z = blockIdx.z;
    const size_t Ha = MODE == A_POOL ? 2 * (size_t)H : MODE == A_UP ? (size_t)(H >> 1) : (size_t)H;
    src.a += z * src.ca * Ha * Ha;
    if (src.b) src.b += z * src.cb * (size_t)H * H;
    out += z * cout * (size_t)H * H;
  }
  {
    const float4 *w4 = reinterpret_cast<const float4 *>(Wp);
    float4 *s4 = reinterpret_cast<float4 *>(sw);
    const int n4 = cin * 9 * CO / 4;
#pragma unroll 4
    for (int e = tid; e < n4; e += NT) s4[e] = w4[e];
  }
  const int x0 = blockIdx.x * CT, y0 = blockIdx.y * CT;
#pragma unroll 4
  for (int e = tid; e < cin * CTH * CTH; e += NT) {
    const int ch = e / (CTH * CTH), r = e % (CTH * CTH);
    const int yy = y0 + r / CTH - 1, xx = x0 + r % CTH - 1;
    float v = 0.f;
    if (yy >= 0 && yy < H && xx >= 0 && xx < H) {
      if (ch < src.ca) {
        if (MODE == A_SAME) {
          v = src.a[((size_t)ch * H + yy) * H + xx];
        } else if (MODE == A_POOL) {
          const int H2 = 2 * H;
          const float *q = src.a + ((size_t)ch * H2 + 2 * yy) * H2 + 2 * xx;
          v = (((q[0] + q[1]) + q[H2]) + q[H2 + 1]) * 0.25f;
        } else {
          const int Hh = H >> 1;
          v = src.a[((size_t)ch * Hh + (yy >> 1)) * Hh + (xx >> 1)];
        }
      } else {
        v = src.b[((size_t)(ch - src.ca) * H + yy) * H + xx];
      }
    }
    sx[e] = v;
  }
  __syncthreads();
  const int ks = tid >> 8, lt = tid & 255;
  const int p = lt & 63, cg = lt >> 6;
  const int px = p & 7, py = p >> 3;
  const int per = (cin + KS - 1) / KS;
  const int c_lo = ks * per, c_hi = min(cin, c_lo + per);
  float acc[8];
#pragma unroll
  for (int o = 0; o < 8; ++o) acc[o] = 0.f;
#pragma unroll 2
  for (int c = c_lo; c < c_hi; ++c) {
    const float *xc = sx + c * CTH * CTH + py * CTH + px;
    const float *wc = sw + c * 9 * CO + cg * 8;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const float v = xc[(t / 3) * CTH + t % 3];
      const float4 w0 = *reinterpret_cast<const float4 *>(wc + t * CO);
      const float4 w1 = *reinterpret_cast<const float4 *>(wc + t * CO + 4);
      acc[0] += w0.x * v;
      acc[1] += w0.y * v;
      acc[2] += w0.z * v;
      acc[3] += w0.w * v;
      acc[4] += w1.x * v;
      acc[5] += w1.y * v;
      acc[6] += w1.z * v;
      acc[7] += w1.w * v;
    }
  }
  if (KS > 1) {
    __syncthreads();  // the weight region is free: partial sums [ks][o][lt]
    if (ks > 0) {
#pragma unroll
      for (int o = 0; o < 8; ++o) sw[((ks - 1) * 8 + o) * 256 + lt] = acc[o];
    }
    __syncthreads();
    if (ks > 0) return;
#pragma unroll
    for (int k = 1; k < KS; ++k)
#pragma unroll
      for (int o = 0; o < 8; ++o) acc[o] += sw[((k - 1) * 8 + o) * 256 + lt];
  }
  const int x = x0 + px, y = y0 + py;
  if (x >= H || y >= H) return;
  const float *bias = Wp + (size_t)cin * 9 * CO;
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int oc = cg * 8 + o;
    if (oc < cout) {
      const float z = acc[o] + bias[oc];
      out[((size_t)oc * H + y) * H + x] = act ? gelu_erf(z) : z;
    }
  }
}

// torch layout W (cout, cin, 3, 3), b (cout) -> Wp [cin][9][CO] (zero-padded outputs), then CO biases
__global__ void f2_prep_kernel(const float *__restrict__ W, const float *__restrict__ b, int cout, int cin,
                               float *__restrict__ Wp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nw = cin * 9 * CO;
  if (e < nw) {
    const int o = e % CO, t = (e / CO) % 9, c = e / (9 * CO);
    Wp[e] = o < cout ? W[((size_t)o * cin + c) * 9 + t] : 0.f;
  } else if (e < nw + CO) {
    const int o = e - nw;
    Wp[e] = o < cout ? b[o] : 0.f;
  }
}

template <int KS>
int conv3_ks(const ConvSrc &s, const float *Wp, int cout, int H, int act, float *out, int batch, cudaStream_t st) {
  {  // opt in to the large shared-memory carve-out (per device, only ever raised)
    const size_t lim = conv_smem(CIN_MAX);
    if (augur::raise_dyn_smem((const void *)f2_conv3_kernel<A_SAME, KS>, lim) ||
        augur::raise_dyn_smem((const void *)f2_conv3_kernel<A_POOL, KS>, lim) ||
        augur::raise_dyn_smem((const void *)f2_conv3_kernel<A_UP, KS>, lim))
      return AUGUR_ECUDA;
  }
  dim3 grid((H + CT - 1) / CT, (H + CT - 1) / CT, batch);
  // the partial-sum exchange reuses the staging region: (KS - 1) x 8 x 256 floats
  const size_t sm = std::max(conv_smem(s.ca + s.cb), (size_t)(KS - 1) * 8 * 256 * sizeof(float));
  switch (s.mode) {
    case A_SAME: f2_conv3_kernel<A_SAME, KS><<<grid, 256 * KS, sm, st>>>(s, Wp, cout, H, act, out); break;
    case A_POOL: f2_conv3_kernel<A_POOL, KS><<<grid, 256 * KS, sm, st>>>(s, Wp, cout, H, act, out); break;
    default: f2_conv3_kernel<A_UP, KS><<<grid, 256 * KS, sm, st>>>(s, Wp, cout, H, act, out); break;
  }
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

// Input channels are split over 2 threads per output at 64^2 and above (two CTAs of 512 per
// SM), over 4 below (the few CTAs of the coarse levels get 32 warps each).
int conv3(const ConvSrc &s, const float *Wp, int cout, int H, int act, float *out, int batch, cudaStream_t st) {
  const int cin = s.ca + s.cb;
  if (cout < 1 || cout > CO || cin < 1 || cin > CIN_MAX || batch < 1 || batch > 65535) return AUGUR_EINVAL;
  return H >= 64 ? conv3_ks<2>(s, Wp, cout, H, act, out, batch, st)
                 : conv3_ks<4>(s, Wp, cout, H, act, out, batch, st);
}

// The U-Net's convolutions in parameter order: (cin, cout) of each.
int unet_layers(int cin, int cout, int width, int levels, int *ci, int *co) {
  int k = 0;
  ci[k] = cin, co[k++] = width;
  for (int l = 0; l <= levels; ++l) {
    ci[k] = width, co[k++] = width;
    ci[k] = width, co[k++] = width;
  }
  for (int l = 0; l < levels; ++l) {
    ci[k] = 2 * width, co[k++] = width;
    ci[k] = width, co[k++] = width;
  }
  ci[k] = width, co[k++] = cout;
  return k;
}
constexpr int UNET_MAX_LAYERS = 4 * 11 + 2;

// ---------------------------------------------------------------------------------
// Grid acceleration -grad(phi) (central differences, zero padding; ScatterField.neg_grad,
// :551-555) plus the kernel acceleration, as a float4 grid (a_x, a_y, 0, 0) for the gather.
// ---------------------------------------------------------------------------------
__global__ void f2_accel_kernel(const float *__restrict__ phi, const float4 *__restrict__ F4k, int G, float two_h,
                                float4 *__restrict__ F4) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G * G) return;
  const int y = e / G, x = e - y * G;
  const float xp = x + 1 < G ? phi[e + 1] : 0.f, xm = x > 0 ? phi[e - 1] : 0.f;
  const float yp = y + 1 < G ? phi[e + G] : 0.f, ym = y > 0 ? phi[e - G] : 0.f;
  float ax = -((xp - xm) / two_h), ay = -((yp - ym) / two_h);
  if (F4k) {
    const float4 k = F4k[e];
    ax += k.x;
    ay += k.y;
  }
  F4[e] = make_float4(ax, ay, 0.f, 0.f);
}

// ---------------------------------------------------------------------------------
// a = a_grid (+ a_pair); momentum fix a -= sum(mm a) / max(sum(mm), 1e-9) (:612-614), then
// a *= mask (:615). FP64 sums in a fixed order: MF_BLOCKS grid-strided partials, one fold.
// ---------------------------------------------------------------------------------
constexpr int MF_BLOCKS = 256;
constexpr int MF_THREADS = 256;

__global__ void __launch_bounds__(MF_THREADS) f2_momsum_kernel(const float *__restrict__ a1,
                                                               const float *__restrict__ a2,
                                                               const float *__restrict__ mass,
                                                               const float *__restrict__ mask, int64_t n,
                                                               double *__restrict__ part) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * MF_THREADS + threadIdx.x; i < n; i += (int64_t)MF_BLOCKS * MF_THREADS) {
    const float mm = mass[i] * mask[i];
    float ax = a1[2 * i], ay = a1[2 * i + 1];
    if (a2) {
      ax += a2[2 * i];
      ay += a2[2 * i + 1];
    }
    s0 += (double)mm;
    s1 += (double)(mm * ax);
    s2 += (double)(mm * ay);
  }
  __shared__ double sh[3][MF_THREADS];
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int w = MF_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) part[threadIdx.x * MF_BLOCKS + blockIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(MF_BLOCKS) f2_momfold_kernel(double *__restrict__ part, float *__restrict__ mean) {
  __shared__ double sh[3][MF_BLOCKS];
  for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] = part[c * MF_BLOCKS + threadIdx.x];
  __syncthreads();
  for (int w = MF_BLOCKS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = fmax(sh[0][0], 1e-9);
    mean[0] = (float)(sh[1][0] / m);
    mean[1] = (float)(sh[2][0] / m);
  }
}

__global__ void f2_finish_kernel(const float *__restrict__ a1, const float *__restrict__ a2,
                                 const float *__restrict__ mask, int64_t n, const float *__restrict__ mean,
                                 float *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float ax = a1[2 * i], ay = a1[2 * i + 1];
  if (a2) {
    ax += a2[2 * i];
    ay += a2[2 * i + 1];
  }
  if (mean) {
    ax -= mean[0];
    ay -= mean[1];
  }
  out[2 * i] = ax * mask[i];
  out[2 * i + 1] = ay * mask[i];
}

// ---------------------------------------------------------------------------------
// Velocity Verlet pieces of ScatterField._step (:677-688).
// ---------------------------------------------------------------------------------
__global__ void f2_drift_kernel(const float *__restrict__ pos, const float *__restrict__ vel,
                                const float *__restrict__ acc, int64_t n2, float dt, float hdt2,
                                float *__restrict__ pos_out, float *__restrict__ vel_pred) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n2) return;
  const float a = acc[e], v = vel[e];
  pos_out[e] = (pos[e] + dt * v) + hdt2 * a;
  vel_pred[e] = v + dt * a;
}

__global__ void f2_kick_kernel(const float *__restrict__ vel, const float *__restrict__ a0,
                               const float *__restrict__ a1, int64_t n2, float hdt, float *__restrict__ vel_out,
                               float *__restrict__ dv) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n2) return;
  const float d = hdt * (a0[e] + a1[e]);
  if (dv) dv[e] = d;
  vel_out[e] = vel[e] + d;
}

// ---------------------------------------------------------------------------------
// Chunked large-N tick (scripts/scatter_bh_1b.py:107-146): body state stored in fp32, fp16 or
// bf16, widened to fp32 per body; relativistic speed v = p / sqrt(1 + |p|^2 / c^2)
// (scripts/scatter_bh.py:22-23); drift fused into the three-channel scatter, gather fused with
// the kick. Unit masses and masks, as the reference's Sim.
// ---------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ float ld_f(const T *p, int64_t i);
template <> __device__ __forceinline__ float ld_f<float>(const float *p, int64_t i) { return p[i]; }
template <> __device__ __forceinline__ float ld_f<__half>(const __half *p, int64_t i) { return __half2float(p[i]); }
template <> __device__ __forceinline__ float ld_f<__nv_bfloat16>(const __nv_bfloat16 *p, int64_t i) {
  return __bfloat162float(p[i]);
}
template <typename T> __device__ __forceinline__ float st_f(T *p, int64_t i, float v);  // returns the stored value
template <> __device__ __forceinline__ float st_f<float>(float *p, int64_t i, float v) { p[i] = v; return v; }
template <> __device__ __forceinline__ float st_f<__half>(__half *p, int64_t i, float v) {
  const __half h = __float2half_rn(v);
  p[i] = h;
  return __half2float(h);
}
template <> __device__ __forceinline__ float st_f<__nv_bfloat16>(__nv_bfloat16 *p, int64_t i, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  p[i] = h;
  return __bfloat162float(h);
}

// (x, y) of body i as one 2-element load / store
template <typename T> __device__ __forceinline__ float2 ld2(const T *p, int64_t i);
template <> __device__ __forceinline__ float2 ld2<float>(const float *p, int64_t i) {
  return reinterpret_cast<const float2 *>(p)[i];
}
template <> __device__ __forceinline__ float2 ld2<__half>(const __half *p, int64_t i) {
  return __half22float2(reinterpret_cast<const __half2 *>(p)[i]);
}
template <> __device__ __forceinline__ float2 ld2<__nv_bfloat16>(const __nv_bfloat16 *p, int64_t i) {
  return __bfloat1622float2(reinterpret_cast<const __nv_bfloat162 *>(p)[i]);
}
template <typename T> __device__ __forceinline__ void st2(T *p, int64_t i, float2 v);  // v already representable
template <> __device__ __forceinline__ void st2<float>(float *p, int64_t i, float2 v) {
  reinterpret_cast<float2 *>(p)[i] = v;
}
template <> __device__ __forceinline__ void st2<__half>(__half *p, int64_t i, float2 v) {
  reinterpret_cast<__half2 *>(p)[i] = __floats2half2_rn(v.x, v.y);
}
template <> __device__ __forceinline__ void st2<__nv_bfloat16>(__nv_bfloat16 *p, int64_t i, float2 v) {
  reinterpret_cast<__nv_bfloat162 *>(p)[i] = __floats2bfloat162_rn(v.x, v.y);
}

template <typename T> __device__ __forceinline__ float round_f(float v);  // v rounded to T, widened back
template <> __device__ __forceinline__ float round_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float round_f<__half>(float v) { return __half2float(__float2half_rn(v)); }
template <> __device__ __forceinline__ float round_f<__nv_bfloat16>(float v) {
  return __bfloat162float(__float2bfloat16_rn(v));
}

struct TickArgs {
  int G;
  float E, h, scale;       // scale = in_scale / h^2
  float ms, c2, dt;        // momentum scale, c^2, drift step
  int e[3];                // fixed-point exponents of the three channels
  float p2[3];             // 2^e, exact in fp32: value * 2^e is exact, so the integer is the rounded value
  float inv_h, inv_ms;     // 1/h, 1/ms when h, ms are powers of two (x / h == x * (1/h) exactly), else 0
};

__device__ __forceinline__ float div_or_mul(float x, float d, float inv) {
  return inv != 0.f ? __fmul_rn(x, inv) : __fdiv_rn(x, d);
}

// fp32 in torch's operation order, no contractions: p / sqrt(1 + (px^2 + py^2) / c^2)
__device__ __forceinline__ void rel_speed(float px, float py, const TickArgs &a, float &vx, float &vy) {
  const float s = __fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py));
  const float d = __fsqrt_rn(__fadd_rn(1.f, __fdiv_rn(s, a.c2)));
  vx = __fdiv_rn(px, d);
  vy = __fdiv_rn(py, d);
}

// Position after the drift as the state type stores it: (pos + dt v) rounded to TP.
template <typename TP, typename TM>
__device__ __forceinline__ void drifted(const TP *pos, const TM *mom, int64_t i, const TickArgs &a, int drift,
                                        float &x, float &y, float &vx, float &vy) {
  const float2 p = ld2(mom, i), q = ld2(pos, i);
  rel_speed(__fmul_rn(p.x, a.ms), __fmul_rn(p.y, a.ms), a, vx, vy);
  x = q.x;
  y = q.y;
  if (drift) {
    x = round_f<TP>(__fadd_rn(x, __fmul_rn(a.dt, vx)));
    y = round_f<TP>(__fadd_rn(y, __fmul_rn(a.dt, vy)));
  }
}

__device__ __forceinline__ void cic_w(float x, float y, const TickArgs &a, int &ix, int &iy, float &wx, float &wy) {
  const float ux = __fsub_rn(div_or_mul(__fadd_rn(x, 0.5f * a.E), a.h, a.inv_h), 0.5f);
  const float uy = __fsub_rn(div_or_mul(__fadd_rn(y, 0.5f * a.E), a.h, a.inv_h), 0.5f);
  const float fx = floorf(ux), fy = floorf(uy);
  wx = __fsub_rn(ux, fx);
  wy = __fsub_rn(uy, fy);
  ix = (int)fx;
  iy = (int)fy;
}

// Scatter at the drifted positions (the state is not written here). SMEM: one channel per CTA
// (blockIdx.y) in int64 shared accumulators (G^2 words), a grid-stride loop over the bodies,
// one flush per CTA into the global int64 grid; otherwise int64 global atomics, all channels.
template <typename TP, typename TM, bool SMEM>
__global__ void __launch_bounds__(1024) t2_scatter_kernel(const TP *__restrict__ pos, const TM *__restrict__ mom,
                                                          int64_t n, TickArgs a, int drift,
                                                          unsigned long long *__restrict__ acc) {
  extern __shared__ unsigned long long s_acc64[];
  const int G = a.G, GG = G * G;
  const int ch = SMEM ? blockIdx.y : 0;
  if (SMEM) {
    for (int e = threadIdx.x; e < GG; e += blockDim.x) s_acc64[e] = 0ull;
    __syncthreads();
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float x, y, vx, vy;
    drifted(pos, mom, i, a, drift, x, y, vx, vy);
    const float val[3] = {a.scale, __fmul_rn(vx, a.scale), __fmul_rn(vy, a.scale)};
    int ix, iy;
    float wx, wy;
    cic_w(x, y, a, ix, iy, wx, wy);
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int cx = ix + ox, cy = iy + oy;
        if (cx < 0 || cx >= G || cy < 0 || cy >= G) continue;
        const float w = __fmul_rn(ox ? wx : __fsub_rn(1.f, wx), oy ? wy : __fsub_rn(1.f, wy));
        if (SMEM) {
          const long long q = __float2ll_rn(__fmul_rn(__fmul_rn(val[ch], w), a.p2[ch]));
          atomicAdd(&s_acc64[cy * G + cx], (unsigned long long)q);
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const long long q = __float2ll_rn(__fmul_rn(__fmul_rn(val[c], w), a.p2[c]));
            atomicAdd(&acc[(size_t)c * GG + cy * G + cx], (unsigned long long)q);
          }
        }
      }
    }
  }
  if (SMEM) {
    __syncthreads();
    for (int e = threadIdx.x; e < GG; e += blockDim.x) {
      const unsigned long long v = s_acc64[e];
      if (v) atomicAdd(&acc[(size_t)ch * GG + e], v);
    }
  }
}

// the drift alone, stored (Sim.scatter_pass's pos update when no scatter follows)
template <typename TP, typename TM>
__global__ void t2_drift_kernel(TP *__restrict__ pos, const TM *__restrict__ mom, int64_t n, TickArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x, y, vx, vy;
  drifted(pos, mom, i, a, 1, x, y, vx, vy);
  st2(pos, i, make_float2(x, y));
}

__global__ void t2_convert_kernel(const unsigned long long *__restrict__ acc, TickArgs a, float *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int GG = a.G * a.G;
  if (e >= 3 * GG) return;
  out[e] = (float)ldexp((double)(long long)acc[e], -a.e[e / GG]);
}

// mean acceleration from the grid: sum_cells acc * rho * cell_mass / n, FP64 in a fixed order
// (Sim.grid_force, scripts/scatter_bh_1b.py:113-121)
__global__ void __launch_bounds__(MF_THREADS) t2_abar_part_kernel(const float4 *__restrict__ F4,
                                                                  const float *__restrict__ rho, int GG,
                                                                  double cell_mass, double *__restrict__ part) {
  double s1 = 0.0, s2 = 0.0;
  for (int e = blockIdx.x * MF_THREADS + threadIdx.x; e < GG; e += MF_BLOCKS * MF_THREADS) {
    const double w = (double)rho[e] * cell_mass;
    const float4 f = F4[e];
    s1 += (double)f.x * w;
    s2 += (double)f.y * w;
  }
  __shared__ double sh[2][MF_THREADS];
  sh[0][threadIdx.x] = s1;
  sh[1][threadIdx.x] = s2;
  __syncthreads();
  for (int w = MF_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = 0.0;  // count slot unused
    part[MF_BLOCKS + blockIdx.x] = sh[0][0];
    part[2 * MF_BLOCKS + blockIdx.x] = sh[1][0];
  }
}

__global__ void __launch_bounds__(MF_BLOCKS) t2_abar_fold_kernel(const double *__restrict__ part, double inv_n,
                                                                 float *__restrict__ abar) {
  __shared__ double sh[2][MF_BLOCKS];
  sh[0][threadIdx.x] = part[MF_BLOCKS + threadIdx.x];
  sh[1][threadIdx.x] = part[2 * MF_BLOCKS + threadIdx.x];
  __syncthreads();
  for (int w = MF_BLOCKS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    abar[0] = (float)(sh[0][0] * inv_n);
    abar[1] = (float)(sh[1][0] * inv_n);
  }
}

// a = gather(acc grid) in the reference's corner order (ScatterField._corner_iter: x offset
// outer, y inner; off-grid corners dropped), mom = mom + kick * (a - abar) / ms
template <typename TP, typename TM>
__global__ void t2_gather_kick_kernel(const float4 *__restrict__ F4, TP *__restrict__ pos, TM *__restrict__ mom,
                                      int64_t n, TickArgs a, int drift, float kick, const float *__restrict__ abar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int G = a.G;
  float x, y, vx, vy;
  drifted(pos, mom, i, a, drift, x, y, vx, vy);
  if (drift) st2(pos, i, make_float2(x, y));
  int ix, iy;
  float wx, wy;
  cic_w(x, y, a, ix, iy, wx, wy);
  float ax = 0.f, ay = 0.f;
#pragma unroll
  for (int ox = 0; ox < 2; ++ox) {
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      const int cx = ix + ox, cy = iy + oy;
      const bool ok = cx >= 0 && cx < G && cy >= 0 && cy < G;
      const float w = __fmul_rn(ox ? wx : __fsub_rn(1.f, wx), oy ? wy : __fsub_rn(1.f, wy));
      const float4 f = F4[min(max(cy, 0), G - 1) * G + min(max(cx, 0), G - 1)];
      const float wk = ok ? w : 0.f;
      ax = __fadd_rn(ax, __fmul_rn(f.x, wk));
      ay = __fadd_rn(ay, __fmul_rn(f.y, wk));
    }
  }
  const float2 m0 = ld2(mom, i);
  st2(mom, i, make_float2(__fadd_rn(m0.x, div_or_mul(__fmul_rn(kick, __fsub_rn(ax, abar[0])), a.ms, a.inv_ms)),
                          __fadd_rn(m0.y, div_or_mul(__fmul_rn(kick, __fsub_rn(ay, abar[1])), a.ms, a.inv_ms))));
}

}  // namespace

extern "C" {

size_t augur_field2d_scatter_work_bytes(int grid) {
  return grid < 1 ? 0 : (size_t)3 * grid * grid * sizeof(unsigned long long) + 16;
}

int augur_field2d_scatter(const float *pos, const float *vel, const float *mass, const float *mask, int64_t n,
                          int grid, double extent, double in_scale, float *out3, void *work, void *stream) {
  if (grid < 2 || grid > 4096 || !(extent > 0.0) || !out3 || !work) return AUGUR_EINVAL;
  if (n < 0 || (n > 0 && (!pos || !vel || !mass || !mask))) return AUGUR_EINVAL;
  if ((reinterpret_cast<uintptr_t>(work) & 7) != 0) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  const size_t GG = (size_t)grid * grid;
  auto *acc = reinterpret_cast<unsigned long long *>(work);
  auto *mx = reinterpret_cast<unsigned *>(acc + 3 * GG);
  if (cudaMemsetAsync(work, 0, augur_field2d_scatter_work_bytes(grid), st) != cudaSuccess) return AUGUR_ECUDA;
  ScatterArgs a;
  a.G = grid;
  a.E = (float)extent;
  a.h = (float)(extent / grid);
  a.scale = (float)(in_scale / ((double)a.h * (double)a.h));
  if (n > 0) {
    f2_absmax_kernel<<<nblocks(n, 256), 256, 0, st>>>(vel, mass, mask, n, a.scale, mx);
    F2_LAUNCH_CHECK();
    f2_scatter_kernel<<<nblocks(n, 256), 256, 0, st>>>(pos, vel, mass, mask, n, a, mx, acc);
    F2_LAUNCH_CHECK();
  }
  f2_convert_kernel<<<nblocks(3 * (int64_t)GG, 256), 256, 0, st>>>(acc, mx, n > 0 ? n : 1, grid, out3);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int augur_field2d_inputs(const float *force4, const float *field, int cf, int grid, float *x, void *stream) {
  if (!force4 || !x || grid < 2 || cf < 0 || cf > 8) return AUGUR_EINVAL;
  f2_inputs_kernel<<<nblocks((int64_t)grid * grid, 256), 256, 0, S(stream)>>>(
      reinterpret_cast<const float4 *>(force4), field, cf, grid, x);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int64_t augur_unet2d_param_count(int cin, int cout, int width, int levels) {
  if (cin < 1 || cout < 1 || width < 1 || levels < 0 || levels > 10) return -1;
  int ci[UNET_MAX_LAYERS], co[UNET_MAX_LAYERS];
  const int nl = unet_layers(cin, cout, width, levels, ci, co);
  int64_t n = 0;
  for (int k = 0; k < nl; ++k) n += (int64_t)co[k] * ci[k] * 9 + co[k];
  return n;
}

int64_t augur_unet2d_prepared_count(int cin, int cout, int width, int levels) {
  if (cin < 1 || cout < 1 || width < 1 || levels < 0 || levels > 10) return -1;
  int ci[UNET_MAX_LAYERS], co[UNET_MAX_LAYERS];
  const int nl = unet_layers(cin, cout, width, levels, ci, co);
  int64_t n = 0;
  for (int k = 0; k < nl; ++k) n += (int64_t)ci[k] * 9 * CO + CO;
  return n;
}

int augur_unet2d_prepare(const float *params, int cin, int cout, int width, int levels, float *prepared,
                         void *stream) {
  if (!params || !prepared || cin < 1 || cin > CIN_MAX || cout < 1 || cout > CO || width < 1 || width > CO ||
      2 * width > CIN_MAX || levels < 0 || levels > 10)
    return AUGUR_EINVAL;
  if (reinterpret_cast<uintptr_t>(prepared) & 15) return AUGUR_EINVAL;
  int ci[UNET_MAX_LAYERS], co[UNET_MAX_LAYERS];
  const int nl = unet_layers(cin, cout, width, levels, ci, co);
  const float *p = params;
  float *q = prepared;
  for (int k = 0; k < nl; ++k) {
    const int64_t nw = (int64_t)ci[k] * 9 * CO + CO;
    f2_prep_kernel<<<nblocks(nw, 256), 256, 0, S(stream)>>>(p, p + (int64_t)co[k] * ci[k] * 9, co[k], ci[k], q);
    F2_LAUNCH_CHECK();
    p += (int64_t)co[k] * ci[k] * 9 + co[k];
    q += nw;
  }
  return AUGUR_OK;
}

size_t augur_unet2d_work_bytes(int grid, int width, int levels, int batch) {
  if (grid < 1 || width < 1 || levels < 0 || batch < 1) return 0;
  size_t f = 2 * (size_t)width * grid * grid;  // two full-resolution temporaries
  for (int l = 0; l <= levels; ++l) f += (size_t)width * (grid >> l) * (grid >> l);  // encoder outputs (skips)
  return f * sizeof(float) * batch;
}

int augur_unet2d_forward(const float *prepared, int cin, int cout, int width, int levels, int grid, int batch,
                         const float *x, float *y, void *work, size_t work_bytes, void *stream) {
  if (!prepared || !x || !y || !work || batch < 1 || batch > 65535) return AUGUR_EINVAL;
  if (cin < 1 || cin > CIN_MAX || cout < 1 || cout > CO || width < 1 || width > CO || 2 * width > CIN_MAX ||
      levels < 0 || levels > 10)
    return AUGUR_EINVAL;
  if (grid < 1 || (grid % (1 << levels)) != 0) return AUGUR_EINVAL;
  if (work_bytes < augur_unet2d_work_bytes(grid, width, levels, batch)) return AUGUR_EINVAL;
  if (reinterpret_cast<uintptr_t>(prepared) & 15) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  const size_t GG = (size_t)grid * grid, B = (size_t)batch;
  // every buffer holds the batch's scenes one after another (channels-first per scene)
  float *T0 = reinterpret_cast<float *>(work), *T1 = T0 + B * width * GG;
  float *Sk[11];
  Sk[0] = T1 + B * width * GG;
  for (int l = 1; l <= levels; ++l) Sk[l] = Sk[l - 1] + B * width * (grid >> (l - 1)) * (grid >> (l - 1));
  int ci[UNET_MAX_LAYERS], co[UNET_MAX_LAYERS];
  const int nl = unet_layers(cin, cout, width, levels, ci, co);
  const float *Lw[UNET_MAX_LAYERS];
  const float *q = prepared;
  for (int k = 0; k < nl; ++k) {
    Lw[k] = q;
    q += (int64_t)ci[k] * 9 * CO + CO;
  }
  const int w = width;
  int rc, k = 0;
  // h = gelu(inp(x)); encoder blocks at grid / 2^l, each after avg_pool2d(2) of the previous
  if ((rc = conv3({x, nullptr, cin, 0, A_SAME}, Lw[k++], w, grid, 1, T0, batch, st))) return rc;
  for (int l = 0; l <= levels; ++l) {
    const int H = grid >> l;
    const ConvSrc s1 = l == 0 ? ConvSrc{T0, nullptr, w, 0, A_SAME} : ConvSrc{Sk[l - 1], nullptr, w, 0, A_POOL};
    if ((rc = conv3(s1, Lw[k++], w, H, 1, T1, batch, st))) return rc;
    if ((rc = conv3({T1, nullptr, w, 0, A_SAME}, Lw[k++], w, H, 1, Sk[l], batch, st))) return rc;
  }
  // decoder blocks are stored dec[0] .. dec[levels-1]; they run from the deepest level up
  const int kdec = k;
  const float *h = Sk[levels];
  for (int l = levels - 1; l >= 0; --l) {
    const int H = grid >> l;
    if ((rc = conv3({h, Sk[l], w, w, A_UP}, Lw[kdec + 2 * l], w, H, 1, T1, batch, st))) return rc;
    if ((rc = conv3({T1, nullptr, w, 0, A_SAME}, Lw[kdec + 2 * l + 1], w, H, 1, T0, batch, st))) return rc;
    h = T0;
  }
  return conv3({h, nullptr, w, 0, A_SAME}, Lw[kdec + 2 * levels], cout, grid, 0, y, batch, st);
}

int augur_field2d_accel(const float *phi, const float *force4_kernel, int grid, double h, float *force4_out,
                        void *stream) {
  if (!phi || !force4_out || grid < 2 || !(h > 0.0)) return AUGUR_EINVAL;
  if ((reinterpret_cast<uintptr_t>(force4_out) & 15) || (reinterpret_cast<uintptr_t>(force4_kernel) & 15))
    return AUGUR_EINVAL;
  f2_accel_kernel<<<nblocks((int64_t)grid * grid, 256), 256, 0, S(stream)>>>(
      phi, reinterpret_cast<const float4 *>(force4_kernel), grid, (float)(2.0 * h),
      reinterpret_cast<float4 *>(force4_out));
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

size_t augur_field2d_finish_work_bytes(void) { return (size_t)3 * MF_BLOCKS * sizeof(double) + 16; }

int augur_field2d_finish(const float *acc_grid, const float *acc_pair, const float *mass, const float *mask,
                         int64_t n, int momfix, float *acc_out, void *work, void *stream) {
  if (n < 0 || (n > 0 && (!acc_grid || !mass || !mask || !acc_out))) return AUGUR_EINVAL;
  if (momfix && (!work || (reinterpret_cast<uintptr_t>(work) & 7))) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  cudaStream_t st = S(stream);
  float *mean = nullptr;
  if (momfix) {
    double *part = reinterpret_cast<double *>(work);
    mean = reinterpret_cast<float *>(part + 3 * MF_BLOCKS);
    f2_momsum_kernel<<<MF_BLOCKS, MF_THREADS, 0, st>>>(acc_grid, acc_pair, mass, mask, n, part);
    F2_LAUNCH_CHECK();
    f2_momfold_kernel<<<1, MF_BLOCKS, 0, st>>>(part, mean);
    F2_LAUNCH_CHECK();
  }
  f2_finish_kernel<<<nblocks(n, 256), 256, 0, st>>>(acc_grid, acc_pair, mask, n, mean, acc_out);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int augur_field2d_drift(const float *pos, const float *vel, const float *acc, int64_t n, double dt, float *pos_out,
                        float *vel_pred, void *stream) {
  if (n < 0 || (n > 0 && (!pos || !vel || !acc || !pos_out || !vel_pred))) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  f2_drift_kernel<<<nblocks(2 * n, 256), 256, 0, S(stream)>>>(pos, vel, acc, 2 * n, (float)dt,
                                                              (float)(0.5 * dt * dt), pos_out, vel_pred);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int augur_field2d_kick(const float *vel, const float *acc0, const float *acc1, int64_t n, double dt, float *vel_out,
                       float *dv_out, void *stream) {
  if (n < 0 || (n > 0 && (!vel || !acc0 || !acc1 || !vel_out))) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  f2_kick_kernel<<<nblocks(2 * n, 256), 256, 0, S(stream)>>>(vel, acc0, acc1, 2 * n, (float)(0.5 * dt), vel_out,
                                                             dv_out);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

}  // extern "C"

// ---- chunked large-N tick ----------------------------------------------------------------
namespace {
TickArgs tick_args(int grid, double extent, double in_scale, double ms, double c, double dt) {
  TickArgs a{};
  a.G = grid;
  a.E = (float)extent;
  a.h = (float)(extent / grid);
  a.scale = (float)(in_scale / ((double)a.h * (double)a.h));
  a.ms = (float)ms;
  a.c2 = (float)(c * c);
  a.dt = (float)dt;
  auto inv_pow2 = [](float v) {
    int e;
    return (v > 0.f && std::frexp(v, &e) == 0.5f) ? 1.0f / v : 0.f;  // exact reciprocal of a power of two
  };
  a.inv_h = inv_pow2(a.h);
  a.inv_ms = inv_pow2(a.ms);
  return a;
}
int ceil_log2(double v) {
  int e;
  std::frexp(v, &e);  // v < 2^e
  return e;
}
constexpr size_t T2_SMEM_MAX = 200 * 1024;

template <typename TP, typename TM>
int tick_launch(int what, void *pos, void *mom, int64_t n, TickArgs a, int drift, unsigned long long *acc,
                const float4 *F4, float kick, const float *abar, cudaStream_t st) {
  if (what == 0) {  // scatter
    const size_t sm = (size_t)a.G * a.G * sizeof(unsigned long long);
    if (sm <= T2_SMEM_MAX) {
      if (augur::raise_dyn_smem((const void *)t2_scatter_kernel<TP, TM, true>, T2_SMEM_MAX)) return AUGUR_ECUDA;
      // persistent CTAs per channel (one per SM at this shared-memory size), each flushes once
      const unsigned per = (unsigned)std::max<int64_t>(1, std::min<int64_t>(101, (n + 1023) / 1024));
      t2_scatter_kernel<TP, TM, true><<<dim3(per, 3), 1024, sm, st>>>((const TP *)pos, (const TM *)mom, n, a, drift,
                                                                      acc);
    } else {
      t2_scatter_kernel<TP, TM, false><<<(unsigned)std::min<int64_t>((n + 1023) / 1024, 4096), 1024, 0, st>>>(
          (const TP *)pos, (const TM *)mom, n, a, drift, acc);
    }
  } else if (what == 1) {
    t2_drift_kernel<TP, TM><<<nblocks(n, 256), 256, 0, st>>>((TP *)pos, (const TM *)mom, n, a);
  } else {
    t2_gather_kick_kernel<TP, TM><<<nblocks(n, 256), 256, 0, st>>>(F4, (TP *)pos, (TM *)mom, n, a, drift, kick, abar);
  }
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}
template <typename TP>
int tick_m(int mt, int what, void *pos, void *mom, int64_t n, TickArgs a, int drift, unsigned long long *acc,
           const float4 *F4, float kick, const float *abar, cudaStream_t st) {
  switch (mt) {
    case AUGUR_DTYPE_F32: return tick_launch<TP, float>(what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
    case AUGUR_DTYPE_F16: return tick_launch<TP, __half>(what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
    case AUGUR_DTYPE_BF16:
      return tick_launch<TP, __nv_bfloat16>(what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
  }
  return AUGUR_EINVAL;
}
int tick_dispatch(int pt, int mt, int what, void *pos, void *mom, int64_t n, TickArgs a, int drift,
                  unsigned long long *acc, const float4 *F4, float kick, const float *abar, cudaStream_t st) {
  switch (pt) {
    case AUGUR_DTYPE_F32: return tick_m<float>(mt, what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
    case AUGUR_DTYPE_F16: return tick_m<__half>(mt, what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
    case AUGUR_DTYPE_BF16: return tick_m<__nv_bfloat16>(mt, what, pos, mom, n, a, drift, acc, F4, kick, abar, st);
  }
  return AUGUR_EINVAL;
}
}  // namespace

extern "C" {

size_t augur_tick2d_work_bytes(int grid) {
  return grid < 1 ? 0 : (size_t)3 * grid * grid * sizeof(unsigned long long) + 3 * MF_BLOCKS * sizeof(double);
}

int augur_tick2d_drift_scatter(const void *pos, const void *mom, int64_t n, int pos_type, int mom_type,
                               double mom_scale, double c, double dt, int drift, int grid, double extent,
                               double in_scale, float *out3, void *work, void *stream) {
  if (grid < 2 || grid > 4096 || !(extent > 0.0) || !(c > 0.0) || !(mom_scale > 0.0) || !out3 || !work)
    return AUGUR_EINVAL;
  if (n < 0 || (n > 0 && (!pos || !mom)) || (reinterpret_cast<uintptr_t>(work) & 7)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  TickArgs a = tick_args(grid, extent, in_scale, mom_scale, c, dt);
  // |v| < c bounds every channel value before the pass: n of them fit in 61 bits
  const double vmax[3] = {(double)a.scale, c * a.scale, c * a.scale};
  for (int k = 0; k < 3; ++k) {
    a.e[k] = 61 - ceil_log2((double)std::max<int64_t>(n, 1)) - ceil_log2(vmax[k]);
    a.e[k] = std::max(-120, std::min(120, a.e[k]));  // 2^e stays a normal fp32 power of two
    a.p2[k] = std::ldexp(1.0f, a.e[k]);
  }
  auto *acc = reinterpret_cast<unsigned long long *>(work);
  if (cudaMemsetAsync(acc, 0, (size_t)3 * grid * grid * sizeof(unsigned long long), st) != cudaSuccess)
    return AUGUR_ECUDA;
  if (n > 0) {
    const int rc = tick_dispatch(pos_type, mom_type, 0, const_cast<void *>(pos), const_cast<void *>(mom), n, a,
                                 drift, acc, nullptr, 0.f, nullptr, st);
    if (rc) return rc;
  }
  t2_convert_kernel<<<nblocks(3 * (int64_t)grid * grid, 256), 256, 0, st>>>(acc, a, out3);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int augur_tick2d_drift(void *pos, const void *mom, int64_t n, int pos_type, int mom_type, double mom_scale, double c,
                       double dt, void *stream) {
  if (!(c > 0.0) || !(mom_scale > 0.0) || n < 0 || (n > 0 && (!pos || !mom))) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  TickArgs a = tick_args(2, 1.0, 1.0, mom_scale, c, dt);
  return tick_dispatch(pos_type, mom_type, 1, pos, const_cast<void *>(mom), n, a, 1, nullptr, nullptr, 0.f, nullptr,
                       S(stream));
}

int augur_tick2d_mean_acc(const float *force4, const float *rho, int grid, double cell_mass, int64_t n, float *abar,
                          void *work, void *stream) {
  if (!force4 || !rho || !abar || !work || grid < 1 || n < 1) return AUGUR_EINVAL;
  if ((reinterpret_cast<uintptr_t>(force4) & 15) || (reinterpret_cast<uintptr_t>(work) & 7)) return AUGUR_EINVAL;
  cudaStream_t st = S(stream);
  double *part = reinterpret_cast<double *>(reinterpret_cast<unsigned long long *>(work) + (size_t)3 * grid * grid);
  t2_abar_part_kernel<<<MF_BLOCKS, MF_THREADS, 0, st>>>(reinterpret_cast<const float4 *>(force4), rho, grid * grid,
                                                        cell_mass, part);
  F2_LAUNCH_CHECK();
  t2_abar_fold_kernel<<<1, MF_BLOCKS, 0, st>>>(part, 1.0 / (double)n, abar);
  F2_LAUNCH_CHECK();
  return AUGUR_OK;
}

int augur_tick2d_gather_kick(const float *force4, void *pos, void *mom, int64_t n, int pos_type, int mom_type,
                             double mom_scale, double kick_dt, const float *abar, int grid, double extent, int drift,
                             double c, double dt, void *stream) {
  if (!force4 || !abar || grid < 2 || !(extent > 0.0) || !(mom_scale > 0.0) || (drift && !(c > 0.0)))
    return AUGUR_EINVAL;
  if (n < 0 || (n > 0 && (!pos || !mom)) || (reinterpret_cast<uintptr_t>(force4) & 15)) return AUGUR_EINVAL;
  if (n == 0) return AUGUR_OK;
  TickArgs a = tick_args(grid, extent, 1.0, mom_scale, drift ? c : 1.0, dt);
  return tick_dispatch(pos_type, mom_type, 2, pos, mom, n, a, drift, nullptr, reinterpret_cast<const float4 *>(force4),
                       (float)kick_dt, abar, S(stream));
}

}  // extern "C"
