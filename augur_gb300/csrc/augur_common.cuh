// augur_common.cuh — shared device helpers for the sm_103a PM kernels.
//
// Cell-index arithmetic is the reference's, restated so that it is bit-exact with
// ScatterField._corners (scripts/scatter_field.py:179-182) as PyTorch evaluates it on
// the CPU: fp32 add of fp32(extent/2), IEEE fp32 true division by fp32(h), fp32
// subtract of 0.5, floor. The explicit __f*_rn intrinsics keep nvcc from contracting
// the sequence into FMAs or replacing the division by a reciprocal multiply (which is
// what a reciprocal-based kernel would do, and which moves floor() for G=96).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/augur_pm.h"

#define AUGUR_ERRBIT_NONFINITE 1u
#define AUGUR_ERRBIT_RANGE 2u

namespace augur {

// ---------------------------------------------------------------------------------
// complex helpers (float2 = re, im)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }

// ---------------------------------------------------------------------------------
// bit-exact CIC axis: u = (x + E/2)/h - 0.5 ; i0 = floor(u) ; w = u - i0
// (scripts/scatter_field.py:179-182). Returns false for non-finite or huge u.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool cic_axis(float x, float half_ext, float h, int &i0, float &w) {
  float t = __fadd_rn(x, half_ext);
  float u = __fsub_rn(__fdiv_rn(t, h), 0.5f);
  if (!(fabsf(u) < 1.0e9f)) {  // catches NaN and inf
    i0 = 0;
    w = 0.f;
    return false;
  }
  float f = floorf(u);
  i0 = (int)f;
  w = __fsub_rn(u, f);
  return true;
}

__device__ __forceinline__ int wrap_idx(int i, int G) {
  int r = i % G;
  return r < 0 ? r + G : r;
}

// weight factor of one axis for corner offset o (0 -> 1-w, 1 -> w), fp32 like the reference
__device__ __forceinline__ float axis_w(float w, int o) { return o ? w : __fsub_rn(1.0f, w); }

__device__ __forceinline__ void set_err(unsigned *err, unsigned bit) {
  if (err) atomicOr(err, bit);
}

// ---------------------------------------------------------------------------------
// Shared-memory mixed-radix Stockham FFT (radix 2,3,4,8), natural order in and out.
//
// Data: nb transforms of length L; element e of transform b sits at
// buf[b*bs + e*es]. Each stage reads `in` and writes `out` (ping-pong), with a
// __syncthreads() after it. tw is the length-L table tw[t] = exp(-2 pi i t / L)
// (or a longer table sampled with stride twmul: tw[t*twmul]).
// ---------------------------------------------------------------------------------
struct FftShape {
  int L;
  int nstages;
  int radix[12];
};

template <int R>
__device__ __forceinline__ void dft(float2 *v, bool inv) {
  if constexpr (R == 2) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 3) {
    const float s3 = 0.86602540378443864676f;
    float2 a = v[0], b = v[1], c = v[2];
    float2 t1 = cadd(b, c);
    float2 t2 = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
    float2 d = make_float2(s3 * (b.x - c.x), s3 * (b.y - c.y));
    // forward: X1 = t2 - i d ; X2 = t2 + i d
    float2 md = inv ? mul_pi(d) : mul_mi(d);
    v[0] = cadd(a, t1);
    v[1] = cadd(t2, md);
    v[2] = csub(t2, md);
  } else if constexpr (R == 4) {
    float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    float2 t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
    float2 r3 = inv ? mul_pi(t3) : mul_mi(t3);
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, r3);
    v[3] = csub(t1, r3);
  } else if constexpr (R == 8) {
    const float r2 = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft<4>(e, inv);
    dft<4>(o, inv);
    // W8^k (forward: exp(-2 pi i k / 8)), conjugated for the inverse
    float s = inv ? 1.f : -1.f;
    float2 o1 = cmul(o[1], make_float2(r2, s * r2));
    float2 o2 = inv ? mul_pi(o[2]) : mul_mi(o[2]);
    float2 o3 = cmul(o[3], make_float2(-r2, s * r2));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
}

template <int R>
__device__ __forceinline__ void fft_stage(const float2 *__restrict__ in, float2 *__restrict__ out, int L, int Ns,
                                          int nb, int es, int bs, const float2 *__restrict__ tw, int twmul,
                                          bool inv, int tid, int nt) {
  const int nbf = L / R;
  const int total = nb * nbf;
  const int tstride = (L / (Ns * R)) * twmul;
  for (int idx = tid; idx < total; idx += nt) {
    int b, j;
    if (es == 1) {
      b = idx / nbf;
      j = idx - b * nbf;
    } else {
      j = idx / nb;
      b = idx - j * nb;
    }
    const float2 *src = in + (size_t)b * bs;
    float2 *dst = out + (size_t)b * bs;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[(j + r * nbf) * es];
    const int k = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 t = tw[r * k * tstride];
        if (inv) t.y = -t.y;
        v[r] = cmul(v[r], t);
      }
    }
    dft<R>(v, inv);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[(base + r * Ns) * es] = v[r];
  }
}

// Runs all stages; returns the buffer holding the result (a or b).
__device__ __forceinline__ float2 *fft_smem(const FftShape &sh, float2 *a, float2 *b, int nb, int es, int bs,
                                            const float2 *tw, int twmul, bool inv) {
  const int tid = threadIdx.x, nt = blockDim.x;
  int Ns = 1;
  float2 *in = a, *out = b;
  for (int s = 0; s < sh.nstages; ++s) {
    const int R = sh.radix[s];
    switch (R) {
      case 2: fft_stage<2>(in, out, sh.L, Ns, nb, es, bs, tw, twmul, inv, tid, nt); break;
      case 3: fft_stage<3>(in, out, sh.L, Ns, nb, es, bs, tw, twmul, inv, tid, nt); break;
      case 4: fft_stage<4>(in, out, sh.L, Ns, nb, es, bs, tw, twmul, inv, tid, nt); break;
      default: fft_stage<8>(in, out, sh.L, Ns, nb, es, bs, tw, twmul, inv, tid, nt); break;
    }
    __syncthreads();
    Ns *= R;
    float2 *t = in;
    in = out;
    out = t;
  }
  return in;
}

}  // namespace augur
