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

#include <map>
#include <mutex>
#include <utility>

#include "../../include/augur_pm.h"

#define AUGUR_ERRBIT_NONFINITE 1u
#define AUGUR_ERRBIT_RANGE 2u
#define AUGUR_ERRBIT_TIMEOUT 4u

namespace augur {

// ---------------------------------------------------------------------------------
// host helpers shared by every translation unit
// ---------------------------------------------------------------------------------
// Opts `kernel` in to `bytes` of dynamic shared memory on the current device. The opt-in is a
// per-device property of the kernel shared by every caller in the process, so it is recorded per
// (device, kernel) under a lock and only ever raised.
inline int raise_dyn_smem(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AUGUR_ECUDA;
  std::lock_guard<std::mutex> lock(mu);
  size_t &cur = done[{dev, kernel}];
  if (bytes <= cur) return AUGUR_OK;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return AUGUR_ECUDA;
  }
  cur = bytes;
  return AUGUR_OK;
}

// Streaming multiprocessors of the current device (152 on GB300 if the query fails).
inline int current_sm_count() {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) {
    cudaGetLastError();
    return 152;
  }
  return nsm;
}

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
__device__ __forceinline__ bool cic_axis(float x, float half_ext, float h, int &i0, float &w, float inv_h = 0.f) {
  float t = __fadd_rn(x, half_ext);
  // when h is a power of two, t / h == t * (1/h) exactly, so the multiply is bit-identical
  float u = __fsub_rn(inv_h != 0.f ? __fmul_rn(t, inv_h) : __fdiv_rn(t, h), 0.5f);
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

// cic_axis with the division resolved at compile time: POW2 when h is a power of two (then
// t * (1/h) == t / h exactly), for loops that take the branch once outside
template <bool POW2>
__device__ __forceinline__ bool cic_axis_t(float x, float half_ext, float h, float inv_h, int &i0, float &w) {
  const float t = __fadd_rn(x, half_ext);
  const float u = __fsub_rn(POW2 ? __fmul_rn(t, inv_h) : __fdiv_rn(t, h), 0.5f);
  if (!(fabsf(u) < 1.0e9f)) {
    i0 = 0;
    w = 0.f;
    return false;
  }
  const float f = floorf(u);
  i0 = (int)f;
  w = __fsub_rn(u, f);
  return true;
}

// GELU x Phi(x) with erfc from Abramowitz & Stegun, Handbook of Mathematical Functions, eq. 7.1.26
// (|erf error| <= 1.5e-7): erfc(z) ~ t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-z^2),
// t = 1 / (1 + p z), z = |x| / sqrt 2 >= 0, and 2 - erfc(z) for the other sign, so negative inputs
// keep their relative accuracy. About half the instructions of the erff form.
__device__ __forceinline__ float as_erfc_exp(float x, float &ez2) {
  const float z = fabsf(x) * 0.70710678118654752440f;
  const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
  const float poly =
      t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 1.061405429f, -1.453152027f), 1.421413741f), -0.284496736f), 0.254829592f);
  ez2 = __expf(-z * z);  // exp(-x^2 / 2)
  return poly * ez2;      // erfc(|x| / sqrt 2)
}
__device__ __forceinline__ float gelu_as(float x) {
  float e;
  const float ec = as_erfc_exp(x, e);
  return 0.5f * x * (x >= 0.f ? 2.0f - ec : ec);
}
// d/dx [x Phi(x)] = Phi(x) + x phi(x), phi(x) = exp(-x^2/2) / sqrt(2 pi) (the same exponential)
__device__ __forceinline__ float gelu_grad_as(float x) {
  float e;
  const float ec = as_erfc_exp(x, e);
  return 0.5f * (x >= 0.f ? 2.0f - ec : ec) + x * (0.39894228040143267794f * e);
}

__device__ __forceinline__ int wrap_idx(int i, int G) {
  int r = i % G;
  return r < 0 ? r + G : r;
}

// wrap into [0, G): the common in-box cases without a division
__device__ __forceinline__ int fwrap(int i, int G) {
  if ((unsigned)i < (unsigned)G) return i;
  if (i == -1) return G - 1;
  if (i == G) return 0;
  return wrap_idx(i, G);
}

// Division by a runtime-invariant divisor for dividends < 2^31 (Granlund & Montgomery,
// PLDI 1994): q = umulhi(n, mul) >> shr with mul = ceil(2^(31+l) / d), l = ceil(log2 d).
struct FastDiv {
  uint32_t d, mul, shr;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) {
    f.mul = 0;
    f.shr = 0;
    return f;
  }
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  uint64_t p = 31 + l;
  f.mul = (uint32_t)(((1ull << p) + d - 1) / d);
  f.shr = (uint32_t)(p - 32);
  return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  return f.mul ? (__umulhi(n, f.mul) >> f.shr) : n;
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

// Row-mode shared-memory layout of the stages between the first load and the last store:
// element e of a row sits at fft_pad(e) = e + e/16, so the stride-R stores of a radix-R
// stage (R = 16: every thread of a row on the same bank) spread over the banks. A row
// needs fft_row_stride(L) float2 (odd count past the padding, so rows start on different
// banks too).
__host__ __device__ constexpr int fft_pad(int e) { return e + (e >> 4); }
__host__ __device__ constexpr int fft_row_stride(int L) { return L + (L >> 4) + 1; }

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
  } else if constexpr (R == 16) {
    // 16 = 4 x 4: DFT4 over n1 of x[4 n1 + n2], twiddle W16^(n2 k1), DFT4 over n2
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, r2 = 0.70710678118654752440f;
    const float sg = inv ? 1.f : -1.f;
    float2 y[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      float2 t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
      dft<4>(t, inv);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = t[k1];
    }
    // twiddles W16^m, m = n2 * k1 (forward: exp(-2 pi i m / 16))
    y[1][1] = cmul(y[1][1], make_float2(c1, sg * s1));
    y[1][2] = cmul(y[1][2], make_float2(r2, sg * r2));
    y[1][3] = cmul(y[1][3], make_float2(s1, sg * c1));
    y[2][1] = cmul(y[2][1], make_float2(r2, sg * r2));
    y[2][2] = inv ? mul_pi(y[2][2]) : mul_mi(y[2][2]);
    y[2][3] = cmul(y[2][3], make_float2(-r2, sg * r2));
    y[3][1] = cmul(y[3][1], make_float2(s1, sg * c1));
    y[3][2] = cmul(y[3][2], make_float2(-r2, sg * r2));
    y[3][3] = cmul(y[3][3], make_float2(-c1, -sg * s1));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      float2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
      dft<4>(t, inv);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
    }
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

// ---------------------------------------------------------------------------------
// Compile-time FFT: Stockham stages with the length (and, for column transforms, the
// number of interleaved columns) as template parameters so that every index division
// folds to shifts and multiplies. Radix order: 3s first, then 16s, then one 8, 4 or 2;
// a radix-16 butterfly is done in registers as 4 x 4, so 128- and 256-point transforms
// take two shared-memory passes.
// ---------------------------------------------------------------------------------
constexpr int fft_radix(int L, int s) {
  int r[16] = {};
  int n = 0, x = L;
  while (x % 3 == 0) {
    r[n++] = 3;
    x /= 3;
  }
  while (x % 16 == 0) {
    r[n++] = 16;
    x /= 16;
  }
  if (x == 8 || x == 4 || x == 2) r[n++] = x;
  return (s < n) ? r[s] : 0;
}
constexpr int fft_nstages(int L) {
  int n = 0;
  while (fft_radix(L, n)) ++n;
  return n;
}
constexpr int fft_ns(int L, int s) {
  int ns = 1;
  for (int i = 0; i < s; ++i) ns *= fft_radix(L, i);
  return ns;
}

// ---------------------------------------------------------------------------------
// Transform with caller-supplied first load and last store: stage 0 reads element e of
// transform b through ld(b, e), the last stage writes through st(b, e, value), and the
// stages in between ping-pong through shared memory (bufA, bufB; row stride bs in row
// mode, column-interleaved in column mode). A two-stage length (128, 256, ...) touches
// shared memory once. Ends with __syncthreads().
// COLS == 0: nb transforms, thread index maps to (b slow, j fast).
// COLS > 0 : COLS transforms, thread index maps to (j slow, b fast), smem buf[e*COLS + b].
// ---------------------------------------------------------------------------------
template <int R, int L, int NS, int COLS, class LD, class ST>
__device__ __forceinline__ void fft_stage_io(int nb, LD &ld, ST &st, const float2 *__restrict__ tw, int twmul,
                                             bool inv) {
  constexpr int nbf = L / R;
  constexpr int tstride = L / (NS * R);
  const int total = (COLS > 0 ? COLS : nb) * nbf;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int b, j;
    if constexpr (COLS > 0) {
      j = idx / COLS;
      b = idx - j * COLS;
    } else {
      b = idx / nbf;
      j = idx - b * nbf;
    }
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = ld(b, j + r * nbf);
    const int k = j % NS;
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 t = tw[r * k * tstride * twmul];
        if (inv) t.y = -t.y;
        v[r] = cmul(v[r], t);
      }
    }
    dft<R>(v, inv);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) st(b, base + r * NS, v[r]);
  }
}

template <int L, int COLS, int S, class LD, class ST>
__device__ __forceinline__ void fft_io_rec(int nb, LD &ld, ST &st, float2 *in, float2 *out, int bs,
                                           const float2 *tw, int twmul, bool inv) {
  constexpr int NSTG = fft_nstages(L);
  constexpr int R = fft_radix(L, S);
  constexpr int NS = fft_ns(L, S);
  auto sld = [&](int b, int e) -> float2 { return COLS > 0 ? in[e * COLS + b] : in[b * bs + fft_pad(e)]; };
  auto sst = [&](int b, int e, float2 v) {
    if (COLS > 0) out[e * COLS + b] = v;
    else out[b * bs + fft_pad(e)] = v;
  };
  if constexpr (NSTG == 1) {
    fft_stage_io<R, L, NS, COLS>(nb, ld, st, tw, twmul, inv);
    __syncthreads();
  } else if constexpr (S == 0) {
    fft_stage_io<R, L, NS, COLS>(nb, ld, sst, tw, twmul, inv);
    __syncthreads();
    fft_io_rec<L, COLS, S + 1>(nb, ld, st, out, in, bs, tw, twmul, inv);
  } else if constexpr (S == NSTG - 1) {
    fft_stage_io<R, L, NS, COLS>(nb, sld, st, tw, twmul, inv);
    __syncthreads();
  } else {
    fft_stage_io<R, L, NS, COLS>(nb, sld, sst, tw, twmul, inv);
    __syncthreads();
    fft_io_rec<L, COLS, S + 1>(nb, ld, st, out, in, bs, tw, twmul, inv);
  }
}

template <int L, int COLS, class LD, class ST>
__device__ __forceinline__ void fft_io(int nb, LD ld, ST st, float2 *bufA, float2 *bufB, int bs, const float2 *tw,
                                       int twmul, bool inv) {
  fft_io_rec<L, COLS, 0>(nb, ld, st, bufA, bufB, bs, tw, twmul, inv);
}

#define AUGUR_FFT_LENGTHS(X) \
  X(8) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(1536) X(2048)

// Calls fft_io<N, COLS>(args...) for the runtime length L (one of AUGUR_FFT_LENGTHS).
#define AUGUR_FFT_IO(L, COLS, ...)                         \
  switch (L) {                                            \
    case 8: fft_io<8, COLS>(__VA_ARGS__); break;          \
    case 16: fft_io<16, COLS>(__VA_ARGS__); break;        \
    case 24: fft_io<24, COLS>(__VA_ARGS__); break;        \
    case 32: fft_io<32, COLS>(__VA_ARGS__); break;        \
    case 48: fft_io<48, COLS>(__VA_ARGS__); break;        \
    case 64: fft_io<64, COLS>(__VA_ARGS__); break;        \
    case 96: fft_io<96, COLS>(__VA_ARGS__); break;        \
    case 128: fft_io<128, COLS>(__VA_ARGS__); break;      \
    case 192: fft_io<192, COLS>(__VA_ARGS__); break;      \
    case 256: fft_io<256, COLS>(__VA_ARGS__); break;      \
    case 384: fft_io<384, COLS>(__VA_ARGS__); break;      \
    case 512: fft_io<512, COLS>(__VA_ARGS__); break;      \
    case 768: fft_io<768, COLS>(__VA_ARGS__); break;      \
    case 1024: fft_io<1024, COLS>(__VA_ARGS__); break;    \
    case 1536: fft_io<1536, COLS>(__VA_ARGS__); break;    \
    case 2048: fft_io<2048, COLS>(__VA_ARGS__); break;    \
    default: break;                                       \
  }

inline bool fft_length_supported(int L) {
  switch (L) {
#define AUGUR_CASE(N) \
  case N: return true;
    AUGUR_FFT_LENGTHS(AUGUR_CASE)
#undef AUGUR_CASE
    default: return false;
  }
}

}  // namespace augur
