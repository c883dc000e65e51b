// ps_common.cuh -- shared device code of the GB300 P_l(k) path: fixed-point
// mesh format, the in-shared-memory mixed-radix FFT engine, and the per-mode
// geometry (bin lookup, window, Legendre) used by the binning sweeps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "powspec_gpu.h"

namespace ps {

// ---------------------------------------------------------------- limits
constexpr int kMaxPole = 7;        // ell = 0..6 (src/define.h:96)
constexpr int kMaxPlan = 24;       // radix passes per transform length
constexpr int kFftThreads = 256;   // threads of every FFT-pass CTA
constexpr int kElemsPerThread = 32;  // complex values a thread stages per pass
constexpr int kCtaElems = kFftThreads * kElemsPerThread;  // 8192 complex = 64 KB
constexpr int kPipeElems = 4096;  // complex values per tile of the pipelined z/y passes
constexpr int kPassCElems = 4096;  // complex per ping-pong buffer of the binning pass

// Fixed-point mesh: every stencil node adds llrint(w_node * 2^32) to an int64
// cell with an integer atomic.  Integer addition is associative, so the mesh
// is bit-identical whatever the order of the atomics.
constexpr float kFixScale = 4294967296.0f;         // 2^32
constexpr double kFixInv = 2.3283064365386963e-10;  // 2^-32
constexpr double kFixMaxWeight = 2147483648.0;      // |cell| < 2^31 weight units

// Radix plan of one transform length (product of 8, 4, 2, 3, 5).
struct FftPlan {
  int n;
  int npass;
  int radix[kMaxPlan];
  int logn;  // log2(n) when n is a power of two, else -1
};

// --------------------------------------------------------------- complex
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
// a * (-i)
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }

// ------------------------------------------------- forward DFT butterflies
// out[q] = sum_r v[r] exp(-2 pi i r q / R), natural order, in place.
template <int R>
__device__ __forceinline__ void dft(float2 (&v)[R]);

template <>
__device__ __forceinline__ void dft<2>(float2 (&v)[2]) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<4>(float2 (&v)[4]) {
  float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]), t3 = cmul_mi(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <>
__device__ __forceinline__ void dft<8>(float2 (&v)[8]) {
  const float h = 0.70710678118654752440f;  // sqrt(1/2)
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft<4>(e);
  dft<4>(o);
  // twiddles W8^q, q = 0..3: 1, h(1-i), -i, -h(1+i)
  float2 o1 = make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
  float2 o2 = cmul_mi(o[2]);
  float2 o3 = make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], o1);
  v[5] = csub(e[1], o1);
  v[2] = cadd(e[2], o2);
  v[6] = csub(e[2], o2);
  v[3] = cadd(e[3], o3);
  v[7] = csub(e[3], o3);
}

template <>
__device__ __forceinline__ void dft<3>(float2 (&v)[3]) {
  const float h = 0.86602540378443864676f;  // sqrt(3)/2
  float2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  float2 a = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
  // -i h d = (h d.y, -h d.x)
  float2 t = make_float2(h * d.y, -h * d.x);
  v[0] = cadd(v[0], s);
  v[1] = cadd(a, t);
  v[2] = csub(a, t);
}

template <>
__device__ __forceinline__ void dft<5>(float2 (&v)[5]) {
  const float c1 = 0.30901699437494742410f;   // cos(2pi/5)
  const float c2 = -0.80901699437494742410f;  // cos(4pi/5)
  const float s1 = 0.95105651629515357212f;   // sin(2pi/5)
  const float s2 = 0.58778525229247312917f;   // sin(4pi/5)
  float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
  float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
  float2 x0 = v[0];
  float2 r1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
  float2 r2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
  // i1 = s1 b1 + s2 b2 ; i2 = s2 b1 - s1 b2 ; out = r -/+ i * i_
  float2 i1 = make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
  float2 i2 = make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
  v[0] = make_float2(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
  v[1] = cadd(r1, cmul_mi(i1));
  v[4] = csub(r1, cmul_mi(i1));
  v[2] = cadd(r2, cmul_mi(i2));
  v[3] = csub(r2, cmul_mi(i2));
}

// x * exp(-2 pi i e / 32) for a compile-time e (folds to constants).
__device__ __forceinline__ float2 rot32(float2 x, int e) {
  e &= 31;
  if (e == 0) return x;
  if (e == 8) return make_float2(x.y, -x.x);
  if (e == 16) return make_float2(-x.x, -x.y);
  if (e == 24) return make_float2(-x.y, x.x);
  // cos, sin of 2 pi r / 32, r = 0..7
  const float C[8] = {1.000000000f, 0.980785280f, 0.923879533f, 0.831469612f,
                      0.707106781f, 0.555570233f, 0.382683432f, 0.195090322f};
  const float S[8] = {0.000000000f, 0.195090322f, 0.382683432f, 0.555570233f,
                      0.707106781f, 0.831469612f, 0.923879533f, 0.980785280f};
  const int q = e >> 3, r = e & 7;
  // rotate by exp(-i 2 pi r / 32) first, then by (-i)^q
  float2 y = make_float2(x.x * C[r] + x.y * S[r], x.y * C[r] - x.x * S[r]);
  if (q == 1) y = make_float2(y.y, -y.x);
  else if (q == 2) y = make_float2(-y.x, -y.y);
  else if (q == 3) y = make_float2(-y.y, y.x);
  return y;
}

// 16-point DFT as 4 x 4 (input n = 4 n1 + n2, output k = k1 + 4 k2).
template <>
__device__ __forceinline__ void dft<16>(float2 (&x)[16]) {
  float2 y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) {
    float2 t[4] = {x[n2], x[4 + n2], x[8 + n2], x[12 + n2]};
    dft<4>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) y[n2][k1] = rot32(t[k1], 2 * n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft<4>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) x[k1 + 4 * k2] = t[k2];
  }
}

// 32-point DFT as 4 x 8 (input n = 8 n1 + n2, output k = k1 + 4 k2).
template <>
__device__ __forceinline__ void dft<32>(float2 (&x)[32]) {
  float2 y[8][4];
#pragma unroll
  for (int n2 = 0; n2 < 8; n2++) {
    float2 t[4] = {x[n2], x[8 + n2], x[16 + n2], x[24 + n2]};
    dft<4>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) y[n2][k1] = rot32(t[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 t[8] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1],
                   y[4][k1], y[5][k1], y[6][k1], y[7][k1]};
    dft<8>(t);
#pragma unroll
    for (int k2 = 0; k2 < 8; k2++) x[k1 + 4 * k2] = t[k2];
  }
}

// Twiddle load that the compiler may not hoist out of a persistent tile
// loop (hoisting 31 loop-invariant twiddles would pin 62 registers).
__device__ __forceinline__ float2 ldtw(const float2* p) {
  float2 v;
  asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}

// ---------------------------------------------------- power-of-two engine
// Lines of n = 2^logn complex in shared memory use a padded layout: element
// e of a line sits at e + e/32, so the stride-32 writes of a radix-32 pass
// fall in distinct banks.  Radix-32 passes run first (no twiddles in the
// first, conflict-free strides in all), then one remainder pass of radix
// 2, 4, 8 or 16.  All index arithmetic is shifts and masks.
__device__ __forceinline__ int pidx(int e) { return e + (e >> 5); }

// Element e of a line in either layout.
template <bool PAD>
__device__ __forceinline__ int lidx(int e) { return PAD ? e + (e >> 5) : e; }

// Line stride (complex) of lines holding `slots` elements: odd, so that
// reading one element from each of 16 consecutive lines is conflict-free.
__host__ __device__ inline int line_stride(int slots, bool pad) {
  int s = pad ? (slots - 1) + ((slots - 1) >> 5) + 1 : slots;
  return (s & 1) ? s : s + 1;
}

// In place: every thread stages 32 complex values (one radix-32 butterfly,
// or 32/R smaller ones), the block synchronises, then stores.
// Requires nlines << logn <= kCtaElems.
template <int R, int LOGR>
__device__ __forceinline__ void fft2_pass(float2* buf, int logn, int nlines, int ls, int logNs,
                                          const float2* __restrict__ tw, int tid = threadIdx.x) {
  constexpr int BPT = 32 / R;
  const int logm = logn - LOGR;
  const int mmask = (1 << logm) - 1, nsmask = (1 << logNs) - 1;
  const int total = nlines << logm;
  const int tws = logn - logNs - LOGR;
  float2 v[BPT][R];
#pragma unroll
  for (int t = 0; t < BPT; t++) {
    const int b = tid + t * blockDim.x;
    if (b < total) {
      const int line = b >> logm, j = b & mmask, k = j & nsmask;
      const float2* src = buf + line * ls;
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int e = j + (r << logm);
        float2 x = src[pidx(e)];
        if (r > 0 && k > 0) x = cmul(x, ldtw(&tw[(r * k) << tws]));
        v[t][r] = x;
      }
      dft<R>(v[t]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < BPT; t++) {
    const int b = tid + t * blockDim.x;
    if (b < total) {
      const int line = b >> logm, j = b & mmask, k = j & nsmask;
      float2* dst = buf + line * ls;
      const int e0 = ((j >> logNs) << (logNs + LOGR)) + k;
#pragma unroll
      for (int r = 0; r < R; r++) dst[pidx(e0 + (r << logNs))] = v[t][r];
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void fft2_lines(float2* buf, int logn, int nlines, int ls,
                                           const float2* __restrict__ tw) {
  int logNs = 0;
  for (; logn - logNs >= 5; logNs += 5) fft2_pass<32, 5>(buf, logn, nlines, ls, logNs, tw);
  switch (logn - logNs) {
    case 4: fft2_pass<16, 4>(buf, logn, nlines, ls, logNs, tw); break;
    case 3: fft2_pass<8, 3>(buf, logn, nlines, ls, logNs, tw); break;
    case 2: fft2_pass<4, 2>(buf, logn, nlines, ls, logNs, tw); break;
    case 1: fft2_pass<2, 1>(buf, logn, nlines, ls, logNs, tw); break;
    default: break;
  }
}

// Ping-pong variant (one butterfly in registers at a time) for persistent
// kernels that loop over tiles.  Returns the buffer holding the result.
template <int R, int LOGR>
__device__ __forceinline__ void fft2_pass_pp(const float2* src, float2* dst, int logn,
                                             int nlines, int ls, int logNs,
                                             const float2* __restrict__ tw, int tid = threadIdx.x) {
  const int logm = logn - LOGR;
  const int mmask = (1 << logm) - 1, nsmask = (1 << logNs) - 1;
  const int total = nlines << logm;
  const int tws = logn - logNs - LOGR;
  for (int b = tid; b < total; b += blockDim.x) {
    const int line = b >> logm, j = b & mmask, k = j & nsmask;
    const float2* s = src + line * ls;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      float2 x = s[pidx(j + (r << logm))];
      if (r > 0 && k > 0) x = cmul(x, ldtw(&tw[(r * k) << tws]));
      v[r] = x;
    }
    dft<R>(v);
    float2* d = dst + line * ls;
    const int e0 = ((j >> logNs) << (logNs + LOGR)) + k;
#pragma unroll
    for (int r = 0; r < R; r++) d[pidx(e0 + (r << logNs))] = v[r];
  }
  __syncthreads();
}

// MAXLOG = 5: radix-32 passes; MAXLOG = 4: radix-16 passes (twice the
// butterflies per pass, for tiles too small to occupy every thread).
template <int MAXLOG = 5>
__device__ __forceinline__ float2* fft2_lines_pp(float2* a, float2* b, int logn, int nlines,
                                                 int ls, const float2* __restrict__ tw) {
  int logNs = 0;
  for (; logn - logNs >= MAXLOG; logNs += MAXLOG) {
    if (MAXLOG == 5) fft2_pass_pp<32, 5>(a, b, logn, nlines, ls, logNs, tw);
    else fft2_pass_pp<16, 4>(a, b, logn, nlines, ls, logNs, tw);
    float2* t = a; a = b; b = t;
  }
  const int rem = logn - logNs;
  if (rem) {
    switch (rem) {
      case 4: fft2_pass_pp<16, 4>(a, b, logn, nlines, ls, logNs, tw); break;
      case 3: fft2_pass_pp<8, 3>(a, b, logn, nlines, ls, logNs, tw); break;
      case 2: fft2_pass_pp<4, 2>(a, b, logn, nlines, ls, logNs, tw); break;
      default: fft2_pass_pp<2, 1>(a, b, logn, nlines, ls, logNs, tw); break;
    }
    float2* t = a; a = b; b = t;
  }
  return a;
}

// One Stockham radix-R pass over `nlines` lines of length n held in shared
// memory (line stride ls complex), in place: every thread first stages the
// inputs of its butterflies in registers, the block synchronises, then the
// outputs go to their autosorted positions.  tw[m] = exp(-2 pi i m / n).
// Requires nlines * n <= kCtaElems (checked on the host).
template <int R>
__device__ __forceinline__ void fft_pass(float2* buf, int n, int nlines, int ls,
                                         int Ns, const float2* __restrict__ tw) {
  constexpr int BPT = (kElemsPerThread + R - 1) / R;
  const int m = n / R;
  const int total = nlines * m;
  const int tws = n / (Ns * R);
  float2 v[BPT][R];
#pragma unroll
  for (int t = 0; t < BPT; t++) {
    const int b = threadIdx.x + t * blockDim.x;
    if (b < total) {
      const int line = b / m;
      const int j = b - line * m;
      const int k = j % Ns;
      const float2* src = buf + line * ls;
#pragma unroll
      for (int r = 0; r < R; r++) {
        float2 x = src[j + r * m];
        if (r > 0 && k > 0) x = cmul(x, __ldg(&tw[r * k * tws]));
        v[t][r] = x;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < BPT; t++) {
    const int b = threadIdx.x + t * blockDim.x;
    if (b < total) {
      const int line = b / m;
      const int j = b - line * m;
      const int k = j % Ns;
      dft<R>(v[t]);
      float2* dst = buf + line * ls + (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) dst[r * Ns] = v[t][r];
    }
  }
  __syncthreads();
}

// Full forward transform of every line in shared memory.  The plan lists
// its passes grouped by radix (8s, 4s, 2s, 3s, 5s; any order of the factors
// is a valid Stockham sequence); one loop per radix keeps every inlined
// butterfly body in its own region, which the register allocator handles
// far better than a switch inside a single loop.
__device__ __forceinline__ void fft_lines(float2* buf, const FftPlan& plan, int nlines,
                                          int ls, const float2* __restrict__ tw) {
  int Ns = 1, p = 0;
  const int np = plan.npass;
  for (; p < np && plan.radix[p] == 8; p++, Ns *= 8) fft_pass<8>(buf, plan.n, nlines, ls, Ns, tw);
  for (; p < np && plan.radix[p] == 4; p++, Ns *= 4) fft_pass<4>(buf, plan.n, nlines, ls, Ns, tw);
  for (; p < np && plan.radix[p] == 2; p++, Ns *= 2) fft_pass<2>(buf, plan.n, nlines, ls, Ns, tw);
  for (; p < np && plan.radix[p] == 3; p++, Ns *= 3) fft_pass<3>(buf, plan.n, nlines, ls, Ns, tw);
  for (; p < np && plan.radix[p] == 5; p++, Ns *= 5) fft_pass<5>(buf, plan.n, nlines, ls, Ns, tw);
}

// Ping-pong variant for kernels that transform many tiles in a loop: every
// butterfly goes from buffer `src` to buffer `dst` with only its R inputs in
// registers, so register use stays that of a single butterfly however many
// passes are inlined.  Returns the buffer holding the result.
template <int R>
__device__ __forceinline__ void fft_pass_pp(const float2* src, float2* dst, int n, int nlines,
                                            int ls, int Ns, const float2* __restrict__ tw) {
  const int m = n / R;
  const int total = nlines * m;
  const int tws = n / (Ns * R);
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / m;
    const int j = b - line * m;
    const int k = j % Ns;
    const float2* s = src + line * ls + j;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      float2 x = s[r * m];
      if (r > 0 && k > 0) x = cmul(x, __ldg(&tw[r * k * tws]));
      v[r] = x;
    }
    dft<R>(v);
    float2* d = dst + line * ls + (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) d[r * Ns] = v[r];
  }
  __syncthreads();
}

__device__ __forceinline__ float2* fft_lines_pp(float2* a, float2* b, const FftPlan& plan,
                                                int nlines, int ls,
                                                const float2* __restrict__ tw) {
  int Ns = 1, p = 0;
  const int np = plan.npass;
  for (; p < np && plan.radix[p] == 8; p++, Ns *= 8) {
    fft_pass_pp<8>(a, b, plan.n, nlines, ls, Ns, tw);
    float2* t = a; a = b; b = t;
  }
  for (; p < np && plan.radix[p] == 4; p++, Ns *= 4) {
    fft_pass_pp<4>(a, b, plan.n, nlines, ls, Ns, tw);
    float2* t = a; a = b; b = t;
  }
  for (; p < np && plan.radix[p] == 2; p++, Ns *= 2) {
    fft_pass_pp<2>(a, b, plan.n, nlines, ls, Ns, tw);
    float2* t = a; a = b; b = t;
  }
  for (; p < np && plan.radix[p] == 3; p++, Ns *= 3) {
    fft_pass_pp<3>(a, b, plan.n, nlines, ls, Ns, tw);
    float2* t = a; a = b; b = t;
  }
  for (; p < np && plan.radix[p] == 5; p++, Ns *= 5) {
    fft_pass_pp<5>(a, b, plan.n, nlines, ls, Ns, tw);
    float2* t = a; a = b; b = t;
  }
  return a;
}

// s += a + b as an unevaluated FP32 pair (hi, lo), renormalised after
// each add: TwoSum of hi and a (exact), the low parts added, then hi + lo
// recombined (Fast2Sum).  Each add loses about 2^-48 of the running sum.
__device__ __forceinline__ void df_add(float& hi, float& lo, float a, float b) {
  const float t = hi + a, bp = t - hi;
  const float err = (hi - (t - bp)) + (a - bp);
  const float l = lo + err + b;
  hi = t + l;
  lo = l - (hi - t);
}

// Fixed-point cell (minus a constant offset) -> float.  d = hi * 2^32 + lo,
// value = d * 2^-32 = hi + lo * 2^-32, using two 32-bit conversions.
__device__ __forceinline__ float fix_to_float(long long d) {
  const int hi = (int)(d >> 32);
  const unsigned lo = (unsigned)(d & 0xffffffffull);
  return (float)hi + (float)lo * 2.3283064365386963e-10f;
}


// ------------------------------------------------ async bulk copies (TMA)
// One-dimensional cp.async.bulk global -> shared with mbarrier completion.
// Addresses and sizes must be multiples of 16 bytes.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` polls (each poll may suspend the
// thread for a hardware-defined time) and reports failure.
constexpr long long kWaitLimit = 1ll << 24;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          long long limit = kWaitLimit) {
  for (long long i = 0; i < limit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// A pass's poll limit: its own (> 0, set by the stall test hook) or the default.
__device__ __forceinline__ long long wait_limit(int lim) { return lim > 0 ? lim : kWaitLimit; }

// Wait for stage it & 1 of a two-stage pipeline (all threads).  On timeout:
// sets bit 1 of *err and the block's abort flag; returns false once aborted.
__device__ __forceinline__ bool pipe_wait(uint64_t* bar, int it, int* err, int* s_abort,
                                          long long limit = kWaitLimit) {
  if (!mbar_wait(&bar[it & 1], (uint32_t)((it >> 1) & 1), limit)) {
    atomicOr(err, 2);
    *s_abort = 1;
  }
  __syncthreads();
  return *s_abort == 0;
}

// Abort drain of a two-stage pipeline, by the thread that issued every copy:
// `issued` copies went out, copy j on stage j & 1, where it completes that
// stage's phase j >> 1.  Only the last two can still be in flight; wait
// (bounded) for exactly their phases, so that the CTA never exits with a
// bulk copy landing in its shared memory.  An older phase's parity would
// not do: a wait on a phase that completed earlier returns at once.
__device__ __forceinline__ void pipe_drain(uint64_t* bar, int issued, long long limit = kWaitLimit) {
  for (int j = issued >= 2 ? issued - 2 : 0; j < issued; j++)
    mbar_wait(&bar[j & 1], (uint32_t)((j >> 1) & 1), limit);
}

// First radix pass of a pipelined transform: reads lines of n = 2^logn
// from an unpadded staging buffer (line stride sstride), writes the padded
// FFT buffer (line stride ls).
template <int R, int LOGR>
__device__ __forceinline__ void fft2_first_pass(const float2* src, int sstride, float2* dst,
                                                int logn, int nlines, int ls,
                                                int tid = threadIdx.x) {
  const int logm = logn - LOGR;
  const int mmask = (1 << logm) - 1;
  const int total = nlines << logm;
  for (int b = tid; b < total; b += blockDim.x) {
    const int line = b >> logm, j = b & mmask;
    const float2* s = src + line * sstride + j;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = s[r << logm];
    dft<R>(v);
    float2* d = dst + line * ls;
#pragma unroll
    for (int r = 0; r < R; r++) d[pidx(j * R + r)] = v[r];
  }
  __syncthreads();
}

// Same, for a first pass that reads fixed-point int64 cells (two per
// complex input value) and subtracts a constant offset while converting.
template <int R, int LOGR>
__device__ __forceinline__ void fft2_first_pass_fix(const long long* src, int sstride,
                                                    long long off, float2* dst, int logn,
                                                    int nlines, int ls, int tid = threadIdx.x) {
  const int logm = logn - LOGR;
  const int mmask = (1 << logm) - 1;
  const int total = nlines << logm;
  for (int b = tid; b < total; b += blockDim.x) {
    const int line = b >> logm, j = b & mmask;
    const longlong2* s = reinterpret_cast<const longlong2*>(src + (size_t)line * sstride) + j;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const longlong2 q = s[r << logm];
      v[r] = make_float2(fix_to_float(q.x - off), fix_to_float(q.y - off));
    }
    dft<R>(v);
    float2* d = dst + line * ls;
#pragma unroll
    for (int r = 0; r < R; r++) d[pidx(j * R + r)] = v[r];
  }
  __syncthreads();
}

// Remaining in-place passes after a first pass of radix 2^first.
__device__ __forceinline__ void fft2_rest(float2* buf, int logn, int first, int nlines, int ls,
                                          const float2* __restrict__ tw, int tid = threadIdx.x) {
  int logNs = first;
  for (; logn - logNs >= 5; logNs += 5) fft2_pass<32, 5>(buf, logn, nlines, ls, logNs, tw, tid);
  switch (logn - logNs) {
    case 4: fft2_pass<16, 4>(buf, logn, nlines, ls, logNs, tw, tid); break;
    case 3: fft2_pass<8, 3>(buf, logn, nlines, ls, logNs, tw, tid); break;
    case 2: fft2_pass<4, 2>(buf, logn, nlines, ls, logNs, tw, tid); break;
    case 1: fft2_pass<2, 1>(buf, logn, nlines, ls, logNs, tw, tid); break;
    default: break;
  }
}

// Ping-pong transform of lines staged unpadded in `stage` (line stride
// sstride): first pass stage -> F, then F <-> stage (the stage buffer is
// free once the first pass has read it; it must hold nlines * ls complex).
// Returns the buffer holding the padded result.  `fix` != NULL: the staged
// lines are int64 fixed-point cells minus `off` (the first pass converts).
template <bool FIX, int MAXLOG = 5>
__device__ __forceinline__ float2* fft2_pp_from(void* stage, int sstride, long long off,
                                                float2* F, int logn, int nlines, int ls,
                                                const float2* __restrict__ tw) {
  static_assert(MAXLOG == 4 || MAXLOG == 5, "radix 16 or 32");
  int first;
  if (MAXLOG == 5 && logn >= 5) {
    if (FIX) fft2_first_pass_fix<32, 5>((const long long*)stage, sstride, off, F, logn, nlines, ls);
    else fft2_first_pass<32, 5>((const float2*)stage, sstride, F, logn, nlines, ls);
    first = 5;
  } else if (logn >= 4) {
    if (FIX) fft2_first_pass_fix<16, 4>((const long long*)stage, sstride, off, F, logn, nlines, ls);
    else fft2_first_pass<16, 4>((const float2*)stage, sstride, F, logn, nlines, ls);
    first = 4;
  } else {
    switch (logn) {
      case 3:
        if (FIX) fft2_first_pass_fix<8, 3>((const long long*)stage, sstride, off, F, logn, nlines, ls);
        else fft2_first_pass<8, 3>((const float2*)stage, sstride, F, logn, nlines, ls);
        break;
      case 2:
        if (FIX) fft2_first_pass_fix<4, 2>((const long long*)stage, sstride, off, F, logn, nlines, ls);
        else fft2_first_pass<4, 2>((const float2*)stage, sstride, F, logn, nlines, ls);
        break;
      default:
        if (FIX) fft2_first_pass_fix<2, 1>((const long long*)stage, sstride, off, F, logn, nlines, ls);
        else fft2_first_pass<2, 1>((const float2*)stage, sstride, F, logn, nlines, ls);
        break;
    }
    first = logn;
  }
  float2* a = F;
  float2* b = (float2*)stage;
  int logNs = first;
  for (; logn - logNs >= MAXLOG; logNs += MAXLOG) {
    if (MAXLOG == 5) fft2_pass_pp<32, 5>(a, b, logn, nlines, ls, logNs, tw);
    else fft2_pass_pp<16, 4>(a, b, logn, nlines, ls, logNs, tw);
    float2* t = a; a = b; b = t;
  }
  const int rem = logn - logNs;
  if (rem) {
    switch (rem) {
      case 4: fft2_pass_pp<16, 4>(a, b, logn, nlines, ls, logNs, tw); break;
      case 3: fft2_pass_pp<8, 3>(a, b, logn, nlines, ls, logNs, tw); break;
      case 2: fft2_pass_pp<4, 2>(a, b, logn, nlines, ls, logNs, tw); break;
      default: fft2_pass_pp<2, 1>(a, b, logn, nlines, ls, logNs, tw); break;
    }
    float2* t = a; a = b; b = t;
  }
  return a;
}

// The thread index as an opaque per-call value: index arithmetic derived
// from it cannot be hoisted out of a persistent tile loop (which would pin
// the 64 addresses of every inlined radix-32 pass in registers).
__device__ __forceinline__ int opaque_tid() {
  int t;
  asm volatile("mov.u32 %0, %%tid.x;" : "=r"(t));
  return t;
}

// Whole transform of lines staged unpadded in `src`, result padded in `dst`.
__device__ __forceinline__ void fft2_lines_from(const float2* src, int sstride, float2* dst,
                                                int logn, int nlines, int ls,
                                                const float2* __restrict__ tw) {
  if (logn >= 5) {
    fft2_first_pass<32, 5>(src, sstride, dst, logn, nlines, ls, opaque_tid());
    fft2_rest(dst, logn, 5, nlines, ls, tw, opaque_tid());
    return;
  }
  const int tid = opaque_tid();
  switch (logn) {
    case 4: fft2_first_pass<16, 4>(src, sstride, dst, logn, nlines, ls, tid); break;
    case 3: fft2_first_pass<8, 3>(src, sstride, dst, logn, nlines, ls, tid); break;
    case 2: fft2_first_pass<4, 2>(src, sstride, dst, logn, nlines, ls, tid); break;
    default: fft2_first_pass<2, 1>(src, sstride, dst, logn, nlines, ls, tid); break;
  }
}


// ---------------------------------------------------------- mode geometry
// Everything a binning sweep needs to turn a lattice vector into a bin,
// window factor and mu.  Tables are built on the host in FP64 (see the
// host code for their definitions).
struct ModeGeom {
  int ng;
  int nbin;
  int nmu;                   // |mu| sub-bins per k bin (1: plain P_l binning)
  int npole;
  int poles[kMaxPole];
  int logscale;
  int nmax;                  // n = i'^2 + j'^2 + k^2 <= nmax
  const short* bintab;       // [nmax+1]: bin, -1 out of range, -2 ambiguous; NULL: none
  const double* ksq;         // [3][ng/2+1]: fl(fl(vec_d * m)^2)
  const float* win;          // [3][ng]: window factor per signed index (FP64 -> FP32)
  const float2* phase;       // [3*ng]: exp(i pi (m - ng) / ng), m = i'+j'+k+ng
  double kedge0, kedgeN, dk;
  float vec[3];              // 2 pi / L per axis (FP32, for mu only)
  float los[3];
  // FP32 bin estimate (linear bins, cubic box): t = (|k| - k0) / dk from the
  // FP32 wave vector; trusted when farther than eps_t from a bin edge, else
  // the table and the exact path
  int fastbin;
  float k0f, inv_dkf, eps_t;
  // L_ell(mu) = [mu if ell odd] * (c0 + c1 mu^2 + c2 mu^4 + c3 mu^6) per pole
  float lc[kMaxPole][4];
  int lodd;                  // bit l: pole l is odd
};

// Bin of a mode with |i'| = ia, |j'| = ja, k = ka, n = ia^2+ja^2+ka^2.
// Unambiguous n come from the table; the rest run the reference's exact FP64
// sequence kmod = sqrt((ki^2 + kj^2) + kk^2), (int)((kmod - kedge0) / dk)
// (src/multipole.c:132-158, :593-605) with correctly rounded intrinsics.
__device__ __forceinline__ int mode_bin(const ModeGeom& g, int ia, int ja, int ka, int n) {
  if (g.bintab) {
    const int t = __ldg(&g.bintab[n]);
    if (t != -2) return t;
  }
  const int h = g.ng / 2 + 1;
  double km2 = __dadd_rn(__ldg(&g.ksq[ia]), __ldg(&g.ksq[h + ja]));
  if (ka) km2 = __dadd_rn(km2, __ldg(&g.ksq[2 * h + ka]));
  const double kmod = g.logscale ? 0.5 * log10(km2) : __dsqrt_rn(km2);
  if (kmod < g.kedge0 || kmod >= g.kedgeN) return -1;
  const int b = (int)__ddiv_rn(__dsub_rn(kmod, g.kedge0), g.dk);
  return (b < 0 || b >= g.nbin) ? -1 : b;
}

inline int signed_index(int i, int ng) { return (i <= (ng >> 1)) ? i : i - ng; }
__device__ __forceinline__ int dsigned(int i, int ng) { return (i <= (ng >> 1)) ? i : i - ng; }

// One real spherical harmonic Y_lm, l <= 6, in the basis of the reference's
// math/spherical.h:54-262 (no Condon-Shortley sign; m > 0: cos(m phi),
// m < 0: sin(|m| phi)).  Y_lm = sin^|m|(t) q(cos t) trig(|m| phi), where
// q = K_lm [sqrt 2 if m != 0] d^|m| P_l / dx^|m| holds the normalisation
// (host: ylm_coef).  The basis matters: the estimator replaces the harmonic
// by 1 for every m on the k_z axis and at k = 0, where sum_m Y_lm(r^)
// enters alone.
struct YlmCoef {
  int am;        // |m|
  int trig;      // 0: m = 0; 1: cos(|m| phi); -1: sin(|m| phi)
  int deg;       // degree of q (l - |m|)
  float q[7];    // coefficients of q, x^0 .. x^deg
};

// The part of Y_lm that depends on (x, y) only, for a row of cells that
// share them: r_xy, r_xy^2 and trig(|m| phi).
struct YlmRow {
  float rxy, rxy2, trig;
};
__device__ __forceinline__ YlmRow ylm_row(const YlmCoef& c, float x, float y) {
  YlmRow w;
  w.rxy2 = fmaf(x, x, y * y);
  w.trig = 1.f;
  w.rxy = 0.f;
  if (c.am) {
    const float ri = rsqrtf(w.rxy2);
    w.rxy = w.rxy2 * ri;
    const float cp = x * ri, sp = y * ri;
    float co = cp, si = sp;
#pragma unroll
    for (int i = 1; i < 6; i++) {
      if (i < c.am) {
        const float c2 = co * cp - si * sp;
        si = fmaf(si, cp, co * sp);
        co = c2;
      }
    }
    w.trig = c.trig > 0 ? co : si;
  }
  return w;
}
// Y_lm at height z above the row: same value as ylm_eval(c, x, y, z).
__device__ __forceinline__ float ylm_cell(const YlmCoef& c, const YlmRow& w, float z) {
  const float rinv = rsqrtf(fmaf(z, z, w.rxy2));
  const float ct = z * rinv;
  float q = c.q[6];
#pragma unroll
  for (int d = 5; d >= 0; d--) q = fmaf(q, ct, c.q[d]);
  if (c.am == 0) return q;
  const float st = w.rxy * rinv;
  float stm = st;
#pragma unroll
  for (int i = 1; i < 6; i++)
    if (i < c.am) stm *= st;
  return q * stm * w.trig;
}

// Y_lm of the direction (x, y, z), not normalised; x = y = 0 gives NaN for
// m != 0 (callers treat the axis themselves).
__device__ __forceinline__ float ylm_eval(const YlmCoef& c, float x, float y, float z) {
  const float rxy2 = fmaf(x, x, y * y);
  const float rinv = rsqrtf(fmaf(z, z, rxy2));
  const float ct = z * rinv;
  // fixed-index Horner over all 7 slots (unused ones are 0): no dynamic
  // indexing, so the coefficients stay in registers
  float q = c.q[6];
#pragma unroll
  for (int d = 5; d >= 0; d--) q = fmaf(q, ct, c.q[d]);
  if (c.am == 0) return q;
  const float ri = rsqrtf(rxy2);  // 1 / r_xy
  const float st = rxy2 * ri * rinv;
  const float cp = x * ri, sp = y * ri;
  float stm = st, co = cp, si = sp;
#pragma unroll
  for (int i = 1; i < 6; i++) {
    if (i < c.am) {
      stm *= st;
      const float c2 = co * cp - si * sp;
      si = fmaf(si, cp, co * sp);
      co = c2;
    }
  }
  return q * stm * (c.trig > 0 ? co : si);
}

}  // namespace ps
