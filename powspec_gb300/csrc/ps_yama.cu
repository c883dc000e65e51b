// ps_yama.cu -- survey multipoles l > 0 by the spherical-harmonic
// decomposition of the Legendre polynomial (Hand et al. 2017; the
// reference's src/mp_template.c:48-149):
//   F_l(k) = sum_m Y_lm(k^) FFT[ F(r) Y_lm(r^) ](k),
//   P_l ~ sum_k Re[F_0(k) F_l(k)*],
// with F the data - alpha x randoms mesh and r^ the direction from the
// observer (the coordinate origin).  Each term runs as the r2c passes with
// the mesh weighted by Y_lm(r^) as pass A reads it (ps_fft.cu) and pass C
// adding Y_lm(k^) times its output into F_l (ps_bin.cu).  This file holds
// the harmonics' coefficients and the c2r of the interlaced field.
//
// The harmonics are the reference's real basis (math/spherical.h:54-262),
// evaluated as sin^|m| t q(cos t) trig(|m| phi) with q's coefficients from
// the host (ylm_coef).  Two conventions of the reference are kept: the
// first mesh row (i = j = 0) and the modes on the k_z axis (k_x = k_y = 0)
// take the harmonic as 1 for every m (src/mp_template.c:71-74, :118-121).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ps_internal.h"

namespace ps {

// FP64 coefficients of the polynomial in cos(theta) of Y_l,m for |m| = am:
// kl times the am-th derivative of P_l, kl the normalisation (with sqrt 2
// for am > 0); q[d] for d <= l - am, 0 above.
void ylm_poly(int l, int am, double* q) {
  // Legendre P_l coefficients by (n + 1) P_(n+1) = (2n + 1) x P_n - n P_(n-1)
  double p0[8] = {1}, p1[8] = {0, 1}, pl[8] = {0};
  if (l == 0) std::copy(p0, p0 + 8, pl);
  if (l == 1) std::copy(p1, p1 + 8, pl);
  for (int n = 1; n < l; n++) {
    double nx[8] = {0};
    for (int d = 0; d < 7; d++) nx[d + 1] += (2 * n + 1) * p1[d] / (n + 1);
    for (int d = 0; d < 8; d++) nx[d] -= n * p0[d] / (n + 1);
    std::copy(p1, p1 + 8, p0);
    std::copy(nx, nx + 8, p1);
    std::copy(nx, nx + 8, pl);
  }
  for (int k = 0; k < am; k++)  // d/dx, |m| times
    for (int d = 0; d < 7; d++) pl[d] = (d + 1) * pl[d + 1];
  double f = 1;  // (l - |m|)! / (l + |m|)!
  for (int r = l - am + 1; r <= l + am; r++) f /= r;
  double kl = std::sqrt((2 * l + 1) / (4 * M_PI) * f);
  if (am) kl *= std::sqrt(2.0);
  for (int d = 0; d < 7; d++) q[d] = d <= l - am ? kl * pl[d] : 0.0;
}

YlmCoef ylm_coef(int l, int m) {
  const int am = std::abs(m);
  double q[7];
  ylm_poly(l, am, q);
  YlmCoef c;
  c.am = am;
  c.trig = m > 0 ? 1 : (m < 0 ? -1 : 0);
  c.deg = l - am;
  for (int d = 0; d < 7; d++) c.q[d] = (float)q[d];
  return c;
}

namespace {

// ------------------------------------------------ c2r of the interlaced field
// With interlacing, the harmonic weights multiply the real-space field of
// the combined F_0: FFT_EXEC_C2R of (F0 + exp(i theta) F1) / 2, divided by
// Ng^3 (src/multipole.c:462-500).  The inverse runs as the c2r transform
// does: inverse complex DFTs along x, then y, over the stored half-complex
// field, then a half-complex -> real transform of each z row that ignores
// the imaginary parts of its kz = 0 and kz = Ng/2 terms.  Inverse DFTs are
// forward ones of the conjugate, conjugated.

struct InvLeadArgs {
  int ng, tz;             // mesh size; kz values per CTA
  float2* in;             // [l][p][kz]; receives the combined field if in2
  const float2* in2;      // shifted mesh's field, or null
  float2* out;            // [p][l][kz]
  const float2* phase;    // exp(i pi n / ng), n = signed kx + ky + kz + ng
  const float2* tw_full;
  FftPlan plan_full;
};

// out[p][l][kz] = sum_l' in[l'][p][kz] exp(+2 pi i l l' / ng): the inverse
// along the leading axis, the two leading axes swapped on the way out, so
// two launches take [kx][ky][kz] to [x][y][kz].  Each CTA transforms the
// lines of one p and tz consecutive kz (contiguous in memory).
template <bool P2>
__global__ void __launch_bounds__(kFftThreads) k_inv_lead(const __grid_constant__ InvLeadArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, ngk = (ng >> 1) + 1;
  const int ls = line_stride(ng, P2);
  const int ntz = (ngk + a.tz - 1) / a.tz;
  const int p = blockIdx.x / ntz;
  const int kz0 = (blockIdx.x - p * ntz) * a.tz;
  const int nl = min(a.tz, ngk - kz0);
  const int pp = dsigned(p, ng);
  for (int e = threadIdx.x; e < ng * nl; e += blockDim.x) {
    const int l = e / nl, r = e - l * nl;
    const size_t idx = ((size_t)l * ng + p) * ngk + kz0 + r;
    float2 v = a.in[idx];
    if (a.in2) {
      const float2 t = cmul(__ldg(&a.phase[dsigned(l, ng) + pp + kz0 + r + ng]), a.in2[idx]);
      v = make_float2(0.5f * (v.x + t.x), 0.5f * (v.y + t.y));
      a.in[idx] = v;
    }
    sm[r * ls + lidx<P2>(l)] = make_float2(v.x, -v.y);
  }
  __syncthreads();
  if (P2)
    fft2_lines(sm, a.plan_full.logn, nl, ls, a.tw_full);
  else
    fft_lines(sm, a.plan_full, nl, ls, a.tw_full);
  float2* ob = a.out + (size_t)p * ng * ngk + kz0;
  for (int e = threadIdx.x; e < ng * nl; e += blockDim.x) {
    const int l = e / nl, r = e - l * nl;
    const float2 v = sm[r * ls + lidx<P2>(l)];
    ob[(size_t)l * ngk + r] = make_float2(v.x, -v.y);
  }
}

struct C2rArgs {
  int ng, ty;             // mesh size; rows per CTA
  float scale;            // 1 / Ng^3
  const float2* in;       // [x][y][0..ng/2]
  float* out;             // [x][y][0..ng)
  const float2* tw_half;
  const float2* tw_full;
  FftPlan plan_half;
};

// Half-complex rows -> real rows, times `scale`.  With M = ng / 2 and
// w_k = exp(2 pi i k / ng),
//   Z[k] = (X[k] + conj X[M-k]) + i w_k (X[k] - conj X[M-k]),  k < M,
// is twice the M-point DFT of x[2m] + i x[2m+1], so one inverse M-point
// transform gives the even and odd samples.  Pairs (k, M - k) go to one
// thread, which reads both before writing either.
template <bool P2>
__global__ void __launch_bounds__(kFftThreads) k_c2r_z(const __grid_constant__ C2rArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, M = ng >> 1, ngk = M + 1;
  const int ls = line_stride(M + 1, P2);
  const size_t rows = (size_t)ng * ng, r0 = (size_t)blockIdx.x * a.ty;
  const int nl = (int)((rows - r0) < (size_t)a.ty ? rows - r0 : (size_t)a.ty);
  const float2* ib = a.in + r0 * ngk;
  for (int e = threadIdx.x; e < nl * ngk; e += blockDim.x) {
    const int r = e / ngk, k = e - r * ngk;
    sm[r * ls + lidx<P2>(k)] = ib[e];
  }
  __syncthreads();
  const int half = (M >> 1) + 1;
  for (int e = threadIdx.x; e < nl * half; e += blockDim.x) {
    const int r = e / half, k = e - r * half;
    float2* L = sm + r * ls;
    if (k == 0) {  // imaginary parts of X[0], X[M] ignored; Z[0] stored conjugated
      const float x0 = L[0].x, xm = L[lidx<P2>(M)].x;
      L[0] = make_float2(x0 + xm, xm - x0);
      continue;
    }
    const int ik = lidx<P2>(k), imk = lidx<P2>(M - k);
    const float2 A = L[ik], B = L[imk];
    const float2 t = __ldg(&a.tw_full[k]);  // exp(-2 pi i k / ng) = conj w_k
    // Z[k]: S = A + conj B, D = A - conj B, q = w_k D
    {
      const float2 S = make_float2(A.x + B.x, A.y - B.y), D = make_float2(A.x - B.x, A.y + B.y);
      const float2 q = cmul(make_float2(t.x, -t.y), D);
      L[ik] = make_float2(S.x - q.y, -(S.y + q.x));
    }
    if (M - k != k) {  // Z[M-k]: w_(M-k) = -conj w_k
      const float2 S = make_float2(B.x + A.x, B.y - A.y), D = make_float2(B.x - A.x, B.y + A.y);
      const float2 q = cmul(make_float2(-t.x, -t.y), D);
      L[imk] = make_float2(S.x - q.y, -(S.y + q.x));
    }
  }
  __syncthreads();
  if (P2)
    fft2_lines(sm, a.plan_half.logn, nl, ls, a.tw_half);
  else
    fft_lines(sm, a.plan_half, nl, ls, a.tw_half);
  float2* ob = reinterpret_cast<float2*>(a.out + r0 * ng);
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int r = e / M, m = e - r * M;
    const float2 v = sm[r * ls + lidx<P2>(m)];
    ob[(size_t)r * M + m] = make_float2(v.x * a.scale, -v.y * a.scale);
  }
}

}  // namespace

int launch_inv_lead(float2* in, const float2* in2, float2* out, int ng, const float2* phase,
                    const float2* tw_full, const FftPlan& plan_full, cudaStream_t s) {
  InvLeadArgs a;
  a.ng = ng;
  a.tz = std::max(1, std::min(32, kCtaElems / ng));
  a.in = in;
  a.in2 = in2;
  a.out = out;
  a.phase = phase;
  a.tw_full = tw_full;
  a.plan_full = plan_full;
  const bool p2 = plan_full.logn >= 0;
  const size_t smem = (size_t)a.tz * line_stride(ng, p2) * sizeof(float2);
  const unsigned grid = (unsigned)(ng * ((ng / 2 + 1 + a.tz - 1) / a.tz));
  if (p2) {
    cudaFuncSetAttribute(k_inv_lead<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_inv_lead<true><<<grid, kFftThreads, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(k_inv_lead<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_inv_lead<false><<<grid, kFftThreads, smem, s>>>(a);
  }
  return 1;
}

int launch_c2r_z(const float2* in, float* out, int ng, int ty, const float2* tw_half,
                 const float2* tw_full, const FftPlan& plan_half, cudaStream_t s) {
  C2rArgs a;
  a.ng = ng;
  a.ty = ty;
  a.scale = (float)(1.0 / ((double)ng * ng * ng));
  a.in = in;
  a.out = out;
  a.tw_half = tw_half;
  a.tw_full = tw_full;
  a.plan_half = plan_half;
  const bool p2 = plan_half.logn >= 0;
  const size_t smem = (size_t)ty * line_stride(ng / 2 + 1, p2) * sizeof(float2);
  const size_t rows = (size_t)ng * ng;
  const unsigned grid = (unsigned)((rows + ty - 1) / ty);
  if (p2) {
    cudaFuncSetAttribute(k_c2r_z<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_c2r_z<true><<<grid, kFftThreads, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(k_c2r_z<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_c2r_z<false><<<grid, kFftThreads, smem, s>>>(a);
  }
  return 1;
}

// ------------------------------------------------- F_l(0) in FP64
// The k = 0 term of F_l is sum_m sum_r F(r) Y_lm(r^) (the harmonic of k^ is
// 1 at k = 0, src/mp_template.c:118-121), a sum that cancels to a small
// fraction of its terms, and the first bin of a survey multipole is W times
// it.  Summed here directly over the mesh in FP64, harmonics included (an
// FP32 harmonic, 1e-7 off, leaves ~1e-4 of the noise scale in that bin when
// W is far from 0).  The +m (cos) and -m (sin) harmonics share their
// polynomial in cos(theta), so sum_m Y_lm = sum_am q_am(cos t) sin^am(t)
// (cos(am phi) + sin(am phi)); the row i = j = 0 takes 1 for every m
// (src/mp_template.c:71-74).  Per-CTA sums, then a fixed-order reduce.
namespace {

struct DcArgs {
  int ng, ell;
  const float* mesh;
  double q[7][7];  // [am][degree]: kl q of Y_l,am (sqrt 2 included for am > 0)
  double org[3], len[3];
  double* part;    // [gridDim.x]
  const double* wsum;  // [ncat][2]: each catalogue's sum of w and of |w|
  int ncat;
};

// The FP64 sum is needed only when a catalogue's weighted total W, which
// multiplies F_l(0) in the first bin, is not small against its sum of |w|;
// otherwise the transform's FP32 DC is kept.
__device__ __forceinline__ bool dc_needed(const double* wsum, int ncat) {
  bool need = false;
  for (int k = 0; k < ncat; k++) need |= fabs(wsum[2 * k]) > kDcGate * wsum[2 * k + 1];
  return need;
}

__global__ void __launch_bounds__(256) k_dc_sum(const __grid_constant__ DcArgs a) {
  if (!dc_needed(a.wsum, a.ncat)) return;
  const int ng = a.ng, ell = a.ell;
  const size_t nrow = (size_t)ng * ng;
  double acc = 0.0;
  for (size_t row = blockIdx.x; row < nrow; row += gridDim.x) {
    const int i = (int)(row / ng), j = (int)(row - (size_t)i * ng);
    const float* r = a.mesh + row * ng;
    if (i == 0 && j == 0) {
      double t = 0.0;
      for (int k = threadIdx.x; k < ng; k += blockDim.x) t += (double)r[k];
      acc = fma(t, (double)(2 * ell + 1), acc);
      continue;
    }
    const double X = (i + a.org[0]) * a.len[0], Y = (j + a.org[1]) * a.len[1];
    const double rxy2 = fma(X, X, Y * Y), rxy = sqrt(rxy2);
    const double cp = X / rxy, sp = Y / rxy;
    double T[7];  // cos(am phi) + sin(am phi)
    T[0] = 1.0;
    double co = 1.0, si = 0.0;
    for (int am = 1; am <= ell; am++) {
      const double c2 = co * cp - si * sp;
      si = fma(si, cp, co * sp);
      co = c2;
      T[am] = co + si;
    }
    for (int k = threadIdx.x; k < ng; k += blockDim.x) {
      const double Z = (k + a.org[2]) * a.len[2];
      const double rinv = rsqrt(fma(Z, Z, rxy2));
      const double ct = Z * rinv, st = rxy * rinv;
      double ysum = 0.0, stm = 1.0;
      for (int am = 0; am <= ell; am++) {
        double q = 0.0;
        for (int d = ell - am; d >= 0; d--) q = fma(q, ct, a.q[am][d]);
        ysum = fma(q * stm, T[am], ysum);
        stm *= st;
      }
      acc = fma((double)r[k], ysum, acc);
    }
  }
  __shared__ double sh[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    a.part[blockIdx.x] = t;
  }
}

// out = the FP64 sum (when needed) or the FP32 transform's DC.
__global__ void k_dc_select(const double* sum, const float2* dc32, const double* wsum, int ncat,
                            double* out) {
  *out = dc_needed(wsum, ncat) ? *sum : (double)dc32->x;
}

}  // namespace

int launch_dc_sum(const float* mesh, int ng, int ell, const double* org, const double* len,
                  const double* wsum, int ncat, const float2* dc32, double* part, int grid,
                  double* out, cudaStream_t s) {
  if (ell < 0 || ell > 6) return -1;
  DcArgs a;
  memset(&a, 0, sizeof a);
  a.ng = ng;
  a.ell = ell;
  a.mesh = mesh;
  for (int am = 0; am <= ell; am++) {
    double q[7];
    ylm_poly(ell, am, q);
    for (int d = 0; d < 7; d++) a.q[am][d] = q[d];
  }
  for (int d = 0; d < 3; d++) {
    a.org[d] = org[d];
    a.len[d] = len[d];
  }
  a.part = part;
  a.wsum = wsum;
  a.ncat = ncat;
  k_dc_sum<<<grid, 256, 0, s>>>(a);
  launch_reduce_f64(part, grid, 1, part + grid, s);
  k_dc_select<<<1, 1, 0, s>>>(part + grid, dc32, wsum, ncat, out);
  return 3;
}

}  // namespace ps
