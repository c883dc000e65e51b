// ps_bin_core.cuh -- the binning core shared by the x-pass kernels of
// ps_bin.cu (block-tiled transforms) and ps_wfft.cu (warp transforms).
//
// Accumulation: every thread walks a run of consecutive modes along x, whose
// |k| grows monotonically, and keeps the run's sums in registers while the
// bin stays the same; on a bin change it adds them to FP32 per-tile
// accumulators in shared memory.  After every few tiles the touched bins are
// added into the CTA's slice of a partial-sum array in global memory (FP32
// pairs), which a final kernel reduces over CTAs in a fixed order.
//
// Reference: dens_k0's interlace combine (src/multipole.c:462-487) and
// count_mode_sim_lin/_log (src/multipole.c:778-1031).
#ifndef PS_BIN_CORE_CUH
#define PS_BIN_CORE_CUH

#include "ps_internal.h"

namespace ps {
namespace {

constexpr int kRun = 8;          // consecutive modes per thread
constexpr int kMergeEvery = 8;   // tiles between FP32 -> FP64 merges

template <int NSPEC>
struct RunAcc {
  int bin;
  float v[NSPEC][kMaxPole];
};

template <int NSPEC>
__device__ __forceinline__ void run_flush(RunAcc<NSPEC>& ra, float* tacc, int npole, int nbin,
                                          int& lo, int& hi) {
  if (ra.bin < 0) return;
#pragma unroll
  for (int s = 0; s < NSPEC; s++)
#pragma unroll
    for (int l = 0; l < kMaxPole; l++)
      if (l < npole) {
        if (ra.v[s][l] != 0.f) atomicAdd(&tacc[(s * npole + l) * nbin + ra.bin], ra.v[s][l]);
        ra.v[s][l] = 0.f;
      }
  lo = min(lo, ra.bin);
  hi = max(hi, ra.bin);
}

// Adds one mode with power p[s] (already windowed and weighted) at mu.
template <int NSPEC>
__device__ __forceinline__ void run_add(RunAcc<NSPEC>& ra, const ModeGeom& g, int b, int nkey,
                                        const float (&p)[NSPEC], float mu, bool skip_odd,
                                        float* tacc, int& lo, int& hi) {
  if (b != ra.bin) {
    run_flush<NSPEC>(ra, tacc, g.npole, nkey, lo, hi);
    ra.bin = b;
  }
  const float m2 = mu * mu;
#pragma unroll
  for (int l = 0; l < kMaxPole; l++) {
    if (l < g.npole) {
      const bool odd = (g.lodd >> l) & 1;
      if (skip_odd && odd) continue;  // cancels between half-spaces (src/multipole.c:844)
      float L = fmaf(fmaf(fmaf(g.lc[l][3], m2, g.lc[l][2]), m2, g.lc[l][1]), m2, g.lc[l][0]);
      if (odd) L *= mu;
#pragma unroll
      for (int s = 0; s < NSPEC; s++) ra.v[s][l] = fmaf(p[s], L, ra.v[s][l]);
    }
  }
}

// Record a thread's touched bin range [lo, hi] into the block's range.
__device__ __forceinline__ void note_range(int* srange, int lo, int hi) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0 && hi >= lo) {
    atomicMin(&srange[0], lo);
    atomicMax(&srange[1], hi);
  }
}

// Merge the FP32 accumulators of the touched bin range into the CTA's
// slice of FP32-pair partials (hi + lo, about 48 bits: FP64 adds are slow
// on this GPU) and clear them.  Starts and ends with a barrier.
__device__ void merge_tile(float* tacc, int* srange, float2* part, int nacc, int nbin) {
  __syncthreads();
  const int blo = srange[0], bhi = srange[1];
  if (bhi >= blo) {
    const int w = bhi - blo + 1;
    for (int e = threadIdx.x; e < nacc * w; e += blockDim.x) {
      const int q = e / w;
      const int idx = q * nbin + blo + (e - q * w);
      float2 pv = part[idx];
      df_add(pv.x, pv.y, tacc[idx], 0.f);
      part[idx] = pv;
      tacc[idx] = 0.f;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
}

// Moment form of the accumulation, for pole sets of even multipoles only
// (MOM = lmax / 2 + 1 moments): per (k, mu) key the FP32 run and tile sums
// hold M_j = sum p mu^(2j), j < MOM, two multiplies and MOM adds a mode
// instead of a Horner evaluation per pole.  The merge turns them into the
// Legendre sums, sum p L_l(mu) = sum_j c_lj M_j with the exact coefficients
// of L_l in mu^2 (math/legpoly.h:47-62), combined in FP32 and added into
// the FP32-pair partials.
template <int NSPEC, int MOM>
struct MomAcc {
  int bin;
  float v[NSPEC][MOM];
};

template <int NSPEC, int MOM>
__device__ __forceinline__ void mom_flush(MomAcc<NSPEC, MOM>& ra, float* tacc, int nkey, int& lo,
                                          int& hi) {
  if (ra.bin < 0) return;
#pragma unroll
  for (int s = 0; s < NSPEC; s++)
#pragma unroll
    for (int j = 0; j < MOM; j++) {
      if (ra.v[s][j] != 0.f) atomicAdd(&tacc[(s * MOM + j) * nkey + ra.bin], ra.v[s][j]);
      ra.v[s][j] = 0.f;
    }
  lo = min(lo, ra.bin);
  hi = max(hi, ra.bin);
}

template <int NSPEC, int MOM>
__device__ __forceinline__ void mom_add(MomAcc<NSPEC, MOM>& ra, int b, int nkey,
                                        const float (&p)[NSPEC], float mu, float* tacc, int& lo,
                                        int& hi) {
  if (b != ra.bin) {
    mom_flush<NSPEC, MOM>(ra, tacc, nkey, lo, hi);
    ra.bin = b;
  }
  const float m2 = mu * mu;
#pragma unroll
  for (int s = 0; s < NSPEC; s++) {
    float t = p[s];
    ra.v[s][0] += t;
#pragma unroll
    for (int j = 1; j < MOM; j++) {
      t *= m2;
      ra.v[s][j] += t;
    }
  }
}

// Merge of moment tile sums: the Legendre sums of the touched keys are added
// into the CTA's FP32-pair slice [NSPEC][npole][nkey], the moments cleared.
template <int NSPEC, int MOM>
__device__ void merge_tile_mom(float* tacc, int* srange, float2* part, const ModeGeom& g,
                               int nkey) {
  __syncthreads();
  const int blo = srange[0], bhi = srange[1];
  if (bhi >= blo) {
    const int w = bhi - blo + 1;
    for (int e = threadIdx.x; e < NSPEC * w; e += blockDim.x) {
      const int s = e / w, key = blo + (e - s * w);
      float m[MOM];
      bool any = false;
#pragma unroll
      for (int j = 0; j < MOM; j++) {
        float* t = &tacc[(s * MOM + j) * nkey + key];
        m[j] = *t;
        any |= m[j] != 0.f;
        *t = 0.f;
      }
      if (!any) continue;  // a key of the range that no mode reached
      // the combination in FP32 (FP64 arithmetic is slow on this GPU; the
      // moments are FP32 sums already), added into the FP32-pair partials
      for (int l = 0; l < g.npole; l++) {
        float v = 0.f;
#pragma unroll
        for (int j = 0; j < MOM; j++) v = fmaf(g.lc[l][j], m[j], v);
        float2& q = part[(s * g.npole + l) * nkey + key];
        float h = q.x, lo = q.y;
        df_add(h, lo, v, 0.f);
        q = make_float2(h, lo);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
}

template <int NSPEC, int MOM>
__device__ __forceinline__ void merge_any(float* tacc, int* srange, float2* part,
                                          const ModeGeom& g, int nkey) {
  if (MOM > 0) merge_tile_mom<NSPEC, (MOM > 0 ? MOM : 1)>(tacc, srange, part, g, nkey);
  else merge_tile(tacc, srange, part, NSPEC * g.npole, nkey);
}

// Accumulators of the tile sums: moments or pole sums.
template <int NSPEC, int MOM>
__device__ __forceinline__ int tile_accs(const ModeGeom& g) {
  return NSPEC * (MOM > 0 ? MOM : g.npole);
}

// Binning of one transformed tile: lines f * nl + r of X (field f, row ky0 + r
// of plane kz), each mode windowed, combined and added to the tile sums.
// Power of the mode at x index xi (signed ip) of line r: the combined field
// of each catalogue, (F0 + exp(i theta) F1) / 2 with interlacing, windowed.
template <int NSPEC, bool P2>
__device__ __forceinline__ void mode_power(const PassCArgs& a, const float2* X, int ls, int nl,
                                           int r, int xi, int ip, int jp, int kz, float wjk,
                                           const int (&spec_a)[NSPEC], const int (&spec_b)[NSPEC],
                                           float (&p)[NSPEC]) {
  const int ng = a.ng;
  const ModeGeom& g = a.geom;
  const int mpc = a.interlace ? 2 : 1;
  const int li = lidx<P2>(xi);
  float2 G0 = X[r * ls + li], G1 = G0;
  float2 ph = make_float2(1.f, 0.f);
  if (a.interlace) {
    ph = __ldg(&g.phase[ip + jp + kz + ng]);
    const float2 t = cmul(ph, X[(nl + r) * ls + li]);
    G0 = make_float2(0.5f * (G0.x + t.x), 0.5f * (G0.y + t.y));
  }
  if (a.ncat > 1) {
    G1 = X[(mpc * nl + r) * ls + li];
    if (a.interlace) {
      const float2 t = cmul(ph, X[((mpc + 1) * nl + r) * ls + li]);
      G1 = make_float2(0.5f * (G1.x + t.x), 0.5f * (G1.y + t.y));
    }
  }
  const float wwin = __ldg(&g.win[xi]) * wjk;
#pragma unroll
  for (int s = 0; s < NSPEC; s++) {
    const float2 A = spec_a[s] ? G1 : G0;
    const float2 B = spec_b[s] ? G1 : G0;
    p[s] = (A.x * B.x + A.y * B.y) * wwin;
  }
}

// Moment binning when the line of sight has no x component: the modes at
// +k_x and -k_x of a line share |k|, mu, the bin and the |mu| sub-bin, so
// they are binned as one: the geometry once and one accumulation of the
// two powers (the window and the interlace phase stay per mode).  Lanes
// walk runs of consecutive |k_x| in [0, Ng/2): kRun long, or shorter so
// that a line gives every lane of a warp a run; the run that ends at Ng/2
// also takes the Nyquist plane k_x = Ng/2.
template <int NSPEC, bool P2, int MOM>
__device__ __forceinline__ void bin_lines_pair(const PassCArgs& a, const float2* X, int ls,
                                               int kz, int ky0, int nl, float* tacc, int& lo,
                                               int& hi, int tid, int nthr) {
  const int ng = a.ng, half = ng >> 1;
  const ModeGeom& g = a.geom;
  const int nkey = g.nbin * g.nmu;
  int spec_a[NSPEC], spec_b[NSPEC];
#pragma unroll
  for (int s = 0; s < NSPEC; s++) {
    spec_a[s] = a.spec_a[s];
    spec_b[s] = a.spec_b[s];
  }
  const bool twice = !(kz == 0 || 2 * kz == ng);
  const float wk = twice ? 2.f : 1.f;
  const float kzf = g.vec[2] * (float)kz;
  const int runp = max(1, min(kRun, half / 32));
  const int chunks = (half + runp - 1) / runp;
  for (int e = tid; e < nl * chunks; e += nthr) {
    const int r = e / chunks;
    const int i0 = (e - r * chunks) * runp;
    const int ky = ky0 + r;
    const int jp = dsigned(ky, ng), ja = abs(jp);
    const float wjk = __ldg(&g.win[ng + ky]) * __ldg(&g.win[2 * ng + kz]) * wk;
    const float kyf = g.vec[1] * (float)jp;
    const float mu_yz = kyf * g.los[1] + kzf * g.los[2];
    const float k2_yz = kyf * kyf + kzf * kzf;
    const int n_yz = ja * ja + kz * kz;
    MomAcc<NSPEC, MOM> rm;
    rm.bin = -1;
#pragma unroll
    for (int s = 0; s < NSPEC; s++)
#pragma unroll
      for (int j = 0; j < MOM; j++) rm.v[s][j] = 0.f;
    int iend = min(i0 + runp, half);
    if (iend == half) iend = half + 1;
    for (int i = i0; i < iend; i++) {
      const int n = i * i + n_yz;
      if (n == 0) continue;  // DC (src/multipole.c:806)
      const float kxf = g.vec[0] * (float)i;
      const float rq = rsqrtf(kxf * kxf + k2_yz);
      int b;
      if (g.fastbin) {
        const float t = (fmaf(kxf, kxf, k2_yz) * rq - g.k0f) * g.inv_dkf;
        const float fl = floorf(t), fr = t - fl;
        b = (fr > g.eps_t && fr < 1.f - g.eps_t) ? ((fl < 0.f || fl >= (float)g.nbin) ? -1 : (int)fl)
                                                 : mode_bin(g, i, ja, kz, n);
      } else {
        b = mode_bin(g, i, ja, kz, n);
      }
      if (b < 0) continue;
      const float mu = mu_yz * rq;
      const int key = (g.nmu == 1) ? b : b * g.nmu + min(g.nmu - 1, (int)(fabsf(mu) * g.nmu));
      float p[NSPEC];
      mode_power<NSPEC, P2>(a, X, ls, nl, r, i, i, jp, kz, wjk, spec_a, spec_b, p);
      if (i != 0 && i != half) {  // the mode at -k_x (x index ng - i)
        float q[NSPEC];
        mode_power<NSPEC, P2>(a, X, ls, nl, r, ng - i, -i, jp, kz, wjk, spec_a, spec_b, q);
#pragma unroll
        for (int s = 0; s < NSPEC; s++) p[s] += q[s];
      }
      mom_add<NSPEC, MOM>(rm, key, nkey, p, mu, tacc, lo, hi);
    }
    mom_flush<NSPEC, MOM>(rm, tacc, nkey, lo, hi);
  }
}

// The +-k_y pairing of bin_lines_pair, for a warp that holds one line per
// field at a time (line ky, then line Ng - ky, at one kz): with the line of
// sight along z the four modes (+-k_x, +-k_y, k_z) share |k|, mu, the bin
// and the |mu| sub-bin, so the geometry is evaluated once for the four.
// Each lane keeps the windowed, combined powers of its runs of |k_x| in
// registers between the two lines (ypair_powers), then walks the geometry
// (ypair_bin); runs as in bin_lines_pair, the last one taking k_x = Ng/2.
template <int N>
struct YPairRuns {
  static constexpr int RP = (N / 64 < kRun) ? N / 64 : kRun;  // modes per run
  static constexpr int NC = (N / 2) / RP / 32;                // runs per lane
};

template <int N, int NSPEC>
__device__ __forceinline__ void ypair_powers(
    const PassCArgs& a, const float2* X, int ls, int kz, int ky,
    float (&pw)[YPairRuns<N>::NC][YPairRuns<N>::RP + 1][NSPEC], bool add, int lane,
    const int (&spec_a)[NSPEC], const int (&spec_b)[NSPEC]) {
  using Y = YPairRuns<N>;
  constexpr int half = N / 2;
  const ModeGeom& g = a.geom;
  const int jp = dsigned(ky, N);
  const bool twice = !(kz == 0 || 2 * kz == N);
  const float wjk = __ldg(&g.win[N + ky]) * __ldg(&g.win[2 * N + kz]) * (twice ? 2.f : 1.f);
#pragma unroll
  for (int c = 0; c < Y::NC; c++) {
    const int i0 = (lane + 32 * c) * Y::RP;
#pragma unroll
    for (int k = 0; k <= Y::RP; k++) {
      const int i = i0 + k;
      if (k == Y::RP && i != half) continue;  // only the last run takes k_x = Ng/2
      float p[NSPEC];
      mode_power<NSPEC, true>(a, X, ls, 1, 0, i, i, jp, kz, wjk, spec_a, spec_b, p);
      if (i != 0 && i != half) {  // the mode at -k_x
        float q[NSPEC];
        mode_power<NSPEC, true>(a, X, ls, 1, 0, N - i, -i, jp, kz, wjk, spec_a, spec_b, q);
#pragma unroll
        for (int s = 0; s < NSPEC; s++) p[s] += q[s];
      }
#pragma unroll
      for (int s = 0; s < NSPEC; s++) pw[c][k][s] = add ? pw[c][k][s] + p[s] : p[s];
    }
  }
}

template <int N, int NSPEC, int MOM>
__device__ __forceinline__ void ypair_bin(
    const PassCArgs& a, int kz, int kyp,
    const float (&pw)[YPairRuns<N>::NC][YPairRuns<N>::RP + 1][NSPEC], float* tacc, int& lo,
    int& hi, int lane) {
  using Y = YPairRuns<N>;
  constexpr int half = N / 2;
  const ModeGeom& g = a.geom;
  const int nkey = g.nbin * g.nmu;
  const float kzf = g.vec[2] * (float)kz;
  const float kyf = g.vec[1] * (float)kyp;
  const float mu_yz = kyf * g.los[1] + kzf * g.los[2];  // los[1] = 0: the same for -k_y
  const float k2_yz = kyf * kyf + kzf * kzf;
  const int n_yz = kyp * kyp + kz * kz;
#pragma unroll
  for (int c = 0; c < Y::NC; c++) {
    const int i0 = (lane + 32 * c) * Y::RP;
    MomAcc<NSPEC, MOM> rm;
    rm.bin = -1;
#pragma unroll
    for (int s = 0; s < NSPEC; s++)
#pragma unroll
      for (int j = 0; j < MOM; j++) rm.v[s][j] = 0.f;
#pragma unroll
    for (int k = 0; k <= Y::RP; k++) {
      const int i = i0 + k;
      if (k == Y::RP && i != half) continue;
      const int n = i * i + n_yz;
      if (n == 0) continue;  // DC (src/multipole.c:806)
      const float kxf = g.vec[0] * (float)i;
      const float rq = rsqrtf(kxf * kxf + k2_yz);
      int b;
      if (g.fastbin) {
        const float t = (fmaf(kxf, kxf, k2_yz) * rq - g.k0f) * g.inv_dkf;
        const float fl = floorf(t), fr = t - fl;
        b = (fr > g.eps_t && fr < 1.f - g.eps_t) ? ((fl < 0.f || fl >= (float)g.nbin) ? -1 : (int)fl)
                                                 : mode_bin(g, i, kyp, kz, n);
      } else {
        b = mode_bin(g, i, kyp, kz, n);
      }
      if (b < 0) continue;
      const float mu = mu_yz * rq;
      const int key = (g.nmu == 1) ? b : b * g.nmu + min(g.nmu - 1, (int)(fabsf(mu) * g.nmu));
      mom_add<NSPEC, MOM>(rm, key, nkey, pw[c][k], mu, tacc, lo, hi);
    }
    mom_flush<NSPEC, MOM>(rm, tacc, nkey, lo, hi);
  }
}

template <int NSPEC, bool P2, int MOM>
__device__ __forceinline__ void bin_lines(const PassCArgs& a, const float2* X, int ls, int kz,
                                          int ky0, int nl, float* tacc, int& lo, int& hi,
                                          int tid, int nthr) {
  if (MOM > 0 && a.geom.los[0] == 0.f) {
    bin_lines_pair<NSPEC, P2, (MOM > 0 ? MOM : 1)>(a, X, ls, kz, ky0, nl, tacc, lo, hi, tid, nthr);
    return;
  }
  constexpr int MM = MOM > 0 ? MOM : 1;
  const int ng = a.ng;
  const ModeGeom& g = a.geom;
  const int nkey = g.nbin * g.nmu;
  const int mpc = a.interlace ? 2 : 1;
  const bool interlace = a.interlace != 0, two_cat = a.ncat > 1;
  int spec_a[NSPEC], spec_b[NSPEC];
#pragma unroll
  for (int s = 0; s < NSPEC; s++) {
    spec_a[s] = a.spec_a[s];
    spec_b[s] = a.spec_b[s];
  }
  const bool twice = !(kz == 0 || 2 * kz == ng);
  const float wk = twice ? 2.f : 1.f;
  const float kzf = g.vec[2] * (float)kz;
  const int chunks = (ng + kRun - 1) / kRun;
  for (int e = tid; e < nl * chunks; e += nthr) {
    const int r = e / chunks;
    const int i0 = (e - r * chunks) * kRun;
    const int ky = ky0 + r;
    const int jp = dsigned(ky, ng), ja = abs(jp);
    const float wjk = __ldg(&g.win[ng + ky]) * __ldg(&g.win[2 * ng + kz]) * wk;
    const float kyf = g.vec[1] * (float)jp;
    const float mu_yz = kyf * g.los[1] + kzf * g.los[2];
    const float k2_yz = kyf * kyf + kzf * kzf;
    const int n_yz = ja * ja + kz * kz;
    RunAcc<(MOM > 0 ? 1 : NSPEC)> ra;  // pole sums (MOM == 0)
    MomAcc<NSPEC, MM> rm;               // moments (MOM > 0)
    ra.bin = -1;
    rm.bin = -1;
    if (MOM == 0) {
#pragma unroll
      for (int s = 0; s < (MOM > 0 ? 1 : NSPEC); s++)
#pragma unroll
        for (int l = 0; l < kMaxPole; l++) ra.v[s][l] = 0.f;
    } else {
#pragma unroll
      for (int s = 0; s < NSPEC; s++)
#pragma unroll
        for (int j = 0; j < MM; j++) rm.v[s][j] = 0.f;
    }
    const int iend = min(i0 + kRun, ng);
    for (int i = i0; i < iend; i++) {
      const int ip = dsigned(i, ng), ia = abs(ip);
      const int n = ia * ia + n_yz;
      if (n == 0) continue;  // DC (src/multipole.c:806)
      // one reciprocal square root gives both |k| (bin estimate) and mu
      const float kxf = g.vec[0] * (float)ip;
      const float rq = rsqrtf(kxf * kxf + k2_yz);
      int b;
      if (g.fastbin) {
        const float t = (fmaf(kxf, kxf, k2_yz) * rq - g.k0f) * g.inv_dkf;
        const float fl = floorf(t), fr = t - fl;
        b = (fr > g.eps_t && fr < 1.f - g.eps_t) ? ((fl < 0.f || fl >= (float)g.nbin) ? -1 : (int)fl)
                                                 : mode_bin(g, ia, ja, kz, n);
      } else {
        b = mode_bin(g, ia, ja, kz, n);
      }
      if (b < 0) continue;
      // combined field of each catalogue: (F0 + exp(i theta) F1) / 2
      const int li = lidx<P2>(i);
      float2 G0 = X[r * ls + li], G1 = G0;
      if (interlace) {
        const float2 ph = __ldg(&g.phase[ip + jp + kz + ng]);
        const float2 t = cmul(ph, X[(nl + r) * ls + li]);
        G0 = make_float2(0.5f * (G0.x + t.x), 0.5f * (G0.y + t.y));
      }
      if (two_cat) {
        G1 = X[(mpc * nl + r) * ls + li];
        if (interlace) {
          const float2 ph = __ldg(&g.phase[ip + jp + kz + ng]);
          const float2 t = cmul(ph, X[((mpc + 1) * nl + r) * ls + li]);
          G1 = make_float2(0.5f * (G1.x + t.x), 0.5f * (G1.y + t.y));
        }
      }
      const float wwin = __ldg(&g.win[i]) * wjk;
      float p[NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; s++) {
        const float2 A = spec_a[s] ? G1 : G0;
        const float2 B = spec_b[s] ? G1 : G0;
        p[s] = (A.x * B.x + A.y * B.y) * wwin;
      }
      const float mu = (kxf * g.los[0] + mu_yz) * rq;
      const int key = (g.nmu == 1) ? b : b * g.nmu + min(g.nmu - 1, (int)(fabsf(mu) * g.nmu));
      if (MOM > 0) {
        mom_add<NSPEC, MM>(rm, key, nkey, p, mu, tacc, lo, hi);
      } else {
        float q[MOM > 0 ? 1 : NSPEC];
#pragma unroll
        for (int s = 0; s < (MOM > 0 ? 1 : NSPEC); s++) q[s] = p[s];
        run_add<(MOM > 0 ? 1 : NSPEC)>(ra, g, key, nkey, q, mu, twice, tacc, lo, hi);
      }
    }
    if (MOM > 0) mom_flush<NSPEC, MM>(rm, tacc, nkey, lo, hi);
    else run_flush<(MOM > 0 ? 1 : NSPEC)>(ra, tacc, g.npole, nkey, lo, hi);
  }
}

}  // namespace
}  // namespace ps

#endif
