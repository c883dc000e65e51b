// ps_bin.cu -- last FFT pass fused with the interlace combine, the window
// compensation and the Legendre-weighted binning; plus the stand-alone
// binning sweep, the geometry sweep and the partial-sum reduction.
//
// Reference: dens_k0's interlace combine (src/multipole.c:462-487),
// count_mode_sim_lin/_log (src/multipole.c:778-1031) and the mode counting
// of powspec_precomp (src/multipole.c:111-257).
//
// Accumulation: every thread walks a run of consecutive modes along x, whose
// |k| grows monotonically, and keeps the run's sums in registers while the
// bin stays the same; on a bin change it adds them to FP32 per-tile
// accumulators in shared memory.  After each tile the touched bins are added
// into this CTA's slice of a partial-sum array in global memory (FP32 pairs), which
// a final kernel reduces over CTAs in a fixed order.
#include "ps_bin_core.cuh"

namespace ps {
namespace {

// Pass C.  Lines of tile: field f, row r -> smem line f * nl + r.
template <int NSPEC, bool STORE, bool P2, int MOM>
__global__ void __launch_bounds__(kFftThreads) k_pass_c(const __grid_constant__ PassCArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, ngk = (ng >> 1) + 1, ls = line_stride(ng, P2), h = ng >> 1;
  // bin mode: a tile is a.ty lines of consecutive ky at one kz; store mode:
  // a.ty lines of consecutive kz at one ky, so that the [x][y][kz] stores
  // of a tile are runs of a.ty consecutive values
  const int nty = STORE ? (ngk + a.ty - 1) / a.ty : (ng + a.ty - 1) / a.ty;
  const int ntile = STORE ? ng * nty : ngk * nty;
  const ModeGeom& g = a.geom;
  const int nacc = NSPEC * g.npole;
  const int nkey = g.nbin * g.nmu;  // accumulator key = k bin * nmu + |mu| bin
  const size_t tile_elems = (size_t)a.nfield * a.ty * ls;  // one ping-pong buffer
  float2* sm2 = sm + tile_elems;  // second FFT buffer (ping-pong)
  float* tacc = reinterpret_cast<float*>(sm + 2 * tile_elems);
  __shared__ int srange[2];
  float2* part = STORE ? nullptr : a.partials + (size_t)blockIdx.x * nacc * nkey;
  if (!STORE) {
    for (int e = threadIdx.x; e < tile_accs<NSPEC, MOM>(g) * nkey; e += blockDim.x) tacc[e] = 0.f;
    if (threadIdx.x == 0) {
      srange[0] = 0x7fffffff;
      srange[1] = -1;
    }
    __syncthreads();
  }
  int ntiles_acc = 0;
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int t0 = tile / nty;
    const int kz = STORE ? (tile - t0 * nty) * a.ty : t0;   // store: first kz
    const int ky0 = STORE ? t0 : (tile - t0 * nty) * a.ty;  // store: the ky
    const int nl = STORE ? min(a.ty, ngk - kz) : min(a.ty, ng - ky0);
    const size_t rstride = STORE ? (size_t)ng * ng : (size_t)ng;  // between lines
    for (int f = 0; f < a.nfield; f++) {
      const float2* src = a.in[f] + ((size_t)kz * ng + ky0) * ng;
      for (int e = threadIdx.x; e < nl * h; e += blockDim.x) {
        const int r = e / h, m = e - r * h;
        const float4 v = __ldcs(reinterpret_cast<const float4*>(src + r * rstride) + m);
        float2* L = sm + (f * nl + r) * ls;
        L[lidx<P2>(2 * m)] = make_float2(v.x, v.y);
        L[lidx<P2>(2 * m + 1)] = make_float2(v.z, v.w);
      }
    }
    __syncthreads();
    const float2* X = P2 ? fft2_lines_pp<4>(sm, sm2, a.plan_full.logn, a.nfield * nl, ls, a.tw_full)
                         : fft_lines_pp(sm, sm2, a.plan_full, a.nfield * nl, ls, a.tw_full);

    if (STORE) {
      // [x][y][kz]: line r holds kz + r; runs of nl consecutive kz per x.
      // Accumulate modes weight by Y_lm(k^) (1 for k_x = k_y = 0,
      // src/mp_template.c:118-121) and add into the field.
      const int jp = dsigned(ky0, ng);
      for (int e = threadIdx.x; e < nl * ng; e += blockDim.x) {
        const int i = e / nl, r = e - i * nl;
        const size_t idx = ((size_t)i * ng + ky0) * ngk + kz + r;
        float2 v = X[r * ls + lidx<P2>(i)];
        if (a.acc_mode) {
          const int ip = dsigned(i, ng);
          const float y = (ip == 0 && jp == 0)
                              ? 1.f
                              : ylm_eval(a.yk, ip * a.kinv[0], jp * a.kinv[1], (kz + r) * a.kinv[2]);
          v = make_float2(v.x * y, v.y * y);
          if (a.acc_mode == 2) {
            const float2 o = a.store[idx];
            v = make_float2(v.x + o.x, v.y + o.y);
          }
        }
        a.store[idx] = v;
      }
      __syncthreads();
      continue;
    }

    int lo = 0x7fffffff, hi = -1;
    bin_lines<NSPEC, P2, MOM>(a, X, ls, kz, ky0, nl, tacc, lo, hi, threadIdx.x, blockDim.x);
    note_range(srange, lo, hi);
    if (++ntiles_acc == kMergeEvery) {
      merge_any<NSPEC, MOM>(tacc, srange, part, g, nkey);
      ntiles_acc = 0;
    } else {
      __syncthreads();
    }
  }
  if (!STORE && ntiles_acc) merge_any<NSPEC, MOM>(tacc, srange, part, g, nkey);
}

// Pass C, pipelined (power-of-two Ng): persistent CTAs, the lines of the next
// tile copied by cp.async.bulk into one stage buffer while the current one is
// transformed (ping-pong between its stage buffer and F) and binned.  Every
// mbarrier wait is bounded; on a timeout the kernel flags a.err, drains its
// copies and stops.
template <int NSPEC, int MOM>
__global__ void __launch_bounds__(kFftThreads, 2) k_pass_c_tma(const __grid_constant__ PassCArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int s_abort;
  __shared__ int srange[2];
  const int ng = a.ng, ngk = (ng >> 1) + 1, ls = line_stride(ng, true);
  const int nty = (ng + a.ty - 1) / a.ty;
  const int ntile = ngk * nty;
  const ModeGeom& g = a.geom;
  const int nacc = NSPEC * g.npole;
  const int nkey = g.nbin * g.nmu;
  const size_t selems = pass_c_tma_elems(ng, a.ty, a.nfield);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  float2* stage[2];
  stage[0] = reinterpret_cast<float2*>(smraw + 128);
  stage[1] = stage[0] + selems;
  float2* F = stage[1] + selems;
  float* tacc = reinterpret_cast<float*>(F + selems);
  float2* part = a.partials + (size_t)blockIdx.x * nacc * nkey;
  for (int e = threadIdx.x; e < tile_accs<NSPEC, MOM>(g) * nkey; e += blockDim.x) tacc[e] = 0.f;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort = 0;
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
  int nissued = 0;  // copies issued (thread 0)
  auto issue = [&](int tile, int s) {
    nissued++;
    const int kz = tile / nty, ky0 = (tile - kz * nty) * a.ty;
    const int nl = min(a.ty, ng - ky0);
    mbar_expect_tx(&bar[s], (uint32_t)(a.nfield * nl * ng * 8));
    if (a.stall && blockIdx.x == 0 && nissued == 2) return;  // test hook: no copy
    for (int f = 0; f < a.nfield; f++)
      for (int r = 0; r < nl; r++)
        bulk_g2s(stage[s] + (size_t)(f * nl + r) * ng, a.in[f] + ((size_t)kz * ng + ky0 + r) * ng,
                 (uint32_t)(ng * 8), &bar[s]);
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < ntile) issue(blockIdx.x, 0);
  int it = 0, ntiles_acc = 0;
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x, it++) {
    const int s = it & 1;
    if (threadIdx.x == 0 && tile + (int)gridDim.x < ntile) {
      fence_proxy_async();
      issue(tile + gridDim.x, s ^ 1);
    }
    if (!pipe_wait(bar, it, a.err, &s_abort, wait_limit(a.wait_limit))) break;
    const int kz = tile / nty, ky0 = (tile - kz * nty) * a.ty;
    const int nl = min(a.ty, ng - ky0);
    const float2* X = fft2_pp_from<false, 4>(stage[s], ng, 0, F, a.plan_full.logn, a.nfield * nl,
                                             ls, a.tw_full);
    int lo = 0x7fffffff, hi = -1;
    bin_lines<NSPEC, true, MOM>(a, X, ls, kz, ky0, nl, tacc, lo, hi, threadIdx.x, blockDim.x);
    note_range(srange, lo, hi);
    if (++ntiles_acc == kMergeEvery) {
      merge_any<NSPEC, MOM>(tacc, srange, part, g, nkey);
      ntiles_acc = 0;
    } else {
      __syncthreads();
    }
  }
  if (ntiles_acc && !s_abort) merge_any<NSPEC, MOM>(tacc, srange, part, g, nkey);
  // never exit with a bulk copy in flight into this CTA's memory
  if (threadIdx.x == 0 && s_abort) pipe_drain(bar, nissued, wait_limit(a.wait_limit));
}

// Stand-alone binning of FFTW-layout fields [x][y][kz]: one line per (x, y).
__global__ void __launch_bounds__(kFftThreads) k_bin_fields(const __grid_constant__ BinFieldArgs a) {
  extern __shared__ float smf[];
  const int ng = a.ng, ngk = (ng >> 1) + 1;
  const ModeGeom& g = a.geom;
  const int nacc = g.npole;
  float* tacc = smf;
  __shared__ int srange[2];
  float2* part = a.partials + (size_t)blockIdx.x * nacc * g.nbin;
  for (int e = threadIdx.x; e < nacc * g.nbin; e += blockDim.x) tacc[e] = 0.f;
  if (threadIdx.x == 0) {
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
  const int chunks = (ngk + kRun - 1) / kRun;
  const int rows_per_tile = max(1, kFftThreads / chunks);
  const int nrows = ng * ng;
  for (int row0 = blockIdx.x * rows_per_tile; row0 < nrows; row0 += gridDim.x * rows_per_tile) {
    int lo = 0x7fffffff, hi = -1;
    for (int e = threadIdx.x; e < rows_per_tile * chunks; e += blockDim.x) {
      const int rr = e / chunks;
      const int row = row0 + rr;
      if (row >= nrows) continue;
      const int i = row / ng, j = row - i * ng;
      const int k0 = (e - rr * chunks) * kRun;
      const int ip = dsigned(i, ng), jp = dsigned(j, ng);
      const int ia = abs(ip), ja = abs(jp);
      const float kxf = g.vec[0] * (float)ip, kyf = g.vec[1] * (float)jp;
      const float wij = __ldg(&g.win[i]) * __ldg(&g.win[ng + j]);
      RunAcc<1> ra;
      ra.bin = -1;
#pragma unroll
      for (int l = 0; l < kMaxPole; l++) ra.v[0][l] = 0.f;
      const int kend = min(k0 + kRun, ngk);
      for (int k = k0; k < kend; k++) {
        const int n = ia * ia + ja * ja + k * k;
        if (n == 0) continue;
        const int b = mode_bin(g, ia, ja, k, n);
        if (b < 0) continue;
        const bool twice = !(k == 0 || 2 * k == ng);
        const size_t idx = (size_t)row * ngk + k;
        const float2 A = a.f1[idx], B = a.f2[idx];
        const float wv = wij * __ldg(&g.win[2 * ng + k]) * (twice ? 2.f : 1.f);
        float p[1] = {(A.x * B.x + A.y * B.y) * wv};
        const float kzf = g.vec[2] * (float)k;
        const float mu = (kxf * g.los[0] + kyf * g.los[1] + kzf * g.los[2]) *
                         rsqrtf(kxf * kxf + kyf * kyf + kzf * kzf);
        run_add<1>(ra, g, b, g.nbin, p, mu, twice, tacc, lo, hi);
      }
      run_flush<1>(ra, tacc, g.npole, g.nbin, lo, hi);
    }
    note_range(srange, lo, hi);
    merge_tile(tacc, srange, part, nacc, g.nbin);
  }
}

// Geometry sweep (FP64, once per context): counts with weight 1 on the k = 0
// and Nyquist planes and 2 between (DC included, src/multipole.c:144-239),
// sum of weight * |k|, and sum of weight * L_l(mu) without DC
// (src/multipole.c:806-880), mu = (k . los) / |k| in FP64 as the reference.
__global__ void __launch_bounds__(256) k_geometry(const __grid_constant__ GeomArgs a) {
  extern __shared__ double smd[];
  const ModeGeom& g = a.geom;
  const int ng = a.ng, ngk = (ng >> 1) + 1, h = ngk;
  const int nbin = g.nbin, npole = g.npole;
  double* s_ks = smd;                           // [nbin]
  double* s_lc = smd + nbin;                    // [npole][nbin]
  unsigned long long* s_cnt =
      reinterpret_cast<unsigned long long*>(smd + (size_t)(1 + npole) * nbin);  // [nbin]
  for (int e = threadIdx.x; e < (2 + npole) * nbin; e += blockDim.x) smd[e] = 0.0;
  __syncthreads();
  const size_t nmodes = (size_t)ng * ng * ngk;
  for (size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x; m < nmodes;
       m += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(m % ngk);
    const size_t row = m / ngk;
    const int i = (int)(row / ng), j = (int)(row % ng);
    const int ip = dsigned(i, ng), jp = dsigned(j, ng);
    const int ia = abs(ip), ja = abs(jp);
    const int n = ia * ia + ja * ja + k * k;
    const int b = mode_bin(g, ia, ja, k, n);
    if (b < 0) continue;
    const bool twice = !(k == 0 || 2 * k == ng);
    const double w = twice ? 2.0 : 1.0;
    double km2 = __dadd_rn(g.ksq[ia], g.ksq[h + ja]);
    if (k) km2 = __dadd_rn(km2, g.ksq[2 * h + k]);
    const double kmod = __dsqrt_rn(km2);
    atomicAdd(&s_cnt[b], twice ? 2ull : 1ull);
    atomicAdd(&s_ks[b], w * (g.logscale ? 0.5 * log10(km2) : kmod));
    if (n == 0) continue;
    const double ki = __dmul_rn(a.vec[0], (double)ip), kj = __dmul_rn(a.vec[1], (double)jp);
    const double kk = __dmul_rn(a.vec[2], (double)k);
    double num = __dadd_rn(__dmul_rn(ki, a.los[0]), __dmul_rn(kj, a.los[1]));
    if (k) num = __dadd_rn(num, __dmul_rn(kk, a.los[2]));
    const double mu = __ddiv_rn(num, kmod);
    const double x2 = mu * mu;
    for (int l = 0; l < npole; l++) {
      const int ell = g.poles[l];
      if (twice && (ell & 1)) continue;
      double L;
      switch (ell) {
        case 0: L = 1.0; break;
        case 1: L = mu; break;
        case 2: L = 1.5 * x2 - 0.5; break;
        case 3: L = 2.5 * mu * (x2 - 0.6); break;
        case 4: L = 4.375 * x2 * x2 - 3.75 * x2 + 0.375; break;
        case 5: L = 8.75 * mu * (0.9 * x2 * x2 - x2 + 0.21428571428571427); break;
        default: L = 14.4375 * x2 * x2 * x2 - 19.6875 * x2 * x2 + 6.5625 * x2 - 0.3125; break;
      }
      atomicAdd(&s_lc[l * nbin + b], w * L);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbin; b += blockDim.x) {
    if (s_cnt[b]) {
      atomicAdd(&a.cnt[b], s_cnt[b]);
      atomicAdd(&a.ksum[b], s_ks[b]);
    }
    for (int l = 0; l < npole; l++)
      if (s_lc[l * nbin + b] != 0.0) atomicAdd(&a.lcnt[l * nbin + b], s_lc[l * nbin + b]);
  }
}

// out[j] = sum over the grid rows of part[row][j], in a fixed order: warp w
// of a block adds rows w, w + 16, ... of 32 consecutive columns (coalesced
// 256-byte rows), then the 16 warp sums are added in warp order.  The
// binning partials are FP32 pairs, added as pairs (FP64 once per column);
// FP64 partials (k_dc_sum) are added in FP64.
constexpr int kReduceWarps = 16;
__global__ void __launch_bounds__(32 * kReduceWarps) k_reduce(const float2* __restrict__ part, int grid,
                                                             int width, double* __restrict__ out) {
  __shared__ float2 sh[kReduceWarps][33];
  const int j = blockIdx.x * 32 + threadIdx.x, w = threadIdx.y;
  float h = 0.f, l = 0.f;
  if (j < width) {
#pragma unroll 4
    for (int gi = w; gi < grid; gi += kReduceWarps) {
      const float2 v = __ldg(&part[(size_t)gi * width + j]);
      df_add(h, l, v.x, v.y);
    }
  }
  sh[w][threadIdx.x] = make_float2(h, l);
  __syncthreads();
  if (w == 0 && j < width) {
    float th = sh[0][threadIdx.x].x, tl = sh[0][threadIdx.x].y;
    for (int q = 1; q < kReduceWarps; q++) df_add(th, tl, sh[q][threadIdx.x].x, sh[q][threadIdx.x].y);
    out[j] = (double)th + (double)tl;
  }
}
__global__ void __launch_bounds__(32 * kReduceWarps) k_reduce_f64(const double* __restrict__ part, int grid,
                                                                 int width, double* __restrict__ out) {
  __shared__ double sh[kReduceWarps][33];
  const int j = blockIdx.x * 32 + threadIdx.x, w = threadIdx.y;
  double s = 0.0;
  if (j < width) {
#pragma unroll 4
    for (int gi = w; gi < grid; gi += kReduceWarps) s += __ldg(&part[(size_t)gi * width + j]);
  }
  sh[w][threadIdx.x] = s;
  __syncthreads();
  if (w == 0 && j < width) {
    double t = sh[0][threadIdx.x];
    for (int q = 1; q < kReduceWarps; q++) t += sh[q][threadIdx.x];
    out[j] = t;
  }
}

}  // namespace

int pass_c_moments(const int* poles, int npole) {
  int lmax = 0;
  for (int l = 0; l < npole; l++) {
    if (poles[l] & 1) return 0;
    lmax = poles[l] > lmax ? poles[l] : lmax;
  }
  const int mom = lmax / 2 + 1;
  return mom < 2 ? 2 : mom;
}

size_t pass_c_smem(int ng, int ty, int nfield, int nacc, int nbin, bool pow2) {
  return 2 * (size_t)nfield * ty * line_stride(ng, pow2) * sizeof(float2) +
         (size_t)nacc * nbin * sizeof(float);
}

size_t pass_c_tma_smem(int ng, int ty, int nfield, int nacc, int nkey) {
  return 128 + 3 * pass_c_tma_elems(ng, ty, nfield) * sizeof(float2) + (size_t)nacc * nkey * sizeof(float);
}

namespace {
template <int NSPEC, bool STORE, bool P2, int MOM = 0>
void launch_c(const PassCArgs& a, unsigned grid, size_t smem, cudaStream_t s) {
  cudaFuncSetAttribute(k_pass_c<NSPEC, STORE, P2, MOM>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_pass_c<NSPEC, STORE, P2, MOM><<<grid, kFftThreads, smem, s>>>(a);
}
template <int MOM, bool P2>
void launch_c_bin(const PassCArgs& a, size_t smem, cudaStream_t s) {
  switch (a.nspec) {
    case 1: launch_c<1, false, P2, MOM>(a, (unsigned)a.grid, smem, s); break;
    case 2: launch_c<2, false, P2, MOM>(a, (unsigned)a.grid, smem, s); break;
    default: launch_c<3, false, P2, MOM>(a, (unsigned)a.grid, smem, s); break;
  }
}
template <int MOM>
void launch_c_tma(const PassCArgs& a, size_t smem, cudaStream_t s) {
#define PS_C_TMA(NS)                                                                    \
  cudaFuncSetAttribute(k_pass_c_tma<NS, MOM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)smem);                                                      \
  k_pass_c_tma<NS, MOM><<<(unsigned)a.grid, kFftThreads, smem, s>>>(a);
  switch (a.nspec) {
    case 1: PS_C_TMA(1); break;
    case 2: PS_C_TMA(2); break;
    default: PS_C_TMA(3); break;
  }
#undef PS_C_TMA
}
template <bool P2>
void launch_c_p(const PassCArgs& a, cudaStream_t s) {
  const int ngk = a.ng / 2 + 1;
  if (a.store) {  // tiles of a.ty consecutive kz at one ky
    const unsigned ntile = (unsigned)(a.ng * ((ngk + a.ty - 1) / a.ty));
    launch_c<1, true, P2>(a, ntile, pass_c_smem(a.ng, a.ty, a.nfield, 0, 0, P2), s);
    return;
  }
  const int nacc_t = a.nspec * pass_c_accs(a.geom.npole, a.mom);
  const size_t smem = pass_c_smem(a.ng, a.ty, a.nfield, nacc_t, a.geom.nbin * a.geom.nmu, P2);
  if (P2 && a.pipe) {
    const size_t sm2 = pass_c_tma_smem(a.ng, a.ty, a.nfield, nacc_t, a.geom.nbin * a.geom.nmu);
    switch (a.mom) {
      case 2: launch_c_tma<2>(a, sm2, s); break;
      case 3: launch_c_tma<3>(a, sm2, s); break;
      case 4: launch_c_tma<4>(a, sm2, s); break;
      default: launch_c_tma<0>(a, sm2, s); break;
    }
    return;
  }
  switch (a.mom) {
    case 2: launch_c_bin<2, P2>(a, smem, s); break;
    case 3: launch_c_bin<3, P2>(a, smem, s); break;
    case 4: launch_c_bin<4, P2>(a, smem, s); break;
    default: launch_c_bin<0, P2>(a, smem, s); break;
  }
}
}  // namespace

int launch_pass_c(const PassCArgs& a, cudaStream_t s) {
  if (a.twl && !a.store && launch_pass_c_w(a, s)) return 1;
  if (a.twl && a.store && launch_pass_c_ws(a, s)) return 1;
  if (a.plan_full.logn >= 0)
    launch_c_p<true>(a, s);
  else
    launch_c_p<false>(a, s);
  return 1;
}

int launch_bin_fields(const BinFieldArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)a.geom.npole * a.geom.nbin * sizeof(float);
  cudaFuncSetAttribute(k_bin_fields, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_bin_fields<<<(unsigned)a.grid, kFftThreads, smem, s>>>(a);
  return 1;
}

int launch_geometry(const GeomArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)(2 + a.geom.npole) * a.geom.nbin * sizeof(double);
  cudaFuncSetAttribute(k_geometry, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t nmodes = (size_t)a.ng * a.ng * (a.ng / 2 + 1);
  size_t blocks = (nmodes + 255) / 256;
  if (blocks > (size_t)nsm * 4) blocks = (size_t)nsm * 4;
  k_geometry<<<(unsigned)blocks, 256, smem, s>>>(a);
  return 1;
}

int launch_reduce_f64(const double* part, int grid, int width, double* out, cudaStream_t s) {
  k_reduce_f64<<<(width + 31) / 32, dim3(32, kReduceWarps), 0, s>>>(part, grid, width, out);
  return 1;
}

int launch_reduce(const float2* part, int grid, int width, double* out, cudaStream_t s) {
  k_reduce<<<(width + 31) / 32, dim3(32, kReduceWarps), 0, s>>>(part, grid, width, out);
  return 1;
}

}  // namespace ps
