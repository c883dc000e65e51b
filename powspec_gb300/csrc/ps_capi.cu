// ps_capi.cu -- context, host-side tables and the extern "C" entry points of
// libpowspec_gpu.so (declared in include/powspec_gpu.h).
//
// Host work here is O(ng) or O(nbin) per call plus one O(ng^2) table per
// context; every O(ng^3) or O(N) loop runs on the GPU.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "powspec_gpu.h"

#include "ps_internal.h"

using namespace ps;

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

// 1-D window / alias factor (src/multipole.c:46-100), FP64.  Note that the
// reference passes the SIGNED frequency: for negative arguments the x > 0.01
// test fails and the Taylor branch is taken, which the tables reproduce.
double alias_corr(int interlace, int assign, double pik) {
  double fac;
  if (interlace) {
    if (pik > 0.01) {
      fac = pik / sin(pik);
    } else {
      const double t = pik * pik;
      fac = 1 + 0x1.5555555555555p-3 * t + 0x1.3e93e93e93e94p-6 * t * t +
            0x1.0cbb766210cbbp-9 * t * t * t;
    }
    fac *= fac;
    switch (assign) {
      case 0: return fac;
      case 1: return fac * fac;
      case 2: return fac * fac * fac;
      default: fac *= fac; return fac * fac;
    }
  }
  if (pik > 0.01) {
    fac = sin(pik);
  } else {
    const double t = pik * pik;
    fac = (1 - 0x1.5555555555555p-3 * t + 0x1.1111111111111p-7 * t * t -
           0x1.a01a01a01a01ap-13 * t * t * t) * pik;
  }
  fac *= fac;
  switch (assign) {
    case 0: return 1;
    case 1: return 1 / (1 - 0x1.5555555555555p-1 * fac);
    case 2: return 1 / (1 - fac + 0x1.1111111111111p-3 * fac * fac);
    default:
      return 1 / (1 - 0x1.5555555555555p+0 * fac + 0.4 * fac * fac -
                  0x1.a01a01a01a01ap-7 * fac * fac * fac);
  }
}

bool make_plan(int n, FftPlan& p) {
  p.n = n;
  p.npass = 0;
  p.logn = -1;
  if ((n & (n - 1)) == 0) {
    int l = 0;
    while ((1 << l) < n) l++;
    p.logn = l;
  }
  int m = n, e = 0;
  while (m % 2 == 0) { m /= 2; e++; }
  while (e > 0) {
    int r;
    if (e == 4) r = 4;
    else if (e >= 3) r = 8;
    else if (e == 2) r = 4;
    else r = 2;
    if (p.npass >= kMaxPlan) return false;
    p.radix[p.npass++] = r;
    e -= (r == 8) ? 3 : (r == 4) ? 2 : 1;
  }
  while (m % 3 == 0) { if (p.npass >= kMaxPlan) return false; p.radix[p.npass++] = 3; m /= 3; }
  while (m % 5 == 0) { if (p.npass >= kMaxPlan) return false; p.radix[p.npass++] = 5; m /= 5; }
  return m == 1;
}

// Table of the warp transform of length n held as L lanes x V values:
// t[k1 L + l] = exp(-2 pi i l k1 / n), l < L, k1 < V (l k1 < n), FP64
// angles reduced as above.
std::vector<float2> warp_twiddles(int n) {
  int L = 0, V = 0;
  wfft_shape(n, &L, &V);
  auto w = [n](int m) {  // W_n^m, the angle reduced to [0, pi]
    m %= n;
    const int mm = (2 * m <= n) ? m : n - m;
    const double a = 2.0 * kPi * (double)mm / (double)n;
    const double sn = (2 * m <= n) ? -sin(a) : sin(a);
    return make_float2((float)cos(a), (float)sn);
  };
  std::vector<float2> t((size_t)L * V);
  for (int k1 = 0; k1 < V; k1++)
    for (int l = 0; l < L; l++) t[(size_t)k1 * L + l] = w(l * k1);
  // the pair-of-warps form (L = 64 lanes over two warps) ends with 64-point
  // DFTs split in two: W_64^k2 = W_n^(32 k2) after the table
  if (L == 64)
    for (int k2 = 0; k2 < 32; k2++) t.push_back(w(32 * k2));
  return t;
}

std::vector<float2> twiddles(int n) {
  std::vector<float2> t(n);
  for (int m = 0; m < n; m++) {
    // angle reduced to [0, pi] for accuracy, sign restored
    const int mm = (2 * m <= n) ? m : n - m;
    const double a = 2.0 * kPi * (double)mm / (double)n;
    const double s = (2 * m <= n) ? -sin(a) : sin(a);
    t[m] = make_float2((float)cos(a), (float)s);
  }
  return t;
}

}  // namespace

struct ps_gpu_ctx {
  ps_gpu_params p;
  int ng = 0, ngk = 0, nbin = 0, nfield = 0, mpc = 1, nsm = 0;
  size_t ntot = 0, ncx = 0;
  cudaStream_t stream = nullptr;
  std::vector<double> kedge, kcen, km, lcnt;
  std::vector<uint64_t> cnt;
  unsigned long long* grid[4] = {nullptr, nullptr, nullptr, nullptr};
  float2* cbuf[4] = {nullptr, nullptr, nullptr, nullptr};
  short* d_bintab = nullptr;
  double* d_ksq = nullptr;
  float* d_win = nullptr;
  float2* d_phase = nullptr;
  float2* d_tw_full = nullptr;
  float2* d_tw_half = nullptr;
  FftPlan plan_full{}, plan_half{};
  ModeGeom geom{};
  int nspec = 0, spec_a[3] = {0, 0, 0}, spec_b[3] = {0, 0, 0}, spec_cat[3] = {0, 0, 0};
  int ty_a = 1, tx_b = 1, ty_c = 1, grid_c = 1;
  int ty_ap = 1, tx_bp = 1;  // tiles of the pipelined passes
  bool radix32_b = false;
  // tuning knobs (ps_gpu_autotune): z-pass variant, gather CTA size (0: by
  // density), pipelined pass C on / off
  bool radix32_a = false;
  int gather_threads = 0;
  unsigned gather_sparse_max = 512;  // records per tile up to which lane groups are used
  int gather_region = -1;  // region gather: 1 on, 0 off, -1 by density (TSC/PCS, 16^3 tiles)
  bool pipe_c_on = true;
  int ty_ct = 1, grid_ct = 0;  // pipelined pass C (grid 0: not available)
  // warp-register transforms (ps_wfft.cu): bit 0 z pass, 1 y pass, 2 x pass
  // + binning, each where the mesh size has one; their tables; the x pass's
  // persistent grid (0: not available)
  int wfft = 0;
  int stall = 0;  // test hook: poll limit of the next evaluation's stalled pipeline
  float2* d_twl_half = nullptr;
  float2* d_twl_full = nullptr;
  int grid_cw = 0;
  int wpc_cw = 4;  // warps per CTA of the warp x pass
  int nmu = 1;               // |mu| sub-bins of the binning pass
  // tile assignment
  int gT = 0, gnt = 0;
  size_t nkeys = 0, gcap = 0;
  unsigned *d_hist = nullptr, *d_bsum = nullptr, *d_rank = nullptr;
  void* d_rec = nullptr;
  unsigned long long* d_region = nullptr;  // region sums of the region gather
  size_t region_bytes = 0;
  // learned correction (ps_gpu_execute_learned): kcen, cnt, lcnt on the
  // device, cell features / BF16 copy / corrections, corrected P_l
  double* d_lgeo = nullptr;
  float* d_lx = nullptr;
  void* d_lxb = nullptr;
  float* d_lc = nullptr;
  double* d_lout = nullptr;
  double* h_lout = nullptr;
  int lcells = 0;
  // staged input (ps_gpu_stage_aos): two device slots filled on a copy
  // stream; copied[s] marks a slot's copy done, used[s] the end of the
  // assignment kernels that read it
  cudaStream_t copy_stream = nullptr;
  void* d_slot[2] = {nullptr, nullptr};
  size_t slot_bytes[2] = {0, 0}, slot_n[2] = {0, 0};
  cudaEvent_t copied[2] = {nullptr, nullptr}, used[2] = {nullptr, nullptr};
  bool slot_full[2] = {false, false};
  // survey normalisation per catalogue (ps_gpu_set_survey)
  bool survey[2] = {false, false};
  double survey_shot[2] = {0, 0}, survey_norm[2] = {0, 0};
  double survey_origin[3] = {0, 0, 0};  // box corner, the observer at 0
  // survey multipoles l > 0: stored fields F_0 and F_l per catalogue, an
  // r2c scratch (3 half-complex fields) and a weighted real mesh
  void* d_yama = nullptr;
  size_t yama_bytes = 0;
  double* d_dc = nullptr;  // F_l at k = 0 per catalogue [pole][cat], FP64
  double* d_dcpart = nullptr;  // its per-CTA partial sums
  bool yama_last = false;  // the last execute took the survey-multipole path
  int last_cat = -1;
  Particles last_pt{};
  std::vector<double> kmu;   // last execute's raw (k, |mu|) sums
  double* d_part = nullptr;
  double* d_sums = nullptr;
  double* d_wsum = nullptr;  // [2 cats][2], then [2 cats] int64 mean cell values
  double* d_wpart = nullptr; // [2 * kAssignMaxBlocks]
  int* d_err = nullptr;      // [2 cats]
  double* h_out = nullptr;   // pinned: sums + wsum + err (+ Re F_l(0) [pole][cat])
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  int assigned[2] = {0, 0};
  size_t npart[2] = {0, 0};
  cudaEvent_t ev[8] = {};
  // a learned evaluation launched and not yet finished (ps_gpu_learned_launch)
  cudaEvent_t ev_done = nullptr;  // its results are on the host
  bool learned_pending = false;
  size_t npart_pending[2] = {0, 0};
  bool assign_timed_pending = false;  // its assignment's events can be read at finish
  unsigned assign_gen = 0, assign_gen_pending = 0;  // assignments started
  bool assign_started = false;
  float timings[6] = {0, 0, 0, 0, 0, 0};
  int launches = 0;
  char err[512] = {0};
};

namespace {

int fail(ps_gpu_ctx* c, int code, const char* fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof c->err, fmt, ap);
    va_end(ap);
  }
  return code;
}

// A failed allocation is PS_GPU_ERR_MEMORY (the reference's
// POWSPEC_ERR_MEMORY, which it raises with exit() inside its OpenMP region,
// src/multipole.c:121-126); any other CUDA failure is PS_GPU_ERR_CUDA.
#define CU(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      (void)cudaGetLastError();                                                       \
      return fail(c, e_ == cudaErrorMemoryAllocation ? PS_GPU_ERR_MEMORY : PS_GPU_ERR_CUDA, \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                    \
    }                                                                                 \
  } while (0)

// Test hook of ps_gpu_debug_fail_alloc: n > 0 makes the n-th next device or
// pinned allocation of this file fail as out of memory (a fake of the
// failing call; the device is never touched by it).
std::atomic<int> g_fail_alloc{0};
bool fake_alloc_failure() {
  int n = g_fail_alloc.load();
  while (n > 0 && !g_fail_alloc.compare_exchange_weak(n, n - 1)) {
  }
  return n == 1;
}
template <typename T>
cudaError_t dev_malloc(T** p, size_t bytes) {
  if (fake_alloc_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc((void**)p, bytes);
}
template <typename T>
cudaError_t host_malloc(T** p, size_t bytes) {
  if (fake_alloc_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost((void**)p, bytes);
}

template <typename T>
int upload(ps_gpu_ctx* c, T** dst, const std::vector<T>& v) {
  CU(dev_malloc(dst, sizeof(T) * (v.empty() ? 1 : v.size())));
  if (!v.empty()) CU(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return 0;
}

// Bin of a squared wave number with the reference's FP64 sequence
// (src/multipole.c:147-158).
int ref_bin(const ps_gpu_ctx* c, double km2) {
  const double kmod = c->p.logscale ? 0.5 * log10(km2) : sqrt(km2);
  if (kmod < c->kedge[0] || kmod >= c->kedge[c->nbin]) return -1;
  const int b = (int)((kmod - c->kedge[0]) / c->p.dk);
  return (b < 0 || b >= c->nbin) ? -1 : b;
}

// Tiles of the pipelined z and y passes for their current variants:
// kPipeElems complex values per tile (radix 16, two CTAs per SM) or twice
// that (radix 32, one CTA per SM).
void plan_pipes(ps_gpu_ctx* c) {
  const int ng = c->ng;
  c->ty_ap = std::max(1, std::min(ng, (c->radix32_a ? 2 * kPipeElems : kPipeElems) / (ng / 2)));
  c->tx_bp = std::max(1, std::min(ng, (c->radix32_b ? 2 * kPipeElems : kPipeElems) / ng));
}

// Tiles and persistent grids of both pass-C kernels for the current number
// of (k, mu) accumulators.  Plain kernel: kPassCElems complex per tile, as
// many CTAs per SM as fit.  Pipelined kernel (power-of-two Ng): the largest
// tile (rows per field) that lets two CTAs share an SM, else one CTA.
// Passes with a warp-register form for the context (ps_gpu_set_warp_fft's
// mask): z (bit 0), y (bit 1) and x (bit 2, when its CTAs fit).
int warp_avail(const ps_gpu_ctx* c) {
  int m = c->d_twl_half ? 1 : 0;
  if (c->d_twl_full) m |= 2 | (c->grid_cw > 0 ? 4 : 0);
  return m;
}

int plan_pass_c(ps_gpu_ctx* c) {
  const int ng = c->ng;
  const int nacc = c->nspec * pass_c_accs(c->p.npole, pass_c_moments(c->p.poles, c->p.npole));
  const int nkey = c->nbin * c->nmu;
  c->ty_c = std::max(1, std::min(ng, kPassCElems / (c->nfield * ng)));
  const size_t smem_c = pass_c_smem(ng, c->ty_c, c->nfield, nacc, nkey, c->plan_full.logn >= 0);
  if (smem_c > 227 * 1024)
    return fail(c, PS_GPU_ERR_ARG, "too many (k, mu) bins (%d) for the binning pass", nkey);
  const int per_sm = std::max(1, std::min(4, (int)((228 * 1024) / (smem_c + 2048))));
  const int ntile_c = c->ngk * ((ng + c->ty_c - 1) / c->ty_c);
  c->grid_c = std::min(ntile_c, c->nsm * per_sm);
  c->grid_ct = 0;
  if (c->plan_full.logn >= 0) {
    const size_t half = 113 * 1024, full = 227 * 1024;
    int ty = std::max(1, std::min(ng, kPassCElems / (c->nfield * ng)));
    while (ty > 1 && pass_c_tma_smem(ng, ty, c->nfield, nacc, nkey) > half) ty >>= 1;
    const size_t sm = pass_c_tma_smem(ng, ty, c->nfield, nacc, nkey);
    if (sm <= full) {
      const int per = sm <= half ? 2 : 1;
      c->ty_ct = ty;
      c->grid_ct = std::min(c->ngk * ((ng + ty - 1) / ty), c->nsm * per);
    }
  }
  // warp x pass: as many persistent CTAs per SM as are resident (shared
  // memory and registers of the instance the launch picks), of the CTA size
  // (4 warps, or 16 sharing the tile sums: one spectrum of the poles 0, 2,
  // 4 at Ng = 256) that keeps the most warps resident (the larger on a tie).
  c->grid_cw = 0;
  c->wpc_cw = 4;
  if (c->d_twl_full && ng == 2048) {
    // pairs of warps: as many as shared memory holds, up to 8 (16 warps)
    for (int wpc = 16; wpc >= 2; wpc -= 2) {
      const size_t smw = pass_c_w_smem(ng, c->nfield, nacc, nkey, wpc);
      if (smw && smw <= 227 * 1024) {
        c->wpc_cw = wpc;
        c->grid_cw = c->nsm;
        break;
      }
    }
  } else if (c->d_twl_full) {
    const int mom = pass_c_moments(c->p.poles, c->p.npole);
    const bool big_ok = ng == 256 && c->nspec == 1 && mom == 3;
    int best = 0;
    for (int wpc : {4, 16}) {
      if (wpc == 16 && !big_ok) continue;
      const size_t smw = pass_c_w_smem(ng, c->nfield, nacc, nkey, wpc);
      if (!smw || smw > 227 * 1024) continue;
      // resident CTAs of the instance the launch will pick (its registers
      // and shared memory); the shared-memory estimate without a device
      PassCArgs q;
      memset(&q, 0, sizeof q);
      q.ng = ng;
      q.nfield = c->nfield;
      q.nspec = c->nspec;
      q.mom = mom;
      q.wpc = wpc;
      q.geom = c->geom;
      q.geom.nmu = c->nmu;
      int per = pass_c_w_per_sm(q);
      if (per < 1) {
        per = std::max(1, (int)((228 * 1024) / (smw + 1024)));
        per = std::min(per, wpc == 16 ? 2 : 2048 / (32 * wpc));
      }
      if (per * wpc >= best) {  // the larger CTA on a tie: fewer partial slices
        best = per * wpc;
        c->wpc_cw = wpc;
        c->grid_cw = c->nsm * per;
      }
    }
  }
  return 0;
}

// Per-CTA partial sums, reduced sums and the pinned host copy, sized for
// nspec * npole * nbin * nmu accumulators.
int alloc_accum(ps_gpu_ctx* c) {
  const size_t width = (size_t)c->nspec * c->p.npole * c->nbin * c->nmu;
  if (c->d_part) cudaFree(c->d_part);
  if (c->d_sums) cudaFree(c->d_sums);
  if (c->h_out) cudaFreeHost(c->h_out);
  c->d_part = nullptr;
  c->d_sums = nullptr;
  c->h_out = nullptr;
  CU(dev_malloc(&c->d_part,
                sizeof(double) * (size_t)std::max({c->grid_c, c->grid_ct, c->grid_cw}) * width));
  CU(dev_malloc(&c->d_sums, sizeof(double) * width));
  CU(host_malloc(&c->h_out, sizeof(double) * (width + 8 + 2 * kMaxPole)));
  return 0;
}

int validate(ps_gpu_ctx* c, const ps_gpu_params* p) {
  if (p->ng < 4 || p->ng % 2) return fail(c, PS_GPU_ERR_ARG, "GRID_SIZE must be even and >= 4: %d", p->ng);
  if (p->assign < 0 || p->assign > 3) return fail(c, PS_GPU_ERR_ARG, "invalid PARTICLE_ASSIGN: %d", p->assign);
  if (p->ncat < 1 || p->ncat > 2) return fail(c, PS_GPU_ERR_ARG, "number of catalogues must be 1 or 2");
  for (int d = 0; d < 3; d++)
    if (!(p->box[d] > 0)) return fail(c, PS_GPU_ERR_ARG, "BOX_SIZE must be positive");
  if (!(p->dk > 0)) return fail(c, PS_GPU_ERR_ARG, "BIN_SIZE must be positive");
  if (p->npole < 1 || p->npole > kMaxPole) return fail(c, PS_GPU_ERR_ARG, "invalid number of multipoles");
  for (int l = 0; l < p->npole; l++) {
    if (p->poles[l] < 0 || p->poles[l] > 6) return fail(c, PS_GPU_ERR_ARG, "MULTIPOLE must be between 0 and 6");
    if (l && p->poles[l] <= p->poles[l - 1]) return fail(c, PS_GPU_ERR_ARG, "MULTIPOLE must be sorted and unique");
  }
  return 0;
}

}  // namespace

extern "C" {

int ps_gpu_create(const ps_gpu_params* params, ps_gpu_ctx** out) {
  if (!params || !out) return PS_GPU_ERR_ARG;
  *out = nullptr;
  ps_gpu_ctx* c = new (std::nothrow) ps_gpu_ctx();
  if (!c) return PS_GPU_ERR_MEMORY;
  c->p = *params;
  const ps_gpu_params& p = c->p;
  int rc = validate(c, &p);
  if (rc) { *out = c; return rc; }
  *out = c;
  c->ng = p.ng;
  c->ngk = p.ng / 2 + 1;
  c->ntot = (size_t)p.ng * p.ng * p.ng;
  c->ncx = (size_t)p.ng * p.ng * c->ngk;
  c->mpc = p.interlace ? 2 : 1;
  c->nfield = p.ncat * c->mpc;
  if (!make_plan(p.ng, c->plan_full) || !make_plan(p.ng / 2, c->plan_half))
    return fail(c, PS_GPU_ERR_ARG, "GRID_SIZE/2 must be a product of 2, 3 and 5: %d", p.ng);
  if ((size_t)c->nfield * p.ng > (size_t)2 * kPassCElems)
    return fail(c, PS_GPU_ERR_ARG, "GRID_SIZE %d too large for %d fields", p.ng, c->nfield);
  c->gT = gather_tile(p.ng);
  if (!c->gT || p.ng > 32767)
    return fail(c, PS_GPU_ERR_ARG, "GRID_SIZE %d: needs a divisor in [4, 16] with at least 2 tiles", p.ng);
  c->gnt = p.ng / c->gT;
  c->nkeys = gather_keys(p.ng);

  // spectra: autos, then the cross (src/multipole.c:1221-1226)
  for (int k = 0; k < p.ncat; k++)
    if (p.isauto[k]) { c->spec_a[c->nspec] = k; c->spec_b[c->nspec] = k; c->spec_cat[c->nspec] = k; c->nspec++; }
  if (p.ncat == 2 && p.iscross) { c->spec_a[c->nspec] = 0; c->spec_b[c->nspec] = 1; c->spec_cat[c->nspec] = -1; c->nspec++; }
  if (!c->nspec) return fail(c, PS_GPU_ERR_ARG, "no auto or cross spectrum requested");

  // bins (src/multipole.c:334-394)
  {
    double bmax = (p.box[0] > p.box[1]) ? p.box[0] : p.box[1];
    if (bmax < p.box[2]) bmax = p.box[2];
    double kny = kPi * p.ng / bmax;
    if (p.logscale) kny = log10(kny);
    double kmax = kny;
    if (p.kmax > 0 && kmax > p.kmax) kmax = p.kmax;
    const double nb = round((kmax - p.kmin) / p.dk);
    if (!(nb < 2147483647.0)) return fail(c, PS_GPU_ERR_PK, "too many wave number bins");
    int nbin = (int)nb;
    if (p.kmin + p.dk * nbin > kny) nbin -= 1;
    if (nbin < 1) return fail(c, PS_GPU_ERR_PK, "not enough k bins given the Nyquist frequency and the bin size");
    c->nbin = nbin;
    c->kedge.resize(nbin + 1);
    c->kcen.resize(nbin);
    for (int i = 0; i <= nbin; i++) c->kedge[i] = p.kmin + p.dk * i;
    for (int i = 0; i < nbin; i++) c->kcen[i] = (c->kedge[i] + c->kedge[i + 1]) * 0.5;
  }

  int dcount = 0;
  if (cudaGetDeviceCount(&dcount) != cudaSuccess || dcount < 1)
    return fail(c, PS_GPU_ERR_CUDA, "no CUDA device available");
  if (p.device < 0 || p.device >= dcount) return fail(c, PS_GPU_ERR_ARG, "invalid device %d", p.device);
  DeviceScope dev_scope_(p.device);
  CU(dev_scope_.err);
  CU(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, p.device));
  CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (auto& e : c->ev) CU(cudaEventCreate(&e));
  CU(cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming));
  // place ps_gpu_bin_fields_noalloc's static scratch now, not on its first
  // call; a failure here is cleared and reported by that entry point
  if (noalloc_prepare(p.device) != cudaSuccess) (void)cudaGetLastError();

  // ---- geometry tables (FP64 on the host)
  const int ng = p.ng, h = c->ngk;
  double vec[3];
  for (int d = 0; d < 3; d++) vec[d] = 2 * kPi / p.box[d];
  std::vector<double> ksq(3 * h);
  for (int d = 0; d < 3; d++)
    for (int m = 0; m < h; m++) {
      const double kv = m * vec[d];
      ksq[d * h + m] = kv * kv;
    }
  std::vector<float> win(3 * ng);
  const double fac = kPi / ng;
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < ng; i++)
      win[d * ng + i] = (float)alias_corr(p.interlace, p.assign, signed_index(i, ng) * fac);
  std::vector<float2> phase(3 * ng);
  for (int m = 0; m < 3 * ng; m++) {
    const double a = kPi * (double)(m - ng) / ng;
    phase[m] = make_float2((float)cos(a), (float)sin(a));
  }
  const bool cubic = (p.box[0] == p.box[1] && p.box[1] == p.box[2]);
  const int nmax = 3 * (ng / 2) * (ng / 2);
  if (cubic && c->nbin < 32000) {
    std::vector<short> tab(nmax + 1);
    const double v2 = vec[0] * vec[0];
    for (int n = 0; n <= nmax; n++) {
      const double t = (double)n * v2;
      const int blo = ref_bin(c, t * (1 - 1e-12)), bhi = ref_bin(c, t * (1 + 1e-12));
      tab[n] = (short)((blo == bhi) ? blo : -2);
    }
    if ((rc = upload(c, &c->d_bintab, tab))) return rc;
  }
  if ((rc = upload(c, &c->d_ksq, ksq))) return rc;
  if ((rc = upload(c, &c->d_win, win))) return rc;
  if ((rc = upload(c, &c->d_phase, phase))) return rc;
  if ((rc = upload(c, &c->d_tw_full, twiddles(ng)))) return rc;
  if ((rc = upload(c, &c->d_tw_half, twiddles(ng / 2)))) return rc;
  if (wfft_supported(ng, 0)) {
    if ((rc = upload(c, &c->d_twl_half, warp_twiddles(ng / 2)))) return rc;
    c->wfft |= 1;
  }
  if (wfft_supported(ng, 1)) {
    if ((rc = upload(c, &c->d_twl_full, warp_twiddles(ng)))) return rc;
    c->wfft |= 2 | 4;
  } else if (ng == 2048) {  // the y pass, and with <= 2 fields the x pass, by pairs of warps
    if ((rc = upload(c, &c->d_twl_full, warp_twiddles(ng)))) return rc;
    c->wfft |= 2 | (c->nfield <= 2 ? 4 : 0);
  }

  ModeGeom& g = c->geom;
  g.ng = ng;
  g.nbin = c->nbin;
  g.nmu = 1;
  g.npole = p.npole;
  for (int l = 0; l < kMaxPole; l++) g.poles[l] = (l < p.npole) ? p.poles[l] : 0;
  g.logscale = p.logscale;
  g.nmax = nmax;
  g.bintab = c->d_bintab;
  // FP32 bin estimate from the FP32 components of k (vec * index, squares,
  // sums, a reciprocal square root): |error of t| <= ~8 ulp of
  // (|k| + |k0|) / dk; trusted beyond twice that from an edge, and only
  // where the table also applies
  {
    const double span = (fabs(c->kedge[0]) + fabs(c->kedge[c->nbin])) / p.dk + 2.0;
    const double eps = 16.0 * 1.1920928955078125e-7 * span;
    g.fastbin = (c->d_bintab && !p.logscale && eps < 0.05) ? 1 : 0;
    g.k0f = (float)c->kedge[0];
    g.inv_dkf = (float)(1.0 / p.dk);
    g.eps_t = (float)eps;
  }
  // Legendre polynomials (math/legpoly.h:47-62) as Horner coefficients in mu^2
  {
    static const float lc[7][4] = {{1.f, 0, 0, 0},           {1.f, 0, 0, 0},
                                   {-0.5f, 1.5f, 0, 0},      {-1.5f, 2.5f, 0, 0},
                                   {0.375f, -3.75f, 4.375f, 0}, {1.875f, -8.75f, 7.875f, 0},
                                   {-0.3125f, 6.5625f, -19.6875f, 14.4375f}};
    g.lodd = 0;
    for (int l = 0; l < kMaxPole; l++)
      for (int q = 0; q < 4; q++) g.lc[l][q] = 0.f;
    for (int l = 0; l < p.npole; l++) {
      for (int q = 0; q < 4; q++) g.lc[l][q] = lc[p.poles[l]][q];
      if (p.poles[l] & 1) g.lodd |= 1 << l;
    }
  }
  g.ksq = c->d_ksq;
  g.win = c->d_win;
  g.phase = c->d_phase;
  g.kedge0 = c->kedge[0];
  g.kedgeN = c->kedge[c->nbin];
  g.dk = p.dk;
  for (int d = 0; d < 3; d++) {
    g.vec[d] = (float)vec[d];
    g.los[d] = (float)p.los[d];
  }

  // ---- tiles and persistent grid of the binning pass
  c->ty_a = std::min({ng, 16, kCtaElems / (ng / 2)});
  c->tx_b = std::min({ng, 16, kCtaElems / ng});
  // y pass: long lines (Ng >= 512) take radix-32 passes on 8192-value tiles,
  // one CTA per SM (fewer shared-memory passes); shorter ones two CTAs per SM.
  // The z pass takes radix-16 passes; both can be retuned (ps_gpu_autotune).
  c->radix32_b = ng >= 512;
  plan_pipes(c);
  const int nacc = c->nspec * p.npole;
  {
    const int rc = plan_pass_c(c);
    if (rc) return rc;
  }

  // ---- device memory
  size_t freeb = 0, totalb = 0;
  CU(cudaMemGetInfo(&freeb, &totalb));
  const size_t need = (size_t)c->nfield * (c->ncx * 16) +
                      (size_t)std::max({c->grid_c, c->grid_ct, c->grid_cw}) * nacc * c->nbin * 8 + c->nkeys * 8 +
                      (64u << 20);
  if (need > freeb)
    return fail(c, PS_GPU_ERR_MEMORY, "need %.1f GB of device memory, %.1f GB free", need / 1e9, freeb / 1e9);
  // per field: the FP32 mesh, later reused for the y-pass output (8 B * Ncmplx
  // >= 4 B * Ng^3), and the z-pass output
  for (int f = 0; f < c->nfield; f++) {
    CU(dev_malloc(&c->grid[f], c->ncx * sizeof(float2)));
    CU(dev_malloc(&c->cbuf[f], c->ncx * sizeof(float2)));
  }
  CU(dev_malloc(&c->d_hist, (c->nkeys + 1) * sizeof(unsigned)));
  CU(dev_malloc(&c->d_bsum, ((c->nkeys + 4095) / 4096 + 1) * sizeof(unsigned)));
  if ((rc = alloc_accum(c))) return rc;
  // [2 cats][2] sums, then [2 cats] mean cell values in fixed point (int64)
  CU(dev_malloc(&c->d_wsum, sizeof(double) * 6));
  CU(dev_malloc(&c->d_wpart, sizeof(double) * 2 * kAssignMaxBlocks));
  CU(dev_malloc(&c->d_err, sizeof(int) * 4));
  CU(cudaMemset(c->d_wsum, 0, sizeof(double) * 6));
  CU(cudaMemset(c->d_err, 0, sizeof(int) * 4));

  // ---- geometry sweep: counts, mean |k|, multipole mode weights
  {
    unsigned long long* d_cnt = nullptr;
    double *d_ks = nullptr, *d_lc = nullptr;
    CU(dev_malloc(&d_cnt, sizeof(unsigned long long) * c->nbin));
    CU(dev_malloc(&d_ks, sizeof(double) * c->nbin));
    CU(dev_malloc(&d_lc, sizeof(double) * (size_t)p.npole * c->nbin));
    CU(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * c->nbin, c->stream));
    CU(cudaMemsetAsync(d_ks, 0, sizeof(double) * c->nbin, c->stream));
    CU(cudaMemsetAsync(d_lc, 0, sizeof(double) * (size_t)p.npole * c->nbin, c->stream));
    GeomArgs ga;
    ga.ng = ng;
    ga.geom = g;
    for (int d = 0; d < 3; d++) { ga.vec[d] = vec[d]; ga.los[d] = p.los[d]; }
    ga.cnt = d_cnt;
    ga.ksum = d_ks;
    ga.lcnt = d_lc;
    launch_geometry(ga, c->stream);
    CU(cudaGetLastError());
    c->cnt.resize(c->nbin);
    c->km.resize(c->nbin);
    c->lcnt.resize((size_t)p.npole * c->nbin);
    std::vector<unsigned long long> cnt(c->nbin);
    CU(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(unsigned long long) * c->nbin, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->km.data(), d_ks, sizeof(double) * c->nbin, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->lcnt.data(), d_lc, sizeof(double) * (size_t)p.npole * c->nbin, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    cudaFree(d_cnt);
    cudaFree(d_ks);
    cudaFree(d_lc);
    for (int b = 0; b < c->nbin; b++) {
      c->cnt[b] = cnt[b];
      if (cnt[b]) c->km[b] /= (double)cnt[b];
    }
  }
  return 0;
}

void ps_gpu_destroy(ps_gpu_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (int f = 0; f < 4; f++) {
    if (c->grid[f]) cudaFree(c->grid[f]);
    if (c->cbuf[f]) cudaFree(c->cbuf[f]);
  }
  void* bufs[] = {c->d_bintab, c->d_ksq, c->d_win, c->d_phase, c->d_tw_full, c->d_tw_half,
                  c->d_twl_full, c->d_twl_half, c->d_part, c->d_sums, c->d_wsum, c->d_wpart, c->d_err, c->d_stage,
                  c->d_hist, c->d_bsum, c->d_rank, c->d_rec, c->d_region, c->d_lgeo,
                  c->d_lx, c->d_lxb, c->d_lc, c->d_lout, c->d_slot[0], c->d_slot[1],
                  c->d_yama, c->d_dc, c->d_dcpart};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->h_lout) cudaFreeHost(c->h_lout);
  for (int k = 0; k < 2; k++) {
    if (c->copied[k]) cudaEventDestroy(c->copied[k]);
    if (c->used[k]) cudaEventDestroy(c->used[k]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->ev_done) cudaEventDestroy(c->ev_done);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int ps_gpu_nbin(const ps_gpu_ctx* c) { return c ? c->nbin : PS_GPU_ERR_ARG; }

const char* ps_gpu_last_error(const ps_gpu_ctx* c) { return c ? c->err : "null context"; }

int ps_gpu_last_timings(const ps_gpu_ctx* c, float* ms, int nmax) {
  if (!c || !ms) return 0;
  int n = std::min(nmax, 6);
  for (int i = 0; i < n; i++) ms[i] = c->timings[i];
  return n;
}

int ps_gpu_last_launches(const ps_gpu_ctx* c) { return c ? c->launches : 0; }

void* ps_gpu_stream(const ps_gpu_ctx* c) { return c ? (void*)c->stream : nullptr; }

}  // extern "C"

namespace {

int ensure_stage(ps_gpu_ctx* c, size_t bytes) {
  if (bytes <= c->stage_bytes) return 0;
  if (c->d_stage) {
    CU(cudaStreamSynchronize(c->stream));
    cudaFree(c->d_stage);
    c->d_stage = nullptr;
    c->stage_bytes = 0;
  }
  CU(dev_malloc(&c->d_stage, bytes));
  c->stage_bytes = bytes;
  return 0;
}

// Region buffer of the region gather: every tile's regions.
size_t region_words(const ps_gpu_ctx* c) {
  return (size_t)c->gnt * c->gnt * c->gnt * (size_t)c->mpc * gather_region_words(c->p.assign);
}
size_t region_need(const ps_gpu_ctx* c) {  // region words, then a flag byte per tile
  return region_words(c) * sizeof(unsigned long long) + (size_t)c->gnt * c->gnt * c->gnt;
}

// The region gather for a catalogue of n particles: forced on or off by the
// tuning knob, else when there is a particle for every 32 cells or more (its
// cost is the region traffic, 2.3x the mesh in int64, whatever the count;
// the tile gather's grows with the particles and their halo replays).
bool use_region(const ps_gpu_ctx* c, size_t n) {
  if (!gather_region_ok(c->ng, c->gT, c->p.assign)) return false;
  if (c->gather_region >= 0) return c->gather_region == 1;
  return (double)n * 32.0 >= (double)c->ntot && region_need(c) <= ((size_t)64 << 30);
}

int ensure_region(ps_gpu_ctx* c) {
  const size_t need = region_need(c);
  if (need <= c->region_bytes) return 0;
  CU(cudaStreamSynchronize(c->stream));
  if (c->d_region) cudaFree(c->d_region);
  c->d_region = nullptr;
  c->region_bytes = 0;
  CU(dev_malloc(&c->d_region, need));
  c->region_bytes = need;
  return 0;
}

GatherArgs gather_args(ps_gpu_ctx* c, int cat, size_t n) {
  GatherArgs g{};
  g.ng = c->ng;
  g.assign = c->p.assign;
  g.interlace = c->p.interlace;
  g.T = c->gT;
  g.nt = c->gnt;
  g.tshift = -1;
  for (int k = 0; k < 31; k++)
    if ((1 << k) == g.T) g.tshift = k;
  for (int d = 0; d < 3; d++) {
    g.box[d] = c->p.box[d];
    // the reference's shifted-grid edges (src/genr_mesh.c), correctly rounded
    const double half = 0.5 * c->p.box[d];
    g.bmin[d] = 0.0 - half / (double)c->ng;
    g.bmax[d] = g.bmin[d] + c->p.box[d];
    const double s = (double)c->ng / c->p.box[d];
    g.s_hi[d] = (float)s;
    g.s_lo[d] = (float)(s - (double)g.s_hi[d]);
    double L = c->p.box[d];
    memcpy(&g.box_bits[d], &L, sizeof L);
    float bf = (float)L;
    if ((double)bf < L) bf = nextafterf(bf, INFINITY);
    g.box_f[d] = bf;
  }
  g.hist = c->d_hist;
  g.bsum = c->d_bsum;
  g.rank = c->d_rank;
  g.rec = c->d_rec;
  for (int m = 0; m < c->mpc; m++) g.out[m] = (float*)c->grid[cat * c->mpc + m];
  g.wsum = c->d_wsum + 2 * cat;
  g.moff_scale = 4294967296.0 / ((double)c->ng * c->ng * c->ng);
  g.moff = reinterpret_cast<long long*>(c->d_wsum + 4) + cat;
  g.wpart = c->d_wpart;
  g.err = c->d_err + cat;
  g.threads = c->gather_threads;
  g.sparse_max = c->gather_sparse_max;
  g.region = use_region(c, n) ? 1 : 0;
  g.regbuf = c->d_region;
  g.nomean = c->survey[cat] ? 1 : 0;
  g.regflag = c->d_region ? reinterpret_cast<unsigned char*>(c->d_region + region_words(c)) : nullptr;
  return g;
}

// Rank and record buffers for n particles (reallocated only to grow).
int ensure_gather_capacity(ps_gpu_ctx* c, size_t n) {
  if (n <= c->gcap) return 0;
  CU(cudaStreamSynchronize(c->stream));
  if (c->d_rank) cudaFree(c->d_rank);
  if (c->d_rec) cudaFree(c->d_rec);
  c->d_rank = nullptr;
  c->d_rec = nullptr;
  c->gcap = 0;
  CU(dev_malloc(&c->d_rank, n * sizeof(unsigned)));
  CU(dev_malloc(&c->d_rec, n * gather_record_bytes()));
  c->gcap = n;
  return 0;
}

int assign_common(ps_gpu_ctx* c, int cat, Particles pt) {
  // ranks and bucket offsets are 32-bit
  if (pt.n >= 0xffffffffull)
    return fail(c, PS_GPU_ERR_RANGE, "%zu particles: at most 2^32 - 2 per catalogue", pt.n);
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  if (!c->assign_started) {
    CU(cudaEventRecord(c->ev[6], c->stream));
    c->assign_started = true;
    c->launches = 0;
    c->assign_gen++;
  }
  {
    int rc = ensure_gather_capacity(c, pt.n);
    if (!rc && use_region(c, pt.n)) rc = ensure_region(c);
    if (rc) return rc;
  }
  CU(cudaMemsetAsync(c->d_wsum + 2 * cat, 0, sizeof(double) * 2, c->stream));
  CU(cudaMemsetAsync(c->d_err + cat, 0, sizeof(int), c->stream));
  if (pt.n) c->launches += launch_gather_assign(pt, gather_args(c, cat, pt.n), c->stream, false);
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[7], c->stream));
  c->assigned[cat] = 1;
  c->npart[cat] = pt.n;
  c->last_cat = cat;
  c->last_pt = pt;
  return 0;
}

}  // namespace

namespace {

// Every launch of one evaluation after the assignment (passes A, B, C and
// the reduction into sums_dst, device [nspec*npole][nbin*nmu]), on the
// context stream, without synchronising: usable inside a stream capture.
int enqueue_passes(ps_gpu_ctx* c, double* sums_dst, bool events) {
  const ps_gpu_params& p = c->p;
  cudaStream_t s = c->stream;
  const int ng = c->ng, npole = p.npole, nbin = c->nbin, nmu = c->nmu;
  const int nacc = c->nspec * npole;
  const int nkey = nbin * nmu;
  const bool pipe = c->plan_full.logn >= 0 && !getenv("PS_GPU_NO_PIPELINE");
  CU(cudaMemsetAsync(c->d_err + 2, 0, sizeof(int), s));
  if (events) CU(cudaEventRecord(c->ev[0], s));
  for (int f = 0; f < c->nfield; f++) {
    PassAArgs a;
    memset(&a, 0, sizeof a);
    a.ng = ng;
    a.ty = pipe ? c->ty_ap : c->ty_a;
    a.pipe_grid = pipe ? (c->radix32_a ? 1 : 2) * c->nsm : 0;
    a.radix32 = c->radix32_a ? 1 : 0;
    a.err = c->d_err + 2;
    a.fgrid = (const float*)c->grid[f];
    a.out = c->cbuf[f];
    a.tw_half = c->d_tw_half;
    a.tw_full = c->d_tw_full;
    a.plan_half = c->plan_half;
    a.twl = (c->wfft & 1) ? c->d_twl_half : nullptr;
    a.stall = c->stall ? 1 : 0;
    a.wait_limit = c->stall;
    c->launches += launch_pass_a(a, s);
  }
  CU(cudaGetLastError());
  if (events) CU(cudaEventRecord(c->ev[1], s));
  for (int f = 0; f < c->nfield; f++) {
    PassBArgs b;
    memset(&b, 0, sizeof b);
    b.ng = ng;
    b.tx = pipe ? c->tx_bp : c->tx_b;
    b.pipe_grid = pipe ? (c->radix32_b ? 1 : 2) * c->nsm : 0;
    b.radix32 = c->radix32_b ? 1 : 0;
    b.err = c->d_err + 2;
    b.in = c->cbuf[f];
    b.out = (float2*)c->grid[f];
    b.tw_full = c->d_tw_full;
    b.plan_full = c->plan_full;
    b.twl = (c->wfft & 2) ? c->d_twl_full : nullptr;
    b.stall = c->stall ? 1 : 0;
    b.wait_limit = c->stall;
    c->launches += launch_pass_b(b, s);
  }
  CU(cudaGetLastError());
  if (events) CU(cudaEventRecord(c->ev[2], s));
  const bool warp_c = (c->wfft & 4) && c->grid_cw > 0;
  const bool pipe_c = !warp_c && pipe && c->pipe_c_on && c->grid_ct > 0;
  const int grid_c = warp_c ? c->grid_cw : pipe_c ? c->grid_ct : c->grid_c;
  CU(cudaMemsetAsync(c->d_part, 0, sizeof(double) * (size_t)grid_c * nacc * nkey, s));
  PassCArgs pc;
  memset(&pc, 0, sizeof pc);
  pc.ng = ng;
  pc.ty = pipe_c ? c->ty_ct : c->ty_c;
  pc.pipe = pipe_c ? 1 : 0;
  pc.mom = pass_c_moments(p.poles, p.npole);
  pc.twl = warp_c ? c->d_twl_full : nullptr;
  pc.wpc = c->wpc_cw;
  pc.stall = c->stall ? 1 : 0;
  pc.wait_limit = c->stall;
  c->stall = 0;  // one evaluation only
  pc.err = c->d_err + 2;
  pc.nfield = c->nfield;
  pc.interlace = p.interlace;
  pc.ncat = p.ncat;
  pc.nspec = c->nspec;
  for (int k = 0; k < 3; k++) { pc.spec_a[k] = c->spec_a[k]; pc.spec_b[k] = c->spec_b[k]; }
  for (int f = 0; f < c->nfield; f++) pc.in[f] = (const float2*)c->grid[f];
  pc.store = nullptr;
  pc.tw_full = c->d_tw_full;
  pc.plan_full = c->plan_full;
  pc.geom = c->geom;
  pc.partials = reinterpret_cast<float2*>(c->d_part);
  pc.grid = grid_c;
  c->launches += launch_pass_c(pc, s);
  CU(cudaGetLastError());
  if (events) CU(cudaEventRecord(c->ev[3], s));
  c->launches += launch_reduce(reinterpret_cast<const float2*>(c->d_part), grid_c, nacc * nkey, sums_dst, s);
  CU(cudaGetLastError());
  if (events) CU(cudaEventRecord(c->ev[4], s));
  return 0;
}

// Host epilogue of one evaluation from its raw results: h = sums
// [nacc][nbin*nmu] followed by wsum[4] and the error flags (4 ints).
int finish(ps_gpu_ctx* c, const double* h, const size_t* npart, ps_gpu_result* r, bool keep_kmu) {
  const ps_gpu_params& p = c->p;
  const int npole = p.npole, nbin = c->nbin, nmu = c->nmu;
  const int nacc = c->nspec * npole;
  const int nkey = nbin * nmu;
  // fold the |mu| sub-bins (kept for ps_gpu_read_kmu)
  std::vector<double> fold;
  const double* sums = h;
  if (nmu > 1) {
    if (keep_kmu) c->kmu.assign(h, h + (size_t)nacc * nkey);
    fold.assign((size_t)nacc * nbin, 0.0);
    for (size_t q = 0; q < (size_t)nacc * nbin; q++)
      for (int j = 0; j < nmu; j++) fold[q] += h[q * nmu + j];
    sums = fold.data();
  }
  const double* wsum = h + (size_t)nacc * nkey;
  const int* errs = (const int*)(h + (size_t)nacc * nkey + 4);
  if (errs[2]) return fail(c, PS_GPU_ERR_CUDA, "pipelined pass: bulk-copy wait timed out (flags %d)", errs[2]);
  for (int k = 0; k < p.ncat; k++) {
    // an empty catalogue has no coordinate range (src/genr_mesh.c:518-521)
    if (!npart[k]) return fail(c, PS_GPU_ERR_CATA, "catalogue %d: no objects", k);
    if (errs[k] & 2) return fail(c, PS_GPU_ERR_CUDA, "catalogue %d: region index out of range", k);
    if (errs[k]) return fail(c, PS_GPU_ERR_CATA, "catalogue %d: coordinate outside [0, BOX_SIZE)", k);
    if (!(wsum[2 * k + 1] < kFixMaxWeight))
      return fail(c, PS_GPU_ERR_RANGE, "catalogue %d: total |weight| %g exceeds the fixed-point range", k, wsum[2 * k + 1]);
  }

  // epilogue (src/genr_mesh.c:904-910, src/multipole.c:1047-1087); surveys:
  // the shot noise and normalisation given (src/read_cata.c:173-183), the
  // shot noise reported as shot / norm (src/save_res.c:89)
  const double vol = p.box[0] * p.box[1] * p.box[2];
  for (int k = 0; k < 2; k++) {
    r->wdata[k] = (k < p.ncat) ? wsum[2 * k] : 0;
    r->shot[k] = (k < p.ncat) ? vol / r->wdata[k] : 0;
    r->norm[k] = (k < p.ncat) ? r->wdata[k] * r->wdata[k] / vol : 0;
    if (k < p.ncat && c->survey[k]) {
      r->shot[k] = c->survey_shot[k] / c->survey_norm[k];
      r->norm[k] = c->survey_norm[k];
    }
  }
  // Surveys sum the k = 0 mode when it lies in a bin (src/multipole.c:593-606;
  // simulation boxes skip it, :806).  Its value is F_a(0) F_b(0) = W_a W_b,
  // the fields' weight sums (the mesh holds mean-free values).
  const bool dc_bin = !p.logscale && c->kedge[0] <= 0.0 && nbin > 0;
  r->nbin = nbin;
  for (int s2 = 0; s2 < c->nspec; s2++) {
    const int cat = c->spec_cat[s2];
    double* dst = (cat >= 0) ? (r->pl ? r->pl + (size_t)cat * npole * nbin : nullptr) : r->xpl;
    if (!dst) continue;
    for (int l = 0; l < npole; l++) {
      for (int i = 0; i < nbin; i++) {
        double v = sums[((size_t)s2 * npole + l) * nbin + i];
        const double cn = (double)c->cnt[i];
        const bool sv = cat >= 0 ? c->survey[cat] : (c->survey[0] && c->survey[1]);
        if (sv && p.poles[l] > 0 && c->yama_last) {
          // src/multipole.c:1118-1150: (F_0, F_l) pairs, the k = 0 mode
          // F_0(0) = W times Re F_l(0) when bin 0 holds it
          const int a = c->spec_a[s2], b = c->spec_b[s2];
          const double* dc = h + (size_t)nacc * nkey + 8 + 2 * l;  // Re F_l(0) per catalogue
          if (dc_bin && i == 0)
            v += (cat >= 0) ? wsum[2 * a] * dc[a] : wsum[2 * a] * dc[b] + wsum[2 * b] * dc[a];
          if (c->cnt[i])
            v *= (cat >= 0 ? 4 * M_PI / r->norm[cat] : 2 * M_PI / sqrt(r->norm[0] * r->norm[1])) / cn;
          dst[(size_t)l * nbin + i] = v;
          continue;
        }
        if (sv && dc_bin && i == 0 && p.poles[l] == 0)
          v += wsum[2 * c->spec_a[s2]] * wsum[2 * c->spec_b[s2]];
        if (cat >= 0) {
          if (c->cnt[i]) {
            v /= r->norm[cat] * cn;
            // surveys subtract the shot noise whole (src/multipole.c:1113)
            v -= sv ? r->shot[cat] : r->shot[cat] * c->lcnt[(size_t)l * nbin + i] / cn;
          }
        } else if (c->cnt[i]) {
          v /= sqrt(r->norm[0] * r->norm[1]) * cn;
        }
        v *= 2 * p.poles[l] + 1;
        dst[(size_t)l * nbin + i] = v;
      }
    }
  }
  for (int i = 0; i < nbin; i++) {
    if (r->k) r->k[i] = c->kcen[i];
    if (r->km) r->km[i] = c->km[i];
    if (r->kedge) r->kedge[i] = c->kedge[i];
    if (r->cnt) r->cnt[i] = c->cnt[i];
  }
  if (r->kedge) r->kedge[nbin] = c->kedge[nbin];
  if (r->lcnt) memcpy(r->lcnt, c->lcnt.data(), sizeof(double) * (size_t)npole * nbin);
  // log bins: src/multipole.c:1267-1274, including its reuse of the rescaled k
  if (p.logscale) {
    for (int i = 0; i < nbin; i++) {
      const double kc = pow(10, c->kcen[i]);
      if (r->k) r->k[i] = kc;
      if (r->km) r->km[i] = pow(10, kc);
      if (r->kedge) r->kedge[i] = pow(10, kc);
    }
    if (r->kedge) r->kedge[nbin] = pow(10, c->kedge[nbin]);
  }
  return 0;
}

}  // namespace

namespace ps {

int ctx_view(const ps_gpu_ctx* c, CtxView* v) {
  if (!c || !v) return 1;
  v->ng = c->ng;
  v->device = c->p.device;
  v->geom = c->geom;
  return 0;
}

int ctx_fail(ps_gpu_ctx* c, int code, const char* fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof c->err, fmt, ap);
    va_end(ap);
  }
  return code;
}

}  // namespace ps

extern "C" {

int ps_gpu_assign_aos(ps_gpu_ctx* c, int cat, const double* xyzw, size_t n, int on_device) {
  if (!c || cat < 0 || cat >= c->p.ncat || (!xyzw && n)) return fail(c, PS_GPU_ERR_ARG, "invalid assign arguments");
  Particles pt{};
  pt.n = n;
  if (on_device) {
    if ((uintptr_t)xyzw & 31)
      return fail(c, PS_GPU_ERR_ARG, "device AoS records must be 32-byte aligned");
    pt.aos = xyzw;
  } else {
    int rc = ensure_stage(c, n * 4 * sizeof(double));
    if (rc) return rc;
    CU(cudaMemcpyAsync(c->d_stage, xyzw, n * 4 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    pt.aos = (const double*)c->d_stage;
  }
  return assign_common(c, cat, pt);
}

int ps_gpu_stage_aos(ps_gpu_ctx* c, int slot, const double* xyzw, size_t n) {
  if (!c || slot < 0 || slot > 1 || (!xyzw && n)) return fail(c, PS_GPU_ERR_ARG, "invalid stage arguments");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  if (!c->copy_stream) {
    CU(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) {
      CU(cudaEventCreateWithFlags(&c->copied[k], cudaEventDisableTiming));
      CU(cudaEventCreateWithFlags(&c->used[k], cudaEventDisableTiming));
      CU(cudaEventRecord(c->used[k], c->stream));
    }
  }
  const size_t bytes = n * 4 * sizeof(double);
  if (bytes > c->slot_bytes[slot]) {
    // the slot may still be read by earlier assignment kernels
    CU(cudaEventSynchronize(c->used[slot]));
    CU(cudaStreamSynchronize(c->copy_stream));
    if (c->d_slot[slot]) cudaFree(c->d_slot[slot]);
    c->d_slot[slot] = nullptr;
    c->slot_bytes[slot] = 0;
    CU(dev_malloc(&c->d_slot[slot], bytes));
    c->slot_bytes[slot] = bytes;
  }
  // the copy waits for the kernels that read this slot's previous catalogue
  CU(cudaStreamWaitEvent(c->copy_stream, c->used[slot], 0));
  if (n) CU(cudaMemcpyAsync(c->d_slot[slot], xyzw, bytes, cudaMemcpyHostToDevice, c->copy_stream));
  CU(cudaEventRecord(c->copied[slot], c->copy_stream));
  c->slot_n[slot] = n;
  c->slot_full[slot] = true;
  return 0;
}

int ps_gpu_assign_staged(ps_gpu_ctx* c, int cat, int slot) {
  if (!c || cat < 0 || cat >= c->p.ncat || slot < 0 || slot > 1)
    return fail(c, PS_GPU_ERR_ARG, "invalid assign arguments");
  if (!c->slot_full[slot]) return fail(c, PS_GPU_ERR_STATE, "staging slot %d holds no catalogue", slot);
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  CU(cudaStreamWaitEvent(c->stream, c->copied[slot], 0));
  Particles pt{};
  pt.n = c->slot_n[slot];
  pt.aos = (const double*)c->d_slot[slot];
  const int rc = assign_common(c, cat, pt);
  // the slot is free again once the classify and scatter kernels are done
  CU(cudaEventRecord(c->used[slot], c->stream));
  c->slot_full[slot] = false;
  return rc;
}

int ps_gpu_assign_soa(ps_gpu_ctx* c, int cat, const float* x, const float* y, const float* z,
                      const float* w, size_t n, int on_device) {
  if (!c || cat < 0 || cat >= c->p.ncat || ((!x || !y || !z) && n))
    return fail(c, PS_GPU_ERR_ARG, "invalid assign arguments");
  Particles pt{};
  pt.n = n;
  if (on_device) {
    if (((uintptr_t)x | (uintptr_t)y | (uintptr_t)z | (uintptr_t)w) & 3)
      return fail(c, PS_GPU_ERR_ARG, "device SoA arrays must be 4-byte aligned");
    pt.x = x; pt.y = y; pt.z = z; pt.w = w;
  } else {
    const int na = w ? 4 : 3;
    int rc = ensure_stage(c, n * na * sizeof(float));
    if (rc) return rc;
    float* s = (float*)c->d_stage;
    const float* src[4] = {x, y, z, w};
    for (int k = 0; k < na; k++)
      CU(cudaMemcpyAsync(s + k * n, src[k], n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    pt.x = s; pt.y = s + n; pt.z = s + 2 * n; pt.w = w ? s + 3 * n : nullptr;
  }
  return assign_common(c, cat, pt);
}

}  // extern "C"

namespace {

// r2c of a real device mesh into a stored half-complex field [x][y][z/2+1]
// (the z, y and x passes; a1, a2: scratch fields; the pipelined z and y
// passes for power-of-two meshes).  With a harmonic yk: the mesh weighted by
// yk(r^) on the way in (observer at the origin), and out = (acc_mode 1) or
// += (acc_mode 2) the transform times yk(k^).
void r2c_store(ps_gpu_ctx* c, const float* in, float2* a1, float2* a2, float2* out,
               int acc_mode = 0, const YlmCoef* yk = nullptr) {
  cudaStream_t s = c->stream;
  const bool pipe = c->plan_full.logn >= 0 && !getenv("PS_GPU_NO_PIPELINE");
  PassAArgs a;
  memset(&a, 0, sizeof a);
  a.ng = c->ng;
  a.ty = pipe ? c->ty_ap : c->ty_a;
  a.pipe_grid = pipe ? (c->radix32_a ? 1 : 2) * c->nsm : 0;
  a.radix32 = c->radix32_a ? 1 : 0;
  a.fgrid = in;
  if (yk) {
    a.yw = 1;
    a.yc = *yk;
    for (int d = 0; d < 3; d++) {
      a.org[d] = (float)(c->survey_origin[d] * c->ng / c->p.box[d]);
      a.len[d] = (float)c->p.box[d];
    }
  }
  a.out = a1;
  a.tw_half = c->d_tw_half;
  a.tw_full = c->d_tw_full;
  a.plan_half = c->plan_half;
  a.twl = (c->wfft & 1) ? c->d_twl_half : nullptr;
  a.err = c->d_err + 2;
  launch_pass_a(a, s);
  PassBArgs b;
  memset(&b, 0, sizeof b);
  b.ng = c->ng;
  b.tx = pipe ? c->tx_bp : c->tx_b;
  b.pipe_grid = pipe ? (c->radix32_b ? 1 : 2) * c->nsm : 0;
  b.radix32 = c->radix32_b ? 1 : 0;
  b.in = a1;
  b.out = a2;
  b.tw_full = c->d_tw_full;
  b.plan_full = c->plan_full;
  b.twl = (c->wfft & 2) ? c->d_twl_full : nullptr;
  b.err = c->d_err + 2;
  launch_pass_b(b, s);
  PassCArgs pc;
  memset(&pc, 0, sizeof pc);
  pc.ng = c->ng;
  // 8 kz per tile: 64-byte runs, and small tiles keep more CTAs resident to
  // hide the accumulator's read-modify-write (Ng = 256: 4.1 ms for the 14
  // harmonic terms of l = 2, 4 against 4.2 ms at 16 and 4.6 ms at 4)
  pc.ty = std::max(1, std::min({c->ng / 2 + 1, 8, kPassCElems / c->ng}));
  pc.nfield = 1;
  pc.ncat = 1;
  pc.nspec = 1;
  pc.in[0] = a2;
  pc.store = out;
  pc.acc_mode = acc_mode;
  if (yk) pc.yk = *yk;
  for (int d = 0; d < 3; d++) pc.kinv[d] = (float)(1.0 / c->p.box[d]);
  pc.tw_full = c->d_tw_full;
  pc.plan_full = c->plan_full;
  pc.geom = c->geom;
  pc.twl = (c->wfft & 4) ? c->d_twl_full : nullptr;
  launch_pass_c(pc, s);
  c->launches += 3;
}

// Per-CTA partial sums of Re[f1 f2*] x window x weight per k bin (the k = 0
// mode left out), added onto the partials (zeroed by the caller).
void bin_pair(ps_gpu_ctx* c, const float2* f1, const float2* f2) {
  BinFieldArgs b;
  b.ng = c->ng;
  b.f1 = f1;
  b.f2 = f2;
  b.geom = c->geom;
  b.geom.nmu = 1;
  b.geom.npole = 1;  // l = 0 weights: the multipole is in the fields
  for (int q = 0; q < 4; q++) b.geom.lc[0][q] = q == 0 ? 1.f : 0.f;
  b.geom.lodd = 0;
  b.partials = reinterpret_cast<float2*>(c->d_part);
  b.grid = c->grid_c;
  launch_bin_fields(b, c->stream);
  c->launches++;
}

// Survey catalogues with multipoles l > 0 (src/multipole.c:1179-1250):
// F_0 of each catalogue's mesh, then per l the field F_l of the harmonic
// decomposition, and the (F_0, F_l) pair sums; raw sums into c->d_sums as
// [spec][pole][bin], F_l(0) into c->d_dc as [pole][catalogue].  With
// interlacing, F_0 is the combination of the two meshes' fields and the
// harmonics weight its c2r / Ng^3, which replaces the plain mesh
// (src/multipole.c:462-500).
int enqueue_survey_multipoles(ps_gpu_ctx* c) {
  const ps_gpu_params& p = c->p;
  cudaStream_t s = c->stream;
  const size_t cx = c->ncx * sizeof(float2);
  const size_t need = (size_t)(3 + 2 * p.ncat) * cx;
  if (need > c->yama_bytes) {
    CU(cudaStreamSynchronize(s));
    if (c->d_yama) cudaFree(c->d_yama);
    c->d_yama = nullptr;
    c->yama_bytes = 0;
    CU(dev_malloc(&c->d_yama, need));
    c->yama_bytes = need;
  }
  if (!c->d_dc) CU(dev_malloc(&c->d_dc, 2 * kMaxPole * sizeof(double)));
  const int grid_dc = std::min(c->ng * c->ng, 4 * c->nsm);
  if (!c->d_dcpart) CU(dev_malloc(&c->d_dcpart, ((size_t)4 * c->nsm + 1) * sizeof(double)));
  double dc_org[3], dc_len[3];
  for (int d = 0; d < 3; d++) {
    dc_org[d] = c->survey_origin[d] * c->ng / c->p.box[d];
    dc_len[d] = c->p.box[d];
  }
  float2* base = (float2*)c->d_yama;
  float2 *a1 = base, *a2 = base + c->ncx, *fa = base + 2 * c->ncx;
  // fields: a1, a2, fa, then F_0 and F_l of catalogue 0 (and 1)
  float2* f0[2] = {base + 3 * c->ncx, base + 5 * c->ncx};
  float2* fl[2] = {base + 4 * c->ncx, base + 6 * c->ncx};
  CU(cudaMemsetAsync(c->d_err + 2, 0, sizeof(int), s));
  CU(cudaEventRecord(c->ev[0], s));
  const int mpc = c->mpc;
  for (int k = 0; k < p.ncat; k++) {
    r2c_store(c, (const float*)c->grid[k * mpc], a1, a2, f0[k]);
    if (p.interlace) {
      r2c_store(c, (const float*)c->grid[k * mpc + 1], a1, a2, fa);
      launch_inv_lead(f0[k], fa, a1, c->ng, c->geom.phase, c->d_tw_full, c->plan_full, s);
      launch_inv_lead(a1, nullptr, a2, c->ng, c->geom.phase, c->d_tw_full, c->plan_full, s);
      launch_c2r_z(a2, (float*)c->grid[k * mpc], c->ng, c->ty_a, c->d_tw_half, c->d_tw_full,
                   c->plan_half, s);
      c->launches += 3;
    }
  }
  CU(cudaEventRecord(c->ev[1], s));
  CU(cudaEventRecord(c->ev[2], s));
  const int nbin = c->nbin, npole = p.npole;
  for (int l = 0; l < npole; l++) {
    const int ell = p.poles[l];
    if (ell > 0)
      for (int k = 0; k < p.ncat; k++) {
        for (int m = -ell; m <= ell; m++) {
          const YlmCoef yk = ylm_coef(ell, m);
          r2c_store(c, (const float*)c->grid[k * mpc], a1, a2, fl[k], m == -ell ? 1 : 2, &yk);
        }
        // F_l(0) in FP64 from the same mesh the harmonic terms weight
        const int nl = launch_dc_sum((const float*)c->grid[k * mpc], c->ng, ell, dc_org, dc_len,
                                     c->d_wsum, p.ncat, fl[k], c->d_dcpart, grid_dc,
                                     c->d_dc + 2 * l + k, s);
        if (nl < 0) return fail(c, PS_GPU_ERR_ARG, "survey multipoles: unsupported multipole %d", ell);
        c->launches += nl;
      }
    for (int sp = 0; sp < c->nspec; sp++) {
      const int a = c->spec_a[sp], b = c->spec_b[sp];
      CU(cudaMemsetAsync(c->d_part, 0, sizeof(double) * (size_t)c->grid_c * nbin, s));
      if (ell == 0) {
        bin_pair(c, f0[a], f0[b]);
      } else {
        bin_pair(c, f0[a], fl[b]);
        if (a != b) bin_pair(c, f0[b], fl[a]);
      }
      launch_reduce(reinterpret_cast<const float2*>(c->d_part), c->grid_c, nbin, c->d_sums + ((size_t)sp * npole + l) * nbin, s);
      c->launches++;
    }
  }
  CU(cudaEventRecord(c->ev[3], s));
  CU(cudaEventRecord(c->ev[4], s));
  CU(cudaGetLastError());
  return 0;
}

bool survey_multipoles(const ps_gpu_ctx* c) {
  bool high = false;
  for (int l = 0; l < c->p.npole; l++) high |= c->p.poles[l] > 0;
  for (int k = 0; k < c->p.ncat; k++) high &= c->survey[k];
  return high;
}

}  // namespace

extern "C" {

int ps_gpu_execute(ps_gpu_ctx* c, ps_gpu_result* r) {
  if (!c || !r) return fail(c, PS_GPU_ERR_ARG, "null argument");
  if (c->learned_pending) return fail(c, PS_GPU_ERR_STATE, "a learned evaluation is pending: finish it first");
  const ps_gpu_params& p = c->p;
  for (int k = 0; k < p.ncat; k++)
    if (!c->assigned[k]) return fail(c, PS_GPU_ERR_STATE, "catalogue %d not assigned", k);
  if (p.ncat == 2 && c->survey[0] != c->survey[1])
    return fail(c, PS_GPU_ERR_STATE, "both catalogues must be survey catalogues, or neither");
  DeviceScope dev_scope_(p.device);
  CU(dev_scope_.err);
  cudaStream_t s = c->stream;
  const int nacc = c->nspec * p.npole;
  const int nkey = c->nbin * c->nmu;
  const bool yama = survey_multipoles(c);
  c->yama_last = yama;
  int rc = yama ? enqueue_survey_multipoles(c) : enqueue_passes(c, c->d_sums, true);
  if (rc) return rc;
  double* h = c->h_out;
  CU(cudaMemcpyAsync(h, c->d_sums, sizeof(double) * (size_t)nacc * nkey, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h + (size_t)nacc * nkey, c->d_wsum, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h + (size_t)nacc * nkey + 4, c->d_err, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
  double dc[2 * kMaxPole] = {};
  if (yama) CU(cudaMemcpyAsync(dc, c->d_dc, sizeof(double) * 2 * p.npole, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  for (int q = 0; q < 2 * p.npole; q++) h[(size_t)nacc * nkey + 8 + q] = dc[q];
  float t = 0;
  if (c->assign_started && cudaEventElapsedTime(&t, c->ev[6], c->ev[7]) == cudaSuccess) c->timings[0] = t;
  for (int i = 0; i < 4; i++)
    if (cudaEventElapsedTime(&t, c->ev[i], c->ev[i + 1]) == cudaSuccess) c->timings[1 + i] = t;
  if (cudaEventElapsedTime(&t, c->ev[0], c->ev[4]) == cudaSuccess) c->timings[5] = t + c->timings[0];
  c->assign_started = false;
  c->assigned[0] = c->assigned[1] = 0;
  return finish(c, h, c->npart, r, true);
}

int ps_gpu_set_survey(ps_gpu_ctx* c, int cat, double shot, double norm, const double* origin) {
  if (!c || cat < 0 || cat >= c->p.ncat) return fail(c, PS_GPU_ERR_ARG, "invalid survey arguments");
  bool high = false;
  for (int l = 0; l < c->p.npole; l++) high |= c->p.poles[l] > 0;
  if (high && !origin) return fail(c, PS_GPU_ERR_ARG, "survey multipoles l > 0 need the box corner");
  if (c->nmu != 1) return fail(c, PS_GPU_ERR_ARG, "survey catalogues take no |mu| sub-bins");
  if (!(norm > 0) || !(shot >= 0)) return fail(c, PS_GPU_ERR_ARG, "survey normalisation must be > 0");
  c->survey[cat] = true;
  c->survey_shot[cat] = shot;
  c->survey_norm[cat] = norm;
  if (origin)
    for (int d = 0; d < 3; d++) c->survey_origin[d] = origin[d];
  return 0;
}

int ps_gpu_learned_launch(ps_gpu_ctx* c, ps_mlp* m) {
  if (!c || !m) return fail(c, PS_GPU_ERR_ARG, "null argument");
  if (c->learned_pending) return fail(c, PS_GPU_ERR_STATE, "a learned evaluation is pending: finish it first");
  const ps_gpu_params& p = c->p;
  if (p.ncat != 1 || p.npole != 3 || p.poles[0] != 0 || p.poles[1] != 2 || p.poles[2] != 4 ||
      p.logscale || c->survey[0])
    return fail(c, PS_GPU_ERR_ARG,
                "the learned correction needs one simulation-box catalogue, poles (0, 2, 4) and "
                "linear bins");
  c->yama_last = false;
  if (!c->assigned[0]) return fail(c, PS_GPU_ERR_STATE, "catalogue 0 not assigned");
  DeviceScope dev_scope_(p.device);
  CU(dev_scope_.err);
  cudaStream_t s = c->stream;
  const int nbin = c->nbin, nmu = c->nmu, nkey = nbin * nmu, nacc = p.npole;
  if (c->lcells != nkey) {  // per-context buffers and constants
    CU(cudaStreamSynchronize(s));
    void* old[] = {c->d_lgeo, c->d_lx, c->d_lxb, c->d_lc, c->d_lout};
    for (void* b : old)
      if (b) cudaFree(b);
    if (c->h_lout) cudaFreeHost(c->h_lout);
    c->d_lgeo = c->d_lout = c->h_lout = nullptr;
    c->d_lx = c->d_lc = nullptr;
    c->d_lxb = nullptr;
    c->lcells = 0;
    const int fw = learned_feature_width();
    std::vector<double> geo((size_t)(2 + nacc) * nbin);
    for (int b = 0; b < nbin; b++) {
      geo[b] = c->kcen[b];
      geo[nbin + b] = (double)c->cnt[b];
    }
    memcpy(geo.data() + 2 * nbin, c->lcnt.data(), sizeof(double) * (size_t)nacc * nbin);
    CU(dev_malloc(&c->d_lgeo, sizeof(double) * geo.size()));
    CU(cudaMemcpy(c->d_lgeo, geo.data(), sizeof(double) * geo.size(), cudaMemcpyHostToDevice));
    CU(dev_malloc(&c->d_lx, sizeof(float) * (size_t)nkey * fw));
    CU(dev_malloc(&c->d_lxb, 2 * (size_t)nkey * fw));
    CU(dev_malloc(&c->d_lc, sizeof(float) * (size_t)nkey));
    CU(dev_malloc(&c->d_lout, sizeof(double) * (size_t)nacc * nbin));
    CU(host_malloc(&c->h_lout, sizeof(double) * (size_t)nacc * nbin));
    c->lcells = nkey;
  }
  int rc = enqueue_passes(c, c->d_sums, true);
  if (rc) return rc;
  LearnedArgs a{};
  a.sums = c->d_sums;
  a.wsum = c->d_wsum;
  a.kcen = c->d_lgeo;
  a.cnt = c->d_lgeo + nbin;
  a.lcnt = c->d_lgeo + 2 * nbin;
  a.volume = p.box[0] * p.box[1] * p.box[2];
  a.kny = M_PI * c->ng / std::max(p.box[0], std::max(p.box[1], p.box[2]));
  a.assign3 = (float)(p.assign / 3.0);
  a.interlace = p.interlace ? 1.f : 0.f;
  a.nbin = nbin;
  a.nmu = nmu;
  a.npole = nacc;
  a.x = c->d_lx;
  a.xb = c->d_lxb;
  a.c = c->d_lc;
  a.out = c->d_lout;
  if ((rc = learned_enqueue(m, a, s))) return fail(c, rc, "learned correction launch failed");
  c->launches += 3;  // features, network, combine
  double* h = c->h_out;
  CU(cudaMemcpyAsync(h, c->d_sums, sizeof(double) * (size_t)nacc * nkey, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h + (size_t)nacc * nkey, c->d_wsum, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h + (size_t)nacc * nkey + 4, c->d_err, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(c->h_lout, c->d_lout, sizeof(double) * (size_t)nacc * nbin, cudaMemcpyDeviceToHost, s));
  CU(cudaEventRecord(c->ev_done, s));
  // the next catalogue may be assigned before the finish: keep what it
  // would overwrite
  c->npart_pending[0] = c->npart[0];
  c->npart_pending[1] = c->npart[1];
  c->assign_timed_pending = c->assign_started;
  c->assign_gen_pending = c->assign_gen;
  c->assign_started = false;
  c->assigned[0] = c->assigned[1] = 0;
  c->learned_pending = true;
  return 0;
}

int ps_gpu_learned_finish(ps_gpu_ctx* c, ps_gpu_result* r, double* pl_corr) {
  if (!c || !r || !pl_corr) return fail(c, PS_GPU_ERR_ARG, "null argument");
  if (!c->learned_pending) return fail(c, PS_GPU_ERR_STATE, "no learned evaluation was launched");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  c->learned_pending = false;
  CU(cudaEventSynchronize(c->ev_done));
  float t = 0;
  // the assignment's events, unless a later assignment has recorded them again
  if (c->assign_timed_pending && c->assign_gen == c->assign_gen_pending &&
      cudaEventElapsedTime(&t, c->ev[6], c->ev[7]) == cudaSuccess)
    c->timings[0] = t;
  for (int i = 0; i < 4; i++)
    if (cudaEventElapsedTime(&t, c->ev[i], c->ev[i + 1]) == cudaSuccess) c->timings[1 + i] = t;
  if (cudaEventElapsedTime(&t, c->ev[0], c->ev[4]) == cudaSuccess) c->timings[5] = t + c->timings[0];
  const int rc = finish(c, c->h_out, c->npart_pending, r, true);
  if (rc) return rc;
  memcpy(pl_corr, c->h_lout, sizeof(double) * (size_t)c->p.npole * c->nbin);
  return 0;
}

int ps_gpu_execute_learned(ps_gpu_ctx* c, ps_mlp* m, ps_gpu_result* r, double* pl_corr) {
  if (!c || !m || !r || !pl_corr) return fail(c, PS_GPU_ERR_ARG, "null argument");
  const int rc = ps_gpu_learned_launch(c, m);
  return rc ? rc : ps_gpu_learned_finish(c, r, pl_corr);
}

int ps_gpu_set_mu_bins(ps_gpu_ctx* c, int nmu) {
  if (!c || nmu < 1 || nmu > 64) return fail(c, PS_GPU_ERR_ARG, "number of mu bins must be 1..64");
  if (nmu != 1 && (c->survey[0] || c->survey[1]))
    return fail(c, PS_GPU_ERR_ARG, "survey catalogues take no |mu| sub-bins");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  CU(cudaStreamSynchronize(c->stream));
  const int old_nmu = c->nmu;
  c->nmu = nmu;
  const int rc = plan_pass_c(c);
  if (rc) {
    c->nmu = old_nmu;
    plan_pass_c(c);
    return rc;
  }
  c->geom.nmu = nmu;
  c->kmu.clear();
  return alloc_accum(c);
}

int ps_gpu_read_kmu(const ps_gpu_ctx* c, double* out) {
  if (!c || !out) return PS_GPU_ERR_ARG;
  if (c->nmu < 2 || c->kmu.empty()) return PS_GPU_ERR_STATE;
  memcpy(out, c->kmu.data(), sizeof(double) * c->kmu.size());
  return 0;
}

int ps_gpu_read_mesh(ps_gpu_ctx* c, int cat, int m, double* out) {
  if (!c || !out || cat < 0 || cat >= c->p.ncat || m < 0 || m >= c->mpc)
    return fail(c, PS_GPU_ERR_ARG, "invalid read_mesh arguments");
  if (c->last_cat != cat || !c->assigned[cat])
    return fail(c, PS_GPU_ERR_STATE, "read_mesh: catalogue %d is not the last one assigned", cat);
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  long long* tmp = nullptr;
  CU(dev_malloc(&tmp, c->ntot * sizeof(long long) * c->mpc));
  GatherArgs g = gather_args(c, cat, c->last_pt.n);
  for (int k = 0; k < c->mpc; k++) g.out64[k] = tmp + (size_t)k * c->ntot;
  launch_gather_assign(c->last_pt, g, c->stream, true);
  std::vector<long long> q(c->ntot);
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaMemcpyAsync(q.data(), tmp + (size_t)m * c->ntot, c->ntot * 8,
                                   cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e3 = cudaStreamSynchronize(c->stream);
  cudaFree(tmp);
  CU(e1);
  CU(e2);
  CU(e3);
  for (size_t i = 0; i < c->ntot; i++) out[i] = (double)q[i] * kFixInv;
  return 0;
}

int ps_gpu_fft_r2c_host(ps_gpu_ctx* c, const float* in, float* out) {
  if (!c || !in || !out) return fail(c, PS_GPU_ERR_ARG, "null argument");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  cudaStream_t s = c->stream;
  const int ng = c->ng;
  float* d_in = (float*)c->grid[0];  // ntot floats fit in the mesh buffer
  CU(cudaMemcpyAsync(d_in, in, c->ntot * sizeof(float), cudaMemcpyHostToDevice, s));
  PassAArgs a;
  memset(&a, 0, sizeof a);
  a.ng = ng;
  a.ty = c->ty_a;
  a.fgrid = d_in;
  a.out = c->cbuf[0];
  a.tw_half = c->d_tw_half;
  a.tw_full = c->d_tw_full;
  a.plan_half = c->plan_half;
  a.pipe_grid = 0;
  a.radix32 = 0;
  a.err = c->d_err + 2;
  a.twl = (c->wfft & 1) ? c->d_twl_half : nullptr;
  launch_pass_a(a, s);
  PassBArgs b;
  memset(&b, 0, sizeof b);
  b.ng = ng;
  b.tx = c->tx_b;
  b.twl = (c->wfft & 2) ? c->d_twl_full : nullptr;
  b.in = c->cbuf[0];
  b.out = (float2*)c->grid[0];
  b.tw_full = c->d_tw_full;
  b.plan_full = c->plan_full;
  b.pipe_grid = 0;
  b.radix32 = 0;
  b.err = c->d_err + 2;
  launch_pass_b(b, s);
  PassCArgs pc;
  memset(&pc, 0, sizeof pc);
  pc.ng = ng;
  pc.ty = std::max(1, std::min(ng, kPassCElems / ng));
  pc.nfield = 1;
  pc.ncat = 1;
  pc.nspec = 1;
  pc.in[0] = (const float2*)c->grid[0];
  pc.store = c->cbuf[0];
  pc.tw_full = c->d_tw_full;
  pc.plan_full = c->plan_full;
  pc.geom = c->geom;
  pc.twl = (c->wfft & 4) ? c->d_twl_full : nullptr;
  launch_pass_c(pc, s);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, c->cbuf[0], c->ncx * sizeof(float2), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int ps_gpu_bin_fields_host(ps_gpu_ctx* c, const float* f1, const float* f2, double* pl) {
  if (!c || !f1 || !f2 || !pl) return fail(c, PS_GPU_ERR_ARG, "null argument");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  cudaStream_t s = c->stream;
  const int npole = c->p.npole, nbin = c->nbin;
  float2* d1 = c->cbuf[0];
  float2* d2 = (float2*)c->grid[0];
  CU(cudaMemcpyAsync(d1, f1, c->ncx * sizeof(float2), cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d2, f2, c->ncx * sizeof(float2), cudaMemcpyHostToDevice, s));
  CU(cudaMemsetAsync(c->d_part, 0, sizeof(double) * (size_t)c->grid_c * npole * nbin, s));
  BinFieldArgs b;
  b.ng = c->ng;
  b.f1 = d1;
  b.f2 = d2;
  b.geom = c->geom;
  b.geom.nmu = 1;
  b.partials = reinterpret_cast<float2*>(c->d_part);
  b.grid = c->grid_c;
  launch_bin_fields(b, s);
  launch_reduce(reinterpret_cast<const float2*>(c->d_part), c->grid_c, npole * nbin, c->d_sums, s);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(pl, c->d_sums, sizeof(double) * (size_t)npole * nbin, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}


// ---- ensembles: one CUDA graph per batch of catalogues -----------------

}  // extern "C"

struct ps_gpu_batch {
  ps_gpu_ctx* c = nullptr;
  int ncat = 0;
  std::vector<size_t> n;
  size_t stride = 0;          // doubles per catalogue: sums, wsum[4], 4 error ints
  double* d_res = nullptr;    // [ncat][stride]
  double* h_res = nullptr;    // pinned copy
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
};

namespace {

void batch_free(ps_gpu_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->d_res) cudaFree(b->d_res);
  if (b->h_res) cudaFreeHost(b->h_res);
  delete b;
}

// Enqueues catalogue i of the batch (assignment, passes, reduction, result
// slot); returns a status like the entry points.
int batch_enqueue(ps_gpu_ctx* c, ps_gpu_batch* b, int i, const double* xyzw) {
  cudaStream_t s = c->stream;
  const int nacc = c->nspec * c->p.npole, nkey = c->nbin * c->nmu;
  double* slot = b->d_res + (size_t)i * b->stride;
  CU(cudaMemsetAsync(c->d_wsum, 0, sizeof(double) * 4, s));
  CU(cudaMemsetAsync(c->d_err, 0, sizeof(int) * 4, s));
  if (b->n[i]) {
    Particles pt{};
    pt.aos = xyzw;
    pt.n = b->n[i];
    b->launches += launch_gather_assign(pt, gather_args(c, 0, pt.n), s, false);
  }
  CU(cudaGetLastError());
  const int launches0 = c->launches;
  const int rc = enqueue_passes(c, slot, false);
  b->launches += c->launches - launches0;
  if (rc) return rc;
  CU(cudaMemcpyAsync(slot + (size_t)nacc * nkey, c->d_wsum, sizeof(double) * 4,
                     cudaMemcpyDeviceToDevice, s));
  CU(cudaMemcpyAsync(slot + (size_t)nacc * nkey + 4, c->d_err, sizeof(int) * 4,
                     cudaMemcpyDeviceToDevice, s));
  return 0;
}

}  // namespace

extern "C" {

int ps_gpu_batch_create(ps_gpu_ctx* c, int ncat, const double* const* xyzw, const size_t* n,
                        ps_gpu_batch** out) {
  if (!c || !out || ncat < 1 || !xyzw || !n) return fail(c, PS_GPU_ERR_ARG, "invalid batch arguments");
  *out = nullptr;
  if (c->p.ncat != 1) return fail(c, PS_GPU_ERR_ARG, "batches need a single-catalogue context");
  if (c->survey[0]) return fail(c, PS_GPU_ERR_ARG, "batches take simulation-box catalogues");
  size_t nmax = 0;
  for (int i = 0; i < ncat; i++) {
    if (n[i] && (!xyzw[i] || ((uintptr_t)xyzw[i] & 31)))
      return fail(c, PS_GPU_ERR_ARG, "batch catalogue %d: device records must be 32-byte aligned", i);
    if (n[i] >= 0xffffffffull) return fail(c, PS_GPU_ERR_RANGE, "batch catalogue %d: too many particles", i);
    nmax = std::max(nmax, n[i]);
  }
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  int rc = ensure_gather_capacity(c, nmax);
  for (int i = 0; i < ncat && !rc; i++)
    if (n[i] && use_region(c, n[i])) rc = ensure_region(c);
  if (rc) return rc;
  ps_gpu_batch* b = new ps_gpu_batch;
  b->c = c;
  b->ncat = ncat;
  b->n.assign(n, n + ncat);
  const int nacc = c->nspec * c->p.npole, nkey = c->nbin * c->nmu;
  b->stride = (size_t)nacc * nkey + 6;
  cudaError_t e = dev_malloc(&b->d_res, sizeof(double) * b->stride * ncat);
  if (e == cudaSuccess) e = host_malloc(&b->h_res, sizeof(double) * b->stride * ncat);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    batch_free(b);
    (void)cudaGetLastError();
    return fail(c, e == cudaErrorMemoryAllocation ? PS_GPU_ERR_MEMORY : PS_GPU_ERR_CUDA,
                "batch set-up: %s", cudaGetErrorString(e));
  }
  // Record every launch; the capture is always ended, also on an error.
  e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    batch_free(b);
    return fail(c, PS_GPU_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
  }
  for (int i = 0; i < ncat && !rc; i++) rc = batch_enqueue(c, b, i, xyzw[i]);
  if (!rc) {
    e = cudaMemcpyAsync(b->h_res, b->d_res, sizeof(double) * b->stride * ncat, cudaMemcpyDeviceToHost,
                        c->stream);
    if (e != cudaSuccess) rc = fail(c, PS_GPU_ERR_CUDA, "batch copy: %s", cudaGetErrorString(e));
  }
  const cudaError_t ee = cudaStreamEndCapture(c->stream, &b->graph);
  if (!rc && ee != cudaSuccess) rc = fail(c, PS_GPU_ERR_CUDA, "stream capture: %s", cudaGetErrorString(ee));
  if (!rc) {
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) rc = fail(c, PS_GPU_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
  }
  if (rc) {
    cudaGetLastError();
    batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}

int ps_gpu_batch_launch(ps_gpu_batch* b, int wait) {
  if (!b) return PS_GPU_ERR_ARG;
  ps_gpu_ctx* c = b->c;
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  CU(cudaGraphLaunch(b->exec, c->stream));
  c->launches = b->launches;
  if (wait) CU(cudaStreamSynchronize(c->stream));
  return 0;
}

int ps_gpu_batch_wait(ps_gpu_batch* b) {
  if (!b) return PS_GPU_ERR_ARG;
  ps_gpu_ctx* c = b->c;
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  CU(cudaStreamSynchronize(c->stream));
  return 0;
}

// ---- one graph over several batches
struct ps_gpu_ensemble {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<ps_gpu_batch*> batches;
};

static void ensemble_free(ps_gpu_ensemble* e) {
  if (!e) return;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

int ps_gpu_ensemble_create(ps_gpu_batch* const* batches, int nbatch, ps_gpu_ensemble** out) {
  if (!batches || nbatch < 1 || !out) return PS_GPU_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < nbatch; i++)
    if (!batches[i] || batches[i]->c->p.device != batches[0]->c->p.device) return PS_GPU_ERR_ARG;
  ps_gpu_ctx* c = batches[0]->c;
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  for (int i = 0; i < nbatch; i++)
    for (int j = 0; j < i; j++)
      if (batches[i]->c == batches[j]->c)
        return fail(c, PS_GPU_ERR_ARG, "ensemble: batches %d and %d share a context", j, i);
  ps_gpu_ensemble* e = new ps_gpu_ensemble;
  e->device = c->p.device;
  e->batches.assign(batches, batches + nbatch);
  cudaError_t err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaGraphCreate(&e->graph, 0);
  // each batch a child graph without dependencies: their contexts' buffers
  // are disjoint, so the batches run concurrently
  for (int i = 0; i < nbatch && err == cudaSuccess; i++) {
    cudaGraphNode_t node;
    err = cudaGraphAddChildGraphNode(&node, e->graph, nullptr, 0, batches[i]->graph);
  }
  if (err == cudaSuccess) err = cudaGraphInstantiate(&e->exec, e->graph, 0);
  if (err != cudaSuccess) {
    (void)cudaGetLastError();
    ensemble_free(e);
    return fail(c, err == cudaErrorMemoryAllocation ? PS_GPU_ERR_MEMORY : PS_GPU_ERR_CUDA,
                "ensemble graph: %s", cudaGetErrorString(err));
  }
  *out = e;
  return 0;
}

int ps_gpu_ensemble_launch(ps_gpu_ensemble* e, int wait) {
  if (!e) return PS_GPU_ERR_ARG;
  ps_gpu_ctx* c = e->batches[0]->c;
  DeviceScope dev_scope_(e->device);
  CU(dev_scope_.err);
  CU(cudaGraphLaunch(e->exec, e->stream));
  if (wait) CU(cudaStreamSynchronize(e->stream));
  return 0;
}

int ps_gpu_ensemble_wait(ps_gpu_ensemble* e) {
  if (!e) return PS_GPU_ERR_ARG;
  ps_gpu_ctx* c = e->batches[0]->c;
  DeviceScope dev_scope_(e->device);
  CU(dev_scope_.err);
  CU(cudaStreamSynchronize(e->stream));
  return 0;
}

void ps_gpu_ensemble_destroy(ps_gpu_ensemble* e) {
  if (!e) return;
  DeviceScope dev_scope_(e->device);
  ensemble_free(e);
}

int ps_gpu_batch_result(ps_gpu_batch* b, int i, ps_gpu_result* r) {
  if (!b || !r || i < 0 || i >= b->ncat) return b ? fail(b->c, PS_GPU_ERR_ARG, "invalid batch result index") : PS_GPU_ERR_ARG;
  return finish(b->c, b->h_res + (size_t)i * b->stride, &b->n[i], r, false);
}

int ps_gpu_batch_launches(const ps_gpu_batch* b) { return b ? b->launches : PS_GPU_ERR_ARG; }

void ps_gpu_batch_destroy(ps_gpu_batch* b) {
  if (!b) return;
  DeviceScope dev_scope_(b->c->p.device);
  cudaStreamSynchronize(b->c->stream);
  batch_free(b);
}

// ---- autotuner ----------------------------------------------------------

int ps_gpu_set_warp_fft(ps_gpu_ctx* c, int mask) {
  if (!c) return PS_GPU_ERR_ARG;
  const int avail = warp_avail(c);
  if (mask >= 0) {
    DeviceScope dev_scope_(c->p.device);
    CU(dev_scope_.err);
    CU(cudaStreamSynchronize(c->stream));
    c->wfft = mask & avail;
  }
  return c->wfft;
}

int ps_gpu_set_tuning(ps_gpu_ctx* c, const int* choice) {
  if (!c || !choice) return fail(c, PS_GPU_ERR_ARG, "invalid set_tuning arguments");
  if (choice[0] != -1 && choice[0] != 0 && choice[0] != 256 && choice[0] != 512)
    return fail(c, PS_GPU_ERR_ARG, "gather threads: 0 (by density), 256 or 512");
  DeviceScope dev_scope_(c->p.device);
  CU(dev_scope_.err);
  CU(cudaStreamSynchronize(c->stream));
  if (choice[0] >= 0) c->gather_threads = choice[0];
  if (choice[1] >= 0) c->radix32_a = choice[1] != 0;
  if (choice[2] >= 0) c->radix32_b = choice[2] != 0;
  if (choice[3] >= 0) c->pipe_c_on = choice[3] != 0;
  if (choice[4] >= 0) c->gather_sparse_max = choice[4] ? 0xffffffffu : 512u;
  if (choice[5] >= 0) c->gather_region = choice[5] >= 2 ? -1 : choice[5];
  plan_pipes(c);
  return 0;
}

int ps_gpu_autotune(ps_gpu_ctx* c, const double* xyzw, size_t n, int reps, int* choice) {
  if (!c || !xyzw || !n || reps < 1) return fail(c, PS_GPU_ERR_ARG, "invalid autotune arguments");
  if (c->p.ncat != 1) return fail(c, PS_GPU_ERR_ARG, "autotune needs a single-catalogue context");
  ps_gpu_result r;
  memset(&r, 0, sizeof r);
  // mean phase times of `reps` evaluations (after one untimed)
  auto measure = [&](float* t) -> int {
    for (int k = 0; k < 6; k++) t[k] = 0.f;
    for (int it = 0; it <= reps; it++) {
      int rc = ps_gpu_assign_aos(c, 0, xyzw, n, 1);
      if (!rc) rc = ps_gpu_execute(c, &r);
      if (rc) return rc;
      if (it)
        for (int k = 0; k < 6; k++) t[k] += c->timings[k] / reps;
    }
    return 0;
  };
  float t[6];
  int rc;
  // gather CTA size (phase 0)
  {
    const int cand[2] = {256, 512};
    float best = 1e30f;
    int arg = c->gather_threads;
    for (int k = 0; k < 2; k++) {
      c->gather_threads = cand[k];
      if ((rc = measure(t))) return rc;
      if (t[0] < best) { best = t[0]; arg = cand[k]; }
    }
    c->gather_threads = arg;
  }
  // region gather or tile gather (phase 0), timed where neither clearly
  // wins: between 1/256 and 1/8 particles per cell, with a region buffer of
  // at most 16 GB; elsewhere the density rule of use_region decides
  c->gather_region = -1;
  const double density = (double)n / (double)c->ntot;
  if (gather_region_ok(c->ng, c->gT, c->p.assign) && region_need(c) <= ((size_t)16 << 30) &&
      density >= 1.0 / 256 && density < 1.0 / 8) {
    float best = 1e30f;
    int arg = c->gather_region;
    for (int k = 0; k < 2; k++) {
      c->gather_region = k;
      if ((rc = measure(t))) return rc;
      if (t[0] < best) { best = t[0]; arg = k; }
    }
    c->gather_region = arg;
  }
  // dense tiles: one record per warp or lane groups (phase 0)
  {
    const unsigned cand[2] = {512u, 0xffffffffu};
    float best = 1e30f;
    unsigned arg = c->gather_sparse_max;
    for (int k = 0; k < 2; k++) {
      c->gather_sparse_max = cand[k];
      if ((rc = measure(t))) return rc;
      if (t[0] < best) { best = t[0]; arg = cand[k]; }
    }
    c->gather_sparse_max = arg;
  }
  const bool pipe = c->plan_full.logn >= 0 && !getenv("PS_GPU_NO_PIPELINE");
  if (pipe) {
    // z-pass variant (phase 1), y-pass variant (phase 2), pass C (phase 3)
    for (int knob = 0; knob < 3; knob++) {
      if (knob == 2 && c->grid_ct <= 0) break;
      bool* v = knob == 0 ? &c->radix32_a : knob == 1 ? &c->radix32_b : &c->pipe_c_on;
      float best = 1e30f;
      bool arg = *v;
      for (int k = 0; k < 2; k++) {
        *v = (k == 1);
        plan_pipes(c);
        if ((rc = measure(t))) return rc;
        if (t[1 + knob] < best) { best = t[1 + knob]; arg = *v; }
      }
      *v = arg;
      plan_pipes(c);
    }
  }
  // warp-register form of each pass against the block-tiled one (phases
  // 1, 2, 3), where the mesh size has one
  {
    const int avail = warp_avail(c);
    for (int bit = 0; bit < 3; bit++) {
      const int m = 1 << bit;
      if (!(avail & m)) continue;
      float best = 1e30f;
      int arg = c->wfft & m;
      for (int k = 0; k < 2; k++) {
        c->wfft = k ? (c->wfft | m) : (c->wfft & ~m);
        if ((rc = measure(t))) return rc;
        if (t[1 + bit] < best) { best = t[1 + bit]; arg = k ? m : 0; }
      }
      c->wfft = (c->wfft & ~m) | arg;
    }
  }
  if (choice) {
    choice[4] = c->gather_sparse_max == 0xffffffffu ? 1 : 0;
    choice[0] = c->gather_threads;
    choice[1] = c->radix32_a;
    choice[2] = c->radix32_b;
    choice[3] = c->pipe_c_on;
    choice[5] = use_region(c, n) ? 1 : 0;
  }
  return 0;
}

void ps_gpu_debug_fail_alloc(int n) { g_fail_alloc.store(n > 0 ? n : 0); }

int ps_gpu_debug_stall_pipeline(ps_gpu_ctx* c, int polls) {
  if (!c || polls < 1) return PS_GPU_ERR_ARG;
  c->stall = polls;
  return 0;
}

}  // extern "C"
