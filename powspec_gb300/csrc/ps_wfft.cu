// ps_wfft.cu -- warp-register FFT passes for power-of-two meshes.
//
// Each warp transforms whole lines in registers, with no block barrier
// inside a transform.  A line of N = L * V complex values is held by L lanes,
// V values each, lane l holding x[l + L m] (G = 32 / L lines per warp, so
// every load instruction reads 32 consecutive values of G lines):
//
//   X[k1 + V k2] = sum_l W_L^(l k2) W_N^(l k1) sum_m x[l + L m] W_V^(m k1)
//
//   1. a V-point DFT over m in each lane's registers;
//   2. the twiddles W_N^(l k1), read as one coalesced row per k1 from a
//      table twl[k1 L + l] built on the host in FP64;
//   3. a transpose through the warp's own shared memory (__syncwarp only);
//   4. R = V / L L-point DFTs over l per lane.
//
// After step 4 lane l of line g holds X[(l R + j) + V k2] in x[j L + k2].
// Shapes: N = 128 (L 8, V 16), 256 (L 16, V 16), 512 (L 16, V 32), 1024
// (L 32, V 32).  The passes that use it:
//
//   k_pass_a_w  z transform of the real mesh rows [x][y][z] (length M =
//               Ng / 2 complex, the half-length r2c), the r2c split and the
//               transposed store A[x][kz][y] from a tile of consecutive y;
//   k_pass_b_w  y transform A[x][kz][y] -> B[kz][ky][x] from a tile of
//               consecutive x, stored through shared memory in runs over x;
//   k_pass_c_w  x transform of every field's line B[kz][ky][.], then the
//               interlace combine, window and binning of ps_bin.cu's
//               bin_lines on the warp's own lines.
//
// The reference transform is FFTW's unnormalised forward r2c
// (src/fftw_define.h:56, called at src/multipole.c:444,459).
#include "ps_bin_core.cuh"

namespace ps {
namespace {

template <int N>
struct WShape;
template <>
struct WShape<128> {
  static constexpr int L = 8, V = 16;
};
template <>
struct WShape<256> {
  static constexpr int L = 16, V = 16;
};
template <>
struct WShape<512> {
  static constexpr int L = 16, V = 32;
};
template <>
struct WShape<1024> {
  static constexpr int L = 32, V = 32;
};

template <int N>
struct WF {
  static constexpr int L = WShape<N>::L, V = WShape<N>::V;
  static constexpr int G = 32 / L;          // lines per warp
  static constexpr int R = V / L;           // L-point DFTs per lane
  static constexpr int SROW = L + 1;        // transpose row (complex)
  static constexpr int SLINE = V * SROW;    // transpose area of one line
  static constexpr int SWARP = G * SLINE;   // of one warp
};

// Forward DFT of the G lines a warp holds (see the file comment).  S: the
// warp's transpose area, WF<N>::SWARP complex values.
template <int N>
__device__ __forceinline__ void wfft(float2 (&x)[WF<N>::V], float2* S,
                                     const float2* __restrict__ twl, int lane) {
  constexpr int L = WF<N>::L, V = WF<N>::V, R = WF<N>::R, SROW = WF<N>::SROW;
  const int g = lane / L, l = lane - g * L;
  dft<V>(x);
#pragma unroll
  for (int k1 = 1; k1 < V; k1++) x[k1] = cmul(x[k1], ldtw(&twl[k1 * L + l]));
  float2* Sg = S + g * WF<N>::SLINE;
#pragma unroll
  for (int k1 = 0; k1 < V; k1++) Sg[k1 * SROW + l] = x[k1];
  __syncwarp();
#pragma unroll
  for (int j = 0; j < R; j++)
#pragma unroll
    for (int q = 0; q < L; q++) x[j * L + q] = Sg[(l * R + j) * SROW + q];
  __syncwarp();
#pragma unroll
  for (int j = 0; j < R; j++) {
    float2 t[L];
#pragma unroll
    for (int q = 0; q < L; q++) t[q] = x[j * L + q];
    dft<L>(t);
#pragma unroll
    for (int q = 0; q < L; q++) x[j * L + q] = t[q];
  }
}

constexpr int kWarpsAB = 4;  // warps per CTA of the z and y passes but below
// warps per CTA of the z pass: 8 at Ng = 512 and 2048, so that its
// transposed stores A[x][kz][y] run over 8 G consecutive y (128 and 64
// bytes) instead of 4 G (z pass 0.425 -> 0.369 ms at 512, 35.1 -> 30.3 ms at
// 2048, two meshes); at 1024 eight warps measured slower (3.55 -> 3.81 ms)
template <int NG>
__host__ __device__ constexpr int warps_a() { return (NG == 512 || NG == 2048) ? 8 : kWarpsAB; }
// warps per CTA of the y pass: 8 at Ng = 1024, whose 4-warp tile stored
// runs of 4 x (32 bytes) at 5 CTAs per SM (y pass 3.95 -> 3.52 ms, two
// meshes); at 512 eight warps measured slower (0.459 -> 0.501 ms), at 256
// the same
template <int N>
__host__ __device__ constexpr int warps_b() { return N == 1024 ? 8 : kWarpsAB; }

// z transform: real rows of the FP32 mesh (minus its mean) -> A[x][kz][y].
template <int NG>
__global__ void __launch_bounds__(32 * warps_a<NG>()) k_pass_a_w(const __grid_constant__ PassAArgs a) {
  constexpr int M = NG / 2;
  using S = WF<M>;
  constexpr int TY = warps_a<NG>() * S::G;  // y rows per tile
  constexpr int TL = M + 1;                 // tile line (odd)
  extern __shared__ float2 wsm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / S::L, l = lane - g * S::L;
  float2* T = wsm;                    // [TY][TL], over the transpose areas once they are done
  float2* scr = wsm + w * S::SWARP;
  constexpr int nty = NG / TY;
  const int x = blockIdx.x / nty, y0 = (blockIdx.x - x * nty) * TY;
  const int r = w * S::G + g;
  const float2* src =
      reinterpret_cast<const float2*>(a.fgrid + ((size_t)x * NG + y0 + r) * NG) + l;
  float2 v[S::V];
#pragma unroll
  for (int m = 0; m < S::V; m++) v[m] = __ldcs(src + m * S::L);
  if (a.yw && (x != 0 || y0 + r != 0)) {
    // survey harmonic: cell (x, y, z) weighted by Y_lm of its position,
    // the (x, y) part once per line (1 on the row x = y = 0, as in k_pass_a)
    const YlmRow w = ylm_row(a.yc, (x + a.org[0]) * a.len[0], (y0 + r + a.org[1]) * a.len[1]);
#pragma unroll
    for (int m = 0; m < S::V; m++) {
      const int z = 2 * (l + S::L * m);
      v[m].x *= ylm_cell(a.yc, w, (z + a.org[2]) * a.len[2]);
      v[m].y *= ylm_cell(a.yc, w, (z + 1 + a.org[2]) * a.len[2]);
    }
  }
  wfft<M>(v, scr, a.twl, lane);
  __syncthreads();  // every warp's transform is done with its transpose area
#pragma unroll
  for (int j = 0; j < S::R; j++)
#pragma unroll
    for (int k2 = 0; k2 < S::L; k2++) T[r * TL + (l * S::R + j) + S::V * k2] = v[j * S::L + k2];
  __syncthreads();
  // r2c split of Z = FFT(x[2m] + i x[2m+1]): X[k] = E[k] + W_NG^k O[k],
  // E = (Z[k] + Z*[M-k]) / 2, O = -i (Z[k] - Z*[M-k]) / 2; stored as runs
  // of TY consecutive y
  float2* dst = a.out + (size_t)x * (M + 1) * NG + y0;
  for (int e = threadIdx.x; e < (M + 1) * TY; e += blockDim.x) {
    const int kz = e / TY, rr = e - kz * TY;
    const float2* Lr = T + rr * TL;
    float2 X;
    if (kz == 0 || kz == M) {
      const float2 z = Lr[0];
      X = make_float2(kz == 0 ? z.x + z.y : z.x - z.y, 0.f);
    } else {
      const float2 A = Lr[kz], B = Lr[M - kz];
      const float2 E = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
      const float2 O = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
      X = cadd(E, cmul(__ldg(&a.tw_full[kz]), O));
    }
    dst[(size_t)kz * NG + rr] = X;
  }
}

// y transform: A[x][kz][y] -> B[kz][ky][x].
template <int N>
__global__ void __launch_bounds__(32 * warps_b<N>()) k_pass_b_w(const __grid_constant__ PassBArgs a) {
  using S = WF<N>;
  constexpr int TX = warps_b<N>() * S::G;  // x lines per tile
  constexpr int TP = TX + 1;           // tile row (odd)
  constexpr int ngk = N / 2 + 1;
  constexpr int ntx = N / TX;
  extern __shared__ float2 wsm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / S::L, l = lane - g * S::L;
  float2* T = wsm;                    // [N][TP], over the transpose areas once they are done
  float2* scr = wsm + w * S::SWARP;
  const int kz = blockIdx.x / ntx, x0 = (blockIdx.x - kz * ntx) * TX;
  const int col = w * S::G + g;
  const float2* src = a.in + ((size_t)(x0 + col) * ngk + kz) * N + l;
  float2 v[S::V];
#pragma unroll
  for (int m = 0; m < S::V; m++) v[m] = __ldcs(src + m * S::L);
  wfft<N>(v, scr, a.twl, lane);
  __syncthreads();  // every warp's transform is done with its transpose area
#pragma unroll
  for (int j = 0; j < S::R; j++)
#pragma unroll
    for (int k2 = 0; k2 < S::L; k2++) T[((l * S::R + j) + S::V * k2) * TP + col] = v[j * S::L + k2];
  __syncthreads();
  float2* dst = a.out + (size_t)kz * N * N + x0;
  for (int e = threadIdx.x; e < N * TX; e += blockDim.x) {
    const int ky = e / TX, xl = e - ky * TX;
    dst[(size_t)ky * N + xl] = T[ky * TP + xl];
  }
}

// x transform in store mode (survey harmonic terms, the host r2c): a CTA
// takes 8 lines of consecutive kz at one ky (one field), each warp
// transforms G of them, and through a shared [kx][9] tile (over the
// transpose areas, after a CTA barrier) the CTA writes F[x][y][kz] in runs
// of 8 kz: out = X (acc_mode 0), X * Y_lm(k^) (1) or out + X * Y_lm(k^)
// (2), with Y_lm = 1 for k_x = k_y = 0 (src/mp_template.c:118-121), as
// k_pass_c does.  The last kz tile holds fewer lines: its idle groups
// transform line kz0 again and store nothing.
constexpr int kStoreKz = 8;
template <int N>
__global__ void __launch_bounds__(32 * (kStoreKz / WF<N>::G)) k_pass_c_ws(const __grid_constant__ PassCArgs a) {
  using S = WF<N>;
  constexpr int ngk = N / 2 + 1, TP = kStoreKz + 1;
  constexpr int nkt = (ngk + kStoreKz - 1) / kStoreKz;
  extern __shared__ float2 wsm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / S::L, l = lane - g * S::L;
  float2* T = wsm;  // [N][TP], over the warps' transpose areas once they are done
  float2* scr = wsm + w * S::SWARP;
  const int ky = blockIdx.x / nkt, kz0 = (blockIdx.x - ky * nkt) * kStoreKz;
  const int nl = min(kStoreKz, ngk - kz0);
  const int r = w * S::G + g;  // this group's line: kz0 + r
  const bool live = r < nl;
  const float2* src = a.in[0] + ((size_t)(live ? kz0 + r : kz0) * N + ky) * N + l;
  float2 v[S::V];
#pragma unroll
  for (int m = 0; m < S::V; m++) v[m] = __ldcs(src + m * S::L);
  wfft<N>(v, scr, a.twl, lane);
  __syncthreads();
  if (live) {
#pragma unroll
    for (int j = 0; j < S::R; j++)
#pragma unroll
      for (int k2 = 0; k2 < S::L; k2++) T[((l * S::R + j) + S::V * k2) * TP + r] = v[j * S::L + k2];
  }
  __syncthreads();
  const int jp = dsigned(ky, N);
  for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
    const int i = e / nl, rr = e - i * nl;
    const size_t idx = ((size_t)i * N + ky) * ngk + kz0 + rr;
    float2 x = T[i * TP + rr];
    if (a.acc_mode) {
      const int ip = dsigned(i, N);
      const float y = (ip == 0 && jp == 0)
                          ? 1.f
                          : ylm_eval(a.yk, ip * a.kinv[0], jp * a.kinv[1], (kz0 + rr) * a.kinv[2]);
      x = make_float2(x.x * y, x.y * y);
      if (a.acc_mode == 2) {
        const float2 o = a.store[idx];
        x = make_float2(x.x + o.x, x.y + o.y);
      }
    }
    a.store[idx] = x;
  }
}

// Complex values per warp of the x pass: NP positions x nfield lines in the
// padded layout, plus what the transpose area needs beyond G lines.
template <int N>
__host__ __device__ constexpr int wc_np(int nfield) {
  return WF<N>::G > nfield ? WF<N>::G / nfield : 1;
}
template <int N>
__host__ __device__ constexpr int wc_line() {
  return N + (N - 1) / 32;  // padded line (odd), as line_stride(N, true)
}
template <int N>
__host__ __device__ constexpr int wc_warp_elems(int nfield) {
  return ((wc_np<N>(nfield) * nfield * wc_line<N>() +
           (WF<N>::SWARP > WF<N>::G * wc_line<N>() ? WF<N>::SWARP - WF<N>::G * wc_line<N>() : 0)) +
          1) &
         ~1;
}
constexpr int kMaxWarpsC = 16;  // warps per CTA of the x pass: 4 or 16 (host's choice)

// x transform + combine + window + binning.  A work item of a warp is NP
// consecutive ky at one kz (NP > 1 when a transform holds more lines than
// there are fields); every CTA step gives one item to each warp, and the
// tile sums are merged into the CTA's FP32-pair partials every kMergeEvery
// steps of 4 warps' items (fewer steps with more warps).  Large tile sums
// (|mu| sub-bins) take the CTA's shared memory: then 16 warps share them,
// so that more warps are resident.
// PY: items are (kz, |ky|) and a warp transforms line ky, then line Ng - ky,
// binned together (ypair_powers / ypair_bin; line of sight along z, moment
// form, one line per field in a transform).
template <int N, int NSPEC, int MOM, int WPC, bool PY>
__global__ void __launch_bounds__(32 * WPC, WPC == 4 ? (PY && N == 512 ? 3 : 0) : (PY ? 1 : 2))
    k_pass_c_w(const __grid_constant__ PassCArgs a) {
  using S = WF<N>;
  constexpr int LS = wc_line<N>();
  extern __shared__ __align__(16) float2 wsm[];
  __shared__ int srange[2];
  constexpr int nwc = WPC;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / S::L, l = lane - g * S::L;
  const int nfield = a.nfield;
  constexpr int merge_every = (kMergeEvery * 4 / WPC > 1) ? kMergeEvery * 4 / WPC : 1;
  const int NP = wc_np<N>(nfield);
  const int nline = NP * nfield;
  const int wel = wc_warp_elems<N>(nfield);
  float2* X = wsm + w * wel;  // this warp's lines [field][pos][LS]
  float* tacc = reinterpret_cast<float*>(wsm + nwc * wel);
  const ModeGeom& gm = a.geom;
  const int nacc = NSPEC * gm.npole;
  const int nkey = gm.nbin * gm.nmu;
  float2* part = a.partials + (size_t)blockIdx.x * nacc * nkey;
  for (int e = threadIdx.x; e < tile_accs<NSPEC, MOM>(gm) * nkey; e += blockDim.x) tacc[e] = 0.f;
  if (threadIdx.x == 0) {
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
  // (kz, ky0) with ky0 a multiple of NP; with PY (kz, |ky|)
  const int nitem = PY ? (N / 2 + 1) * (N / 2 + 1) : (N / 2 + 1) * (N / NP);
  const int nstep = (nitem + (int)gridDim.x * nwc - 1) / ((int)gridDim.x * nwc);
  int nacc_steps = 0;
  for (int st = 0; st < nstep; st++) {
    const int item = (st * (int)gridDim.x + (int)blockIdx.x) * nwc + w;
    int lo = 0x7fffffff, hi = -1;
    if (PY && item < nitem) {
      if constexpr (PY) {
        const int kz = item / (N / 2 + 1), kyp = item - kz * (N / 2 + 1);
        int spec_a[NSPEC], spec_b[NSPEC];
#pragma unroll
        for (int s = 0; s < NSPEC; s++) {
          spec_a[s] = a.spec_a[s];
          spec_b[s] = a.spec_b[s];
        }
        float pw[YPairRuns<N>::NC][YPairRuns<N>::RP + 1][NSPEC];
        const int nly = (kyp == 0 || 2 * kyp == N) ? 1 : 2;
        for (int t = 0; t < nly; t++) {
          const int ky = t ? N - kyp : kyp;
          // field f of line ky, G at a time (nfield >= G here)
          for (int f0 = 0; f0 < nfield; f0 += S::G) {
            const int f = f0 + g;
            const float2* src = a.in[f] + ((size_t)kz * N + ky) * N + l;
            float2 v[S::V];
#pragma unroll
            for (int m = 0; m < S::V; m++) v[m] = __ldcs(src + m * S::L);
            wfft<N>(v, X + f0 * LS, a.twl, lane);
            float2* out = X + f * LS;
#pragma unroll
            for (int j = 0; j < S::R; j++)
#pragma unroll
              for (int k2 = 0; k2 < S::L; k2++) {
                const int kx = (l * S::R + j) + S::V * k2;
                out[kx + (kx >> 5)] = v[j * S::L + k2];
              }
            __syncwarp();
          }
          ypair_powers<N, NSPEC>(a, X, LS, kz, ky, pw, t > 0, lane, spec_a, spec_b);
          __syncwarp();  // the next line's transform overwrites X
        }
        ypair_bin<N, NSPEC, MOM>(a, kz, kyp, pw, tacc, lo, hi, lane);
      }
    } else if (item < nitem) {
      const int kz = item / (N / NP), ky0 = (item - kz * (N / NP)) * NP;
      // lines e = pos * nfield + f, G at a time; line e -> buffer f * NP + pos
      for (int e0 = 0; e0 < nline; e0 += S::G) {
        const int e = e0 + g, f = e % nfield, pos = e / nfield;
        const float2* src = a.in[f] + ((size_t)kz * N + ky0 + pos) * N + l;
        float2 v[S::V];
#pragma unroll
        for (int m = 0; m < S::V; m++) v[m] = __ldcs(src + m * S::L);
        wfft<N>(v, X + e0 * LS, a.twl, lane);  // transpose area: this group's lines onward
        float2* out = X + (f * NP + pos) * LS;
#pragma unroll
        for (int j = 0; j < S::R; j++)
#pragma unroll
          for (int k2 = 0; k2 < S::L; k2++) {
            const int kx = (l * S::R + j) + S::V * k2;
            out[kx + (kx >> 5)] = v[j * S::L + k2];
          }
        __syncwarp();
      }
      bin_lines<NSPEC, true, MOM>(a, X, LS, kz, ky0, NP, tacc, lo, hi, lane, 32);
    }
    note_range(srange, lo, hi);
    if (++nacc_steps == merge_every) {
      merge_any<NSPEC, MOM>(tacc, srange, part, gm, nkey);
      nacc_steps = 0;
    } else {
      __syncthreads();
    }
  }
  if (nacc_steps) merge_any<NSPEC, MOM>(tacc, srange, part, gm, nkey);
}

using CwKernel = void (*)(const PassCArgs);

// The warp x pass's instance for these arguments.  The +-k_y pairing: one
// spectrum, moment form, line of sight along z, every transform holding
// lines of one ky only.
template <int N, int NSPEC, int MOM, int WPC>
CwKernel pick_c_w_at(const PassCArgs& a) {
  if constexpr (NSPEC == 1 && MOM > 0) {
    if (a.geom.los[0] == 0.f && a.geom.los[1] == 0.f && wc_np<N>(a.nfield) == 1 &&
        a.nfield % WF<N>::G == 0)
      return k_pass_c_w<N, NSPEC, MOM, WPC, true>;
  }
  return k_pass_c_w<N, NSPEC, MOM, WPC, false>;
}

// 16 warps per CTA only at Ng = 256 for one spectrum of the poles 0, 2, 4
// (the learned form's |mu| sub-bins, whose tile sums the CTA's warps share;
// larger transforms would spill); the host plans by the same rule
template <int N, int NSPEC, int MOM>
CwKernel pick_c_w(const PassCArgs& a) {
  if constexpr (N == 256 && NSPEC == 1 && MOM == 3) {
    if (a.wpc == kMaxWarpsC) return pick_c_w_at<N, NSPEC, MOM, kMaxWarpsC>(a);
  }
  return pick_c_w_at<N, NSPEC, MOM, 4>(a);
}

template <int N, int MOM>
CwKernel pick_c_w_ns(const PassCArgs& a) {
  switch (a.nspec) {
    case 1: return pick_c_w<N, 1, MOM>(a);
    case 2: return pick_c_w<N, 2, MOM>(a);
    default: return pick_c_w<N, 3, MOM>(a);
  }
}

template <int N>
CwKernel pick_c_w_mom(const PassCArgs& a) {
  switch (a.mom) {
    case 2: return pick_c_w_ns<N, 2>(a);
    case 3: return pick_c_w_ns<N, 3>(a);
    case 4: return pick_c_w_ns<N, 4>(a);
    default: return pick_c_w_ns<N, 0>(a);
  }
}

// Ng = 256 ... 1024 (nullptr otherwise); a.wpc: 4 or 16 warps per CTA
CwKernel pick_c_w_any(const PassCArgs& a) {
  switch (a.ng) {
    case 256: return pick_c_w_mom<256>(a);
    case 512: return pick_c_w_mom<512>(a);
    case 1024: return pick_c_w_mom<1024>(a);
    default: return nullptr;
  }
}

// ---- Ng = 2048: a pair of warps per line.  A line of 2048 complex values
// needs 64 values a lane in one warp; two warps share it instead, 64 lanes
// of 32 values, lane p holding x[p + 64 m]:
//
//   X[k1 + 32 k2] = sum_p W_64^(p k2) W_2048^(p k1) sum_m x[p + 64 m] W_32^(m k1)
//
//   1. a 32-point DFT over m in registers, then the twiddles W_2048^(p k1)
//      from the host table twl[k1 64 + p];
//   2. a transpose through the pair's shared memory S[k1][p] (rows of 66,
//      so that the reads below fall in distinct banks);
//   3. the 64-point DFTs over p by lane pairs: lane q takes k1 = q / 2 and
//      the even (q even) or odd (q odd) p, a 32-point DFT of them, the odd
//      half times W_64^k2 (table entries 2048 + k2), and the radix-2
//      butterfly with its neighbour through one shuffle per value: lane q
//      ends with X[k1 + 32 (k2 + 32 (q & 1))], k2 = 0..31.
//
// The pair synchronises on its own named barrier (id 1 + pair, 64
// threads), reached by both warps on the same pair-uniform path.
constexpr int kLine2k = 2112;  // line buffer of 2048 (+ 1/32 padding), and the 32 x 66 transpose
__device__ __forceinline__ void pair_sync(int pair) {
  __syncwarp();
  asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory");
}

__device__ __forceinline__ void wfft_pair2k(float2 (&v)[32], float2* S, const float2* __restrict__ twl,
                                            int p, int pair) {
  dft<32>(v);
#pragma unroll
  for (int k1 = 1; k1 < 32; k1++) v[k1] = cmul(v[k1], ldtw(&twl[k1 * 64 + p]));
  pair_sync(pair);  // S (a line buffer) is free: its last readers have passed
#pragma unroll
  for (int k1 = 0; k1 < 32; k1++) S[k1 * 66 + p] = v[k1];
  pair_sync(pair);
  const int k1 = p >> 1, h = p & 1;
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = S[k1 * 66 + 2 * i + h];
  pair_sync(pair);  // S is read; the caller writes the transformed line over it
  dft<32>(v);
  if (h) {
#pragma unroll
    for (int k2 = 1; k2 < 32; k2++) v[k2] = cmul(v[k2], ldtw(&twl[2048 + k2]));
  }
#pragma unroll
  for (int k2 = 0; k2 < 32; k2++) {
    const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, v[k2].x, 1),
                                 __shfl_xor_sync(0xffffffffu, v[k2].y, 1));
    // lane h = 0 holds E, its neighbour W O: X = E + W O; lane h = 1: E - W O
    v[k2] = h ? csub(o, v[k2]) : cadd(v[k2], o);
  }
}

// x transform + combine + window + binning at Ng = 2048: a work item of a
// pair is one (ky, kz); each field's line is loaded (lane p: x[p + 64 m]),
// transformed and stored into the pair's line buffer in the padded layout
// of bin_lines, which then bins the item with the pair's 64 threads.  The
// tile sums are merged every kMergeEvery steps, as k_pass_c_w does.
template <int NSPEC, int MOM>
__global__ void __launch_bounds__(512) k_pass_c_w2k(const __grid_constant__ PassCArgs a) {
  constexpr int N = 2048;
  extern __shared__ __align__(16) float2 wsm[];
  __shared__ int srange[2];
  const int pair = threadIdx.x >> 6, p = threadIdx.x & 63, npair = blockDim.x >> 6;
  const int nfield = a.nfield;
  float2* X = wsm + (size_t)pair * nfield * kLine2k;  // this pair's lines [field][kLine2k]
  float* tacc = reinterpret_cast<float*>(wsm + (size_t)npair * nfield * kLine2k);
  const ModeGeom& gm = a.geom;
  const int nacc = NSPEC * gm.npole;
  const int nkey = gm.nbin * gm.nmu;
  float2* part = a.partials + (size_t)blockIdx.x * nacc * nkey;
  for (int e = threadIdx.x; e < tile_accs<NSPEC, MOM>(gm) * nkey; e += blockDim.x) tacc[e] = 0.f;
  if (threadIdx.x == 0) {
    srange[0] = 0x7fffffff;
    srange[1] = -1;
  }
  __syncthreads();
  const int nitem = (N / 2 + 1) * N;  // (kz, ky)
  const int nstep = (nitem + (int)gridDim.x * npair - 1) / ((int)gridDim.x * npair);
  const int merge_every = max(1, kMergeEvery * 2 / npair);
  int nacc_steps = 0;
  for (int st = 0; st < nstep; st++) {
    const int item = (st * (int)gridDim.x + (int)blockIdx.x) * npair + pair;
    int lo = 0x7fffffff, hi = -1;
    if (item < nitem) {  // pair-uniform
      const int kz = item / N, ky = item - kz * N;
      for (int f = 0; f < nfield; f++) {
        const float2* src = a.in[f] + ((size_t)kz * N + ky) * N + p;
        float2 v[32];
#pragma unroll
        for (int m = 0; m < 32; m++) v[m] = __ldcs(src + 64 * m);
        float2* line = X + f * kLine2k;
        wfft_pair2k(v, line, a.twl, p, pair);
        const int k1 = p >> 1, h = p & 1;
#pragma unroll
        for (int k2 = 0; k2 < 32; k2++) {
          const int kx = k1 + 32 * (k2 + 32 * h);
          line[kx + (kx >> 5)] = v[k2];
        }
      }
      pair_sync(pair);  // every line of the item is stored
      bin_lines<NSPEC, true, MOM>(a, X, kLine2k, kz, ky, 1, tacc, lo, hi, p, 64);
    }
    note_range(srange, lo, hi);
    if (++nacc_steps == merge_every) {
      merge_any<NSPEC, MOM>(tacc, srange, part, gm, nkey);
      nacc_steps = 0;
    } else {
      __syncthreads();
    }
  }
  if (nacc_steps) merge_any<NSPEC, MOM>(tacc, srange, part, gm, nkey);
}

// y transform at Ng = 2048 by pairs of warps: pair c of the CTA transforms
// the line (x0 + c, kz) of A[x][kz][y]; the CTA stores B[kz][ky][x0 ..
// x0 + 4) through a shared [ky][5] tile, in runs of 4 x (whole 32-byte
// sectors).  The tile lies over the pairs' transpose areas, so that two
// CTAs fit an SM.
constexpr int kPairsB2k = 4;
__global__ void __launch_bounds__(64 * kPairsB2k) k_pass_b_w2k(const __grid_constant__ PassBArgs a) {
  constexpr int N = 2048, ngk = N / 2 + 1, TP = kPairsB2k + 1;
  constexpr int ntx = N / kPairsB2k;
  static_assert(N % kPairsB2k == 0, "whole tiles of x");
  extern __shared__ __align__(16) float2 wsm[];
  float2* T = wsm;  // [N][TP], over the pairs' transpose areas once they are done
  const int pair = threadIdx.x >> 6, p = threadIdx.x & 63;
  float2* S = wsm + (size_t)pair * kLine2k;  // the pair's transpose area
  const int kz = blockIdx.x / ntx, x0 = (blockIdx.x - kz * ntx) * kPairsB2k;
  const float2* src = a.in + ((size_t)(x0 + pair) * ngk + kz) * N + p;
  float2 v[32];
#pragma unroll
  for (int m = 0; m < 32; m++) v[m] = __ldcs(src + 64 * m);
  wfft_pair2k(v, S, a.twl, p, pair);
  __syncthreads();  // every pair's transform is done with its transpose area
  const int k1 = p >> 1, h = p & 1;
#pragma unroll
  for (int k2 = 0; k2 < 32; k2++) T[(k1 + 32 * (k2 + 32 * h)) * TP + pair] = v[k2];
  __syncthreads();
  float2* dst = a.out + (size_t)kz * N * N + x0;
  for (int e = threadIdx.x; e < N * kPairsB2k; e += blockDim.x) {
    const int ky = e / kPairsB2k, xl = e - ky * kPairsB2k;
    dst[(size_t)ky * N + xl] = T[ky * TP + xl];
  }
}

template <int NSPEC, int MOM>
void launch_c_w2k(const PassCArgs& a, cudaStream_t s) {
  const size_t smem = pass_c_w_smem(2048, a.nfield, a.nspec * pass_c_accs(a.geom.npole, a.mom),
                                    a.geom.nbin * a.geom.nmu, a.wpc);
  cudaFuncSetAttribute(k_pass_c_w2k<NSPEC, MOM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_pass_c_w2k<NSPEC, MOM><<<(unsigned)a.grid, 32 * a.wpc, smem, s>>>(a);
}

template <int MOM>
void launch_c_w2k_ns(const PassCArgs& a, cudaStream_t s) {
  switch (a.nspec) {
    case 1: launch_c_w2k<1, MOM>(a, s); break;
    case 2: launch_c_w2k<2, MOM>(a, s); break;
    default: launch_c_w2k<3, MOM>(a, s); break;
  }
}

}  // namespace

bool wfft_supported(int ng, int pass) {
  if (pass == 0) return ng == 256 || ng == 512 || ng == 1024 || ng == 2048;
  return ng == 256 || ng == 512 || ng == 1024;
}

void wfft_shape(int n, int* L, int* V) {
  switch (n) {
    case 2048: *L = 64; *V = 32; break;  // the pair-of-warps x pass (k_pass_c_w2k)
    case 128: *L = WShape<128>::L; *V = WShape<128>::V; break;
    case 256: *L = WShape<256>::L; *V = WShape<256>::V; break;
    case 512: *L = WShape<512>::L; *V = WShape<512>::V; break;
    case 1024: *L = WShape<1024>::L; *V = WShape<1024>::V; break;
    default: *L = *V = 0; break;
  }
}

size_t pass_c_w_smem(int ng, int nfield, int nacc, int nkey, int wpc) {
  if (ng == 2048) {  // wpc / 2 pairs, each with its nfield (<= 2) line buffers
    if (wpc < 2 || wpc > 16 || wpc % 2 || nfield > 2) return 0;
    return (size_t)(wpc / 2) * nfield * kLine2k * sizeof(float2) + (size_t)nacc * nkey * sizeof(float);
  }
  int wel = 0;
  switch (ng) {
    case 256: wel = wc_warp_elems<256>(nfield); break;
    case 512: wel = wc_warp_elems<512>(nfield); break;
    case 1024: wel = wc_warp_elems<1024>(nfield); break;
    default: return 0;
  }
  if (wpc != 4 && wpc != kMaxWarpsC) return 0;
  return (size_t)wpc * wel * sizeof(float2) + (size_t)nacc * nkey * sizeof(float);
}

int launch_pass_a_w(const PassAArgs& a, cudaStream_t s) {
#define PS_A_W(NG)                                                                              \
  {                                                                                             \
    constexpr int M = (NG) / 2, TY = warps_a<NG>() * WF<M>::G;                                  \
    const size_t smem = std::max((size_t)TY * (M + 1), (size_t)warps_a<NG>() * WF<M>::SWARP) * sizeof(float2); \
    cudaFuncSetAttribute(k_pass_a_w<NG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_pass_a_w<NG><<<(unsigned)((NG) * ((NG) / TY)), 32 * warps_a<NG>(), smem, s>>>(a);         \
    return 1;                                                                                   \
  }
  switch (a.ng) {
    case 256: PS_A_W(256)
    case 512: PS_A_W(512)
    case 1024: PS_A_W(1024)
    case 2048: PS_A_W(2048)
    default: return 0;
  }
#undef PS_A_W
}

int launch_pass_b_w(const PassBArgs& a, cudaStream_t s) {
#define PS_B_W(N)                                                                               \
  {                                                                                             \
    constexpr int TX = warps_b<N>() * WF<N>::G;                                                 \
    const size_t smem = std::max((size_t)(N) * (TX + 1), (size_t)warps_b<N>() * WF<N>::SWARP) * sizeof(float2); \
    cudaFuncSetAttribute(k_pass_b_w<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_pass_b_w<N><<<(unsigned)(((N) / 2 + 1) * ((N) / TX)), 32 * warps_b<N>(), smem, s>>>(a);  \
    return 1;                                                                                   \
  }
  switch (a.ng) {
    case 256: PS_B_W(256)
    case 512: PS_B_W(512)
    case 1024: PS_B_W(1024)
    case 2048: {
      constexpr int N = 2048;
      const size_t smem = std::max((size_t)N * (kPairsB2k + 1), (size_t)kPairsB2k * kLine2k) * sizeof(float2);
      cudaFuncSetAttribute(k_pass_b_w2k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_pass_b_w2k<<<(unsigned)((N / 2 + 1) * (N / kPairsB2k)), 64 * kPairsB2k, smem,
                     s>>>(a);
      return 1;
    }
    default: return 0;
  }
#undef PS_B_W
}

int launch_pass_c_ws(const PassCArgs& a, cudaStream_t s) {
  if (a.nfield != 1 || !a.store) return 0;
#define PS_C_WS(N)                                                                                \
  {                                                                                               \
    constexpr int W = kStoreKz / WF<N>::G;                                                        \
    const size_t smem = std::max((size_t)(N) * (kStoreKz + 1), (size_t)W * WF<N>::SWARP) * sizeof(float2); \
    cudaFuncSetAttribute(k_pass_c_ws<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    k_pass_c_ws<N><<<(unsigned)((N) * (((N) / 2 + 1 + kStoreKz - 1) / kStoreKz)), 32 * W, smem, s>>>(a); \
    return 1;                                                                                     \
  }
  switch (a.ng) {
    case 256: PS_C_WS(256)
    case 512: PS_C_WS(512)
    case 1024: PS_C_WS(1024)
    default: return 0;
  }
#undef PS_C_WS
}

int launch_pass_c_w(const PassCArgs& a, cudaStream_t s) {
  if (a.ng == 2048) {
    switch (a.mom) {
      case 2: launch_c_w2k_ns<2>(a, s); break;
      case 3: launch_c_w2k_ns<3>(a, s); break;
      case 4: launch_c_w2k_ns<4>(a, s); break;
      default: launch_c_w2k_ns<0>(a, s); break;
    }
    return 1;
  }
  const CwKernel k = pick_c_w_any(a);
  if (!k) return 0;
  const int wpc = (a.wpc == kMaxWarpsC) ? kMaxWarpsC : 4;
  const size_t smem = pass_c_w_smem(a.ng, a.nfield, a.nspec * pass_c_accs(a.geom.npole, a.mom),
                                    a.geom.nbin * a.geom.nmu, wpc);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k<<<(unsigned)a.grid, 32 * wpc, smem, s>>>(a);
  return 1;
}

int pass_c_w_per_sm(const PassCArgs& a) {
  if (a.ng == 2048) return 0;
  const CwKernel k = pick_c_w_any(a);
  if (!k) return 0;
  const int wpc = (a.wpc == kMaxWarpsC) ? kMaxWarpsC : 4;
  const size_t smem = pass_c_w_smem(a.ng, a.nfield, a.nspec * pass_c_accs(a.geom.npole, a.mom),
                                    a.geom.nbin * a.geom.nmu, wpc);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 32 * wpc, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

}  // namespace ps
