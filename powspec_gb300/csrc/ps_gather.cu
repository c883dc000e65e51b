// ps_gather.cu -- deterministic particle assignment by tiles: every mesh cell
// is written exactly once, as FP32 (minus the mean cell value), with no
// global atomics and no zeroing pass.
//
// Reference: ngp/cic/tsc/pcs (src/genr_mesh.c:50-412), interlace shift
// (src/genr_mesh.c:590-602, :815-833), sim-box bound check
// (src/genr_mesh.c:523-531).
//
//  classify  per particle: the stencil base node and fraction on the plain
//            and the half-cell-shifted grid; its 16^3 tile and which of the
//            neighbouring tiles its stencils reach (27 classes); histogram
//            of the (tile, class) keys; weight sums (per-block partials).
//  scan      exclusive prefix sum of the key counts.
//  scatter   compact records in key order.
//  gather    one CTA per tile reads the 125 (neighbour tile, class) buckets
//            that can reach it, adds every stencil node that falls in the
//            tile into int64 fixed-point accumulators in shared memory
//            (integer sums: independent of the order), then writes the tile.
//
// Grid coordinates: x = pos * Ng / L is evaluated in double-float FP32
// arithmetic (error ~1e-7 cell); only when the fraction lies within 4e-6 of
// a decision point of the reference (0, 1/2, 1) is the reference's exact
// FP64 sequence (pos - bmin) * Ng / L used instead, so cell indices and
// branches are the reference's while FP64 work stays rare.
#include <cstddef>
#include <type_traits>

#include "ps_internal.h"

namespace ps {
namespace {

constexpr int kGatherThreads = 512;  // 16 warps; 3 CTAs per SM fit (registers, shared memory)
constexpr int kMeshPad = 8;  // words between the two meshes' accumulators (bank offset)
constexpr float kEdge = 4e-6f;

// wsum[0..1] = sums of the per-block partials (k_classify: the signed sum as
// an FP32 pair, the sum of |w| in FP32): thread t adds blocks t, t + 256,
// ... in order, then a fixed tree (same order every run); FP64 once at the
// end (this GPU's FP64 pipe is narrow).  *moff = the mean cell value in
// fixed point, W * scale rounded (0 with nomean), computed once here for
// the gather kernels.
constexpr int kWsumThreads = 256;
__global__ void __launch_bounds__(kWsumThreads) k_wsum(const float4* __restrict__ wpart, int nblocks,
                                                       double* wsum, long long* moff, double scale,
                                                       int nomean) {
  __shared__ float sh[kWsumThreads / 32][3];
  float h = 0.f, l = 0.f, ab = 0.f;
  for (int b = threadIdx.x; b < nblocks; b += kWsumThreads) {
    const float4 v = wpart[b];
    df_add(h, l, v.x, v.y);
    ab += v.z;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, h, o), ol = __shfl_down_sync(0xffffffffu, l, o);
    ab += __shfl_down_sync(0xffffffffu, ab, o);
    df_add(h, l, oh, ol);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[threadIdx.x >> 5][0] = h;
    sh[threadIdx.x >> 5][1] = l;
    sh[threadIdx.x >> 5][2] = ab;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float th = 0.f, tl = 0.f, ta = 0.f;
    for (int k = 0; k < kWsumThreads / 32; k++) {
      df_add(th, tl, sh[k][0], sh[k][1]);
      ta += sh[k][2];
    }
    const double w = (double)th + (double)tl;
    wsum[0] = w;
    wsum[1] = (double)ta;
    *moff = nomean ? 0 : __double2ll_rn(w * scale);
  }
}

// Stencil base node and parameter of one axis (see node_weights).
struct Axis {
  int base;
  float par;
};

// Record of one particle in key order (48 bytes).
struct Rec {
  short base[2][3];  // [mesh][axis]
  float par[2][3];
  float wf;          // weight * 2^32 (FP32, for the node products)
  long long q;       // llrint(weight * 2^32): the exact NGP node value
};
static_assert(sizeof(Rec) == 48, "record layout");

// Record of a TSC/PCS particle for the gather (112 bytes): the 1-D node
// weights per mesh and axis, with weight * 2^32 folded into the x weights.
struct __align__(16) WRec {
  float w[2][3][4];   // [mesh][axis][node]
  short base[2][4];   // [mesh][axis]; [mesh][3]: node value bound (k_scatter)
};
static_assert(sizeof(WRec) == 112, "weighted record layout");
static_assert(offsetof(WRec, base) == 96 && sizeof(WRec::w[0]) == 48,
              "region gather reads w[m] at m * 48 and base[m] at 96 + m * 8");
constexpr size_t kRecBytes = 112;  // room for either record kind

// round-to-nearest-even of v as int64 from 32-bit conversions only (the
// direct FP32 -> int64 conversion runs several times slower): v = hi * 2^32
// + r with hi = trunc(v / 2^32) and r exact (an FMA of multiples of ulp(v)),
// |r| < 2^32.  Valid for |v| < 2^63.
__device__ __forceinline__ long long round_fix(float v) {
  const int hi = __float2int_rz(v * 2.3283064365386963e-10f);
  const float r = fmaf((float)(-hi), 4294967296.f, v);
  const long long lo = (long long)__float2uint_rn(fabsf(r));
  const long long h = (long long)hi * 4294967296ll;
  return (r < 0.f) ? h - lo : h + lo;
}
// |v| < 2^31: one 32-bit conversion
__device__ __forceinline__ long long round_small(float v) { return (long long)__float2int_rn(v); }

// Offset of the first stencil node from the base and stencil width.
__host__ __device__ inline int first_off(int assign) { return assign >= 2 ? -1 : 0; }
__host__ __device__ inline int width(int assign) { return assign + 1; }

// Exact reference grid coordinate (FP64, correctly rounded operations).
// Shifted grid: its lower edge bmin = -(L / 2) / Ng and bmax = bmin + L,
// computed on the host (loop-invariant FP64 divisions would otherwise be
// hoisted into every thread's preamble).
__device__ __forceinline__ void exact_coord(double pos, double L, int ng, bool shift, double bmin,
                                            double bmax, int& i0, double& d) {
  if (shift) {
    if (pos >= bmax) pos = __dsub_rn(pos, L);
  } else {
    bmin = 0.0;
  }
  const double x = __ddiv_rn(__dmul_rn(__dsub_rn(pos, bmin), (double)ng), L);
  i0 = (int)x;
  d = __dsub_rn(x, (double)i0);
  if (i0 >= ng) i0 -= ng;
}

// Base node and parameter from (cell, fraction).  NGP: nearest node (rounds
// up at d >= 1/2, src/genr_mesh.c:64-66).  CIC, PCS: the cell, d.  TSC: the
// nearest node c and the offset u = d or d - 1 from it (src/genr_mesh.c:157-172).
__device__ __forceinline__ Axis make_axis(int assign, int i0, double d, int ng) {
  Axis a;
  if (assign == 0 || assign == 2) {
    const bool up = d >= 0.5;
    a.base = up ? ((i0 == ng - 1) ? 0 : i0 + 1) : i0;
    a.par = up ? (float)__dsub_rn(d, 1.0) : (float)d;
  } else {
    a.base = i0;
    a.par = (float)d;
  }
  return a;
}

// The same from a float fraction (the fast path): d - 1 is exact for d in
// [1/2, 1), so the parameter equals the FP64 form's.
__device__ __forceinline__ Axis make_axis(int assign, int i0, float d, int ng) {
  Axis a;
  if (assign == 0 || assign == 2) {
    const bool up = d >= 0.5f;
    a.base = up ? ((i0 == ng - 1) ? 0 : i0 + 1) : i0;
    a.par = up ? d - 1.f : d;
  } else {
    a.base = i0;
    a.par = d;
  }
  return a;
}

__device__ __forceinline__ bool near_edge(float d) {
  return d < kEdge || d > 1.f - kEdge || fabsf(d - 0.5f) < kEdge;
}

// The plain grid's axis for one coordinate; i, d: the double-float cell and
// fraction it started from.  pos_hi + pos_lo = pos; s_hi + s_lo = Ng / L.
// pos() gives the FP64 coordinate, asked for only on the exact path (FP64
// conversions run on this GPU's narrow FP64 pipe).
template <class Pos>
__device__ __forceinline__ Axis plain_axis(int assign, Pos pos, float pos_hi, float pos_lo,
                                           float s_hi, float s_lo, double L, int ng, int& i,
                                           float& d) {
  // x = pos * s in double-float: p + t
  const float p = pos_hi * s_hi;
  const float e = fmaf(pos_hi, s_hi, -p);
  const float t = e + fmaf(pos_hi, s_lo, pos_lo * s_hi);
  i = (int)floorf(p);
  d = (p - (float)i) + t;
  if (d < 0.f) { i -= 1; d += 1.f; }
  if (d >= 1.f) { i += 1; d -= 1.f; }
  if (near_edge(d) || i < 0 || i >= ng) {
    int i0;
    double dd;
    exact_coord(pos(), L, ng, false, 0.0, 0.0, i0, dd);
    return make_axis(assign, i0, dd, ng);
  }
  return make_axis(assign, i, d, ng);
}

// Both grids' axis for one coordinate.
template <class Pos>
__device__ __forceinline__ void axis_pair(int assign, Pos pos, float pos_hi, float pos_lo,
                                          float s_hi, float s_lo, double L, double bmin,
                                          double bmax, int ng, bool il, Axis& a0, Axis& a1) {
  int i;
  float d;
  a0 = plain_axis(assign, pos, pos_hi, pos_lo, s_hi, s_lo, L, ng, i, d);
  if (!il) {
    a1 = a0;
    return;
  }
  // shifted grid: x' = x + 1/2, wrapped (the reference moves pos by -L)
  int i1 = i;
  float d1 = d + 0.5f;
  if (d1 >= 1.f) { i1 += 1; d1 -= 1.f; }
  if (i1 >= ng) i1 -= ng;
  if (near_edge(d1) || near_edge(d) || i1 < 0 || i1 >= ng) {
    int i0;
    double dd;
    exact_coord(pos(), L, ng, true, bmin, bmax, i0, dd);
    a1 = make_axis(assign, i0, dd, ng);
  } else {
    a1 = make_axis(assign, i1, d1, ng);
  }
}

// 1-D weights of the stencil nodes base + first_off + k.  The outermost
// weight is 1 minus the others, so each axis's weights sum to 1 within one
// FP32 rounding.
template <int S>
__device__ __forceinline__ void node_weights(float par, float (&w)[4]) {
  if (S == 1) {
    w[0] = 1.f;
  } else if (S == 2) {
    w[0] = 1.f - par;
    w[1] = par;
  } else if (S == 3) {
    const float a = 0.5f - par;
    w[0] = 0.5f * a * a;
    w[1] = 0.75f - par * par;
    w[2] = 1.f - w[0] - w[1];
  } else {
    const float f = par, f2 = f * f, f3 = f2 * f, s = 1.f / 6.f;
    w[3] = f3 * s;
    w[2] = (1.f + 3.f * (f + f2 - f3)) * s;
    w[1] = (4.f - 6.f * f2 + 3.f * f3) * s;
    w[0] = 1.f - w[1] - w[2] - w[3];
  }
}

// 2^k as a float (0 below the normal range, infinity above it).
__device__ __forceinline__ float exp2i(int k) {
  return k < -126 ? 0.f : (k > 127 ? __int_as_float(0x7f800000) : __int_as_float((k + 127) << 23));
}

// round-to-nearest-even of m 2^sh as an integer (m >= 0, m < 2^53, sh <=
// 10), integer operations only; negated if neg.
__device__ __forceinline__ long long round_shift(long long m, int sh, bool neg) {
  long long r;
  if (sh >= 0) {
    r = m << min(sh, 10);
  } else if (sh < -53) {
    r = 0;  // m 2^sh < 1/2
  } else {
    const int t = -sh;
    r = m >> t;
    const long long rem = m & ((1LL << t) - 1), half = 1LL << (t - 1);
    if (rem > half || (rem == half && (r & 1))) r++;
  }
  return neg ? -r : r;
}

// llrint(w 2^32) from the bits of the double w (|w| < 2^31, which the
// total-weight limit checked on the host implies): equals
// __double2ll_rn(w * 4294967296.0), without FP64 arithmetic.
__device__ __forceinline__ long long fix_from_bits(long long b) {
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0;  // zero or subnormal: |w| 2^32 < 2^-990
  return round_shift((b & 0xfffffffffffffLL) | 0x10000000000000LL, e - 1043, b < 0);
}

// Non-negative double (bit pattern b) as hi + lo floats with integer
// operations only (FP64 arithmetic is slow on this GPU): hi = the top 24
// significand bits (rounded), lo = the rest rounded to float.  The error of
// hi + lo is below 2^-48 relative for values above 2^-74 (smaller ones lose
// lo, an absolute error below 2^-98), far inside the tolerance that sends a
// coordinate to the exact FP64 path.
__device__ __forceinline__ void split_pos(long long b, float& hi, float& lo) {
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) {  // zero (subnormals count as 0)
    hi = lo = 0.f;
    return;
  }
  const long long m = (b & 0xfffffffffffffLL) | 0x10000000000000LL;  // 53 bits
  const int hm = (int)((m + (1LL << 28)) >> 29);                     // <= 2^24
  const int lm = (int)(m - ((long long)hm << 29));                   // |lm| <= 2^28
  hi = __int2float_rn(hm) * exp2i(e - 1046);
  lo = __int2float_rn(lm) * exp2i(e - 1075);
}

struct Particle {
  double pos[3];     // AoS input: the coordinates as given (exact path only)
  float hi[3], lo[3];
  float wh, wl;      // weight = wh + wl (FP64 input: to about 2^-48 relative)
  long long wbits;   // the weight as FP64 bits (NGP node value)
  float wf;          // weight as float
  bool ok;           // inside [0, L) on every axis
  bool aos;          // FP64 input (pos holds the coordinates)
  // the FP64 coordinate of axis a, for the exact path
  __device__ __forceinline__ double exact(int a) const { return aos ? pos[a] : (double)hi[a]; }
};

__device__ __forceinline__ Particle load_particle(const Particles& p, const GatherArgs& g, size_t i) {
  Particle q;
  q.ok = true;
  q.aos = p.aos != nullptr;
  if (p.aos) {
    const double4_32a r = reinterpret_cast<const double4_32a*>(p.aos)[i];  // 32-byte aligned (checked)
    const double v[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      q.pos[a] = v[a];
      long long b = __double_as_longlong(v[a]);
      if (b == (long long)0x8000000000000000ull) b = 0;  // -0.0 >= 0 holds
      // 0 <= pos < L on the bit patterns (ordered as the values for pos >= 0;
      // negatives have the sign bit, NaN sorts above any finite L)
      if (b < 0 || b >= g.box_bits[a]) q.ok = false;
      split_pos(b, q.hi[a], q.lo[a]);
    }
    const long long wb = __double_as_longlong(r.w);
    float wh, wl;
    split_pos(wb & 0x7fffffffffffffffLL, wh, wl);
    if (((wb >> 52) & 0x7ff) == 0x7ff) wh = __int_as_float(0x7fc00000);  // inf, NaN: NaN sums
    q.wh = (wb < 0) ? -wh : wh;
    q.wl = (wb < 0) ? -wl : wl;
    q.wbits = wb;
    q.wf = (wb < 0) ? -(wh + wl) : (wh + wl);
  } else {
    const float v[3] = {p.x[i], p.y[i], p.z[i]};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      q.hi[a] = v[a];
      q.lo[a] = 0.f;
      q.pos[a] = 0.0;  // not used: the exact path converts hi
      if (!(v[a] >= 0.f && v[a] < g.box_f[a])) q.ok = false;  // box_f: smallest float >= L
    }
    q.wf = p.w ? p.w[i] : 1.f;
    q.wh = q.wf;
    q.wl = 0.f;
    // the float's value as FP64 bits (zero for subnormals, whose node value
    // rounds to 0 anyway)
    const unsigned fb = __float_as_uint(q.wf), ef = (fb >> 23) & 0xff;
    q.wbits = (long long)((unsigned long long)(fb >> 31) << 63) |
              (ef ? ((long long)(ef + 1023 - 127) << 52) | ((long long)(fb & 0x7fffff) << 29) : 0);
  }
  return q;
}

// Tile of a base node: a shift when the tile edge is a power of two (the
// usual 16), else an integer division.
__device__ __forceinline__ int tile_of(int base, const GatherArgs& g) {
  return g.tshift >= 0 ? (base >> g.tshift) : base / g.T;
}

// Record and key of one particle; returns false if it lies outside the box.
__device__ __forceinline__ bool make_record(const Particle& q, const GatherArgs& g, Rec& r,
                                            unsigned& key) {
  const int ng = g.ng;
  int tile[3], cls[3];
  if (!q.ok) return false;
  for (int a = 0; a < 3; a++) {
    Axis a0, a1;
    axis_pair(g.assign, [&] { return q.exact(a); }, q.hi[a], q.lo[a], g.s_hi[a], g.s_lo[a],
              g.box[a], g.bmin[a], g.bmax[a], ng, g.interlace != 0, a0, a1);
    r.base[0][a] = (short)a0.base;
    r.base[1][a] = (short)a1.base;
    r.par[0][a] = a0.par;
    r.par[1][a] = a1.par;
    // reach of both stencils relative to the plain base's tile
    int diff = a1.base - a0.base;
    if (diff > ng / 2) diff -= ng;
    if (diff < -ng / 2) diff += ng;
    const int t = tile_of(a0.base, g);
    const int rel = a0.base - t * g.T;
    const int of = first_off(g.assign), S = width(g.assign);
    const int lo_r = rel + of + (g.interlace ? min(0, diff) : 0);
    const int hi_r = rel + of + S - 1 + (g.interlace ? max(0, diff) : 0);
    tile[a] = t;
    cls[a] = (lo_r < 0) ? 1 : ((hi_r >= g.T) ? 2 : 0);
  }
  r.wf = q.wf * kFixScale;
  r.q = (g.assign == 0) ? fix_from_bits(q.wbits) : 0;  // NGP node value only
  const unsigned t = ((unsigned)tile[0] * g.nt + tile[1]) * g.nt + tile[2];
  key = t * 27u + (unsigned)(cls[0] + 3 * cls[1] + 9 * cls[2]);
  return true;
}

// Key of a particle for the region gather, which takes every record of its
// home tile (the tile of the plain grid's base node) from one bucket: the
// tile's index, from the plain grid alone.  The same tile as make_record's.
__device__ __forceinline__ bool region_key(const Particle& q, const GatherArgs& g, unsigned& key) {
  if (!q.ok) return false;
  int tile[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    int i;
    float d;
    const Axis a0 = plain_axis(g.assign, [&] { return q.exact(a); }, q.hi[a], q.lo[a],
                               g.s_hi[a], g.s_lo[a], g.box[a], g.ng, i, d);
    tile[a] = tile_of(a0.base, g);
  }
  key = ((unsigned)tile[0] * g.nt + tile[1]) * g.nt + tile[2];
  return true;
}

__global__ void __launch_bounds__(256) k_classify(const __grid_constant__ GatherArgs g, Particles p) {
  // weight sums: the signed one as an FP32 pair (the per-particle FP64 add
  // would load this GPU's narrow FP64 pipe), |w| in FP32 (only compared
  // against limits)
  float ws_hi = 0.f, ws_lo = 0.f, waf = 0.f;
  int bad = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n;
       i += (size_t)gridDim.x * blockDim.x) {
    const Particle q = load_particle(p, g, i);
    unsigned key;
    bool ok;
    if (g.region) {
      ok = region_key(q, g, key);
    } else {
      Rec r;
      ok = make_record(q, g, r, key);
    }
    if (!ok) {
      bad = 1;
      g.rank[i] = 0xffffffffu;
      continue;
    }
    df_add(ws_hi, ws_lo, q.wh, q.wl);
    waf += fabsf(q.wh + q.wl);
    // Rank within the key, aggregated over the lanes of this warp that share
    // it (catalogues are often spatially ordered: whole warps hit one key).
    const unsigned peers = __match_any_sync(__activemask(), key);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&g.hist[key], (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    g.rank[i] = base + __popc(peers & ((1u << lane) - 1u));
  }
  // block partials, still as FP32 pairs (FP64 once per block)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, ws_hi, o);
    const float ol = __shfl_down_sync(0xffffffffu, ws_lo, o);
    waf += __shfl_down_sync(0xffffffffu, waf, o);
    df_add(ws_hi, ws_lo, oh, ol);
  }
  __shared__ float sws[8][2], swa[8];
  if ((threadIdx.x & 31) == 0) {
    sws[threadIdx.x >> 5][0] = ws_hi;
    sws[threadIdx.x >> 5][1] = ws_lo;
    swa[threadIdx.x >> 5] = waf;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float th = 0.f, tl = 0.f, ta = 0.f;
    for (int k = 0; k < 8; k++) {
      df_add(th, tl, sws[k][0], sws[k][1]);
      ta += swa[k];
    }
    reinterpret_cast<float4*>(g.wpart)[blockIdx.x] = make_float4(th, tl, ta, 0.f);
  }
  if (bad) atomicOr(g.err, 1);
}

// Region geometry of the region gather (kernels below): R cells per axis
// cover every node a home tile's records reach, local cells [of - 1, T + of
// + S - 1]; shared-memory z rows are padded to RZ words.
constexpr int kRegT = 16;
constexpr int reg_row(int r) { return (r % 16 == 4 || r % 16 == 12) ? r : reg_row(r + 1); }
template <int S>
struct RegGeom {
  static constexpr int R = kRegT + S + 1;  // region edge (cells)
  static constexpr int RG = (R + 1) & ~1;  // z row of a region in memory (even: 16-byte pairs)
  static constexpr int RP = R * R * RG;    // words per mesh in memory
  // Shared-memory z rows padded to RZ = 4 or 12 (mod 16) words: the 4 x 4
  // (y, z) nodes of a mesh then fall in 16 distinct 8-byte bank pairs.
  static constexpr int RZ = reg_row(R);
  static constexpr int SM = (R * R * RZ + 1) & ~1;  // shared words per mesh
};

// Gather record of a TSC/PCS particle: the node weights of both meshes per
// axis (weight * 2^32 folded into x), the region word offset and the node
// value bound.
__device__ __forceinline__ WRec weighted_record(const Rec& r, const GatherArgs& g) {
  WRec v;
#pragma unroll
  for (int m = 0; m < 2; m++) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float w[4];
      if (g.assign == 2) {
        node_weights<3>(r.par[m][a], w);
        w[3] = 0.f;
      } else {
        node_weights<4>(r.par[m][a], w);
      }
#pragma unroll
      for (int k = 0; k < 4; k++) v.w[m][a][k] = (a == 0) ? w[k] * r.wf : w[k];
      v.base[m][a] = r.base[m][a];
    }
    if (g.region) {
      // Region word offset of the first node: region index = base -
      // home tile origin + 1 per axis, wrapped into [0, T + 1] (the
      // shifted grid's base may sit one cell outside the home tile,
      // across the periodic edge).
      int l[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        l[a] = (int)r.base[m][a] - tile_of(r.base[0][a], g) * g.T + 1;
        l[a] += (l[a] < 0) ? g.ng : 0;
        l[a] -= (l[a] > g.T + 1) ? g.ng : 0;
        if (l[a] < 0 || l[a] > g.T + 1) {  // the grids' bases differ by at most a cell
          atomicOr(g.err, 2);
          l[a] = 0;
        }
      }
      const int R = (g.assign == 2) ? RegGeom<3>::R : RegGeom<4>::R;
      const int RZ = (g.assign == 2) ? RegGeom<3>::RZ : RegGeom<4>::RZ;
      v.base[m][0] = (short)((l[0] * R + l[1]) * RZ + l[2]);
      v.base[m][1] = v.base[m][2] = 0;
    }
    // bound of every node value of this mesh: product of the axis maxima
    float bound = 1.f;
#pragma unroll
    for (int a = 0; a < 3; a++)
      bound *= fmaxf(fmaxf(fabsf(v.w[m][a][0]), fabsf(v.w[m][a][1])),
                     fmaxf(fabsf(v.w[m][a][2]), fabsf(v.w[m][a][3])));
    // [mesh][3]: bit 8 set when every node value is below 2^31 (one
    // 32-bit conversion); bits 0-7 the least e >= 0 with bound < 2^e
    const int e = max(0, ((__float_as_int(bound) >> 23) & 0xff) - 126);
    v.base[m][3] = (short)((bound < 0.999f * 2147483648.f ? 0x100 : 0) | min(e, 255));
    if (g.region) v.base[m][1] = v.base[m][3];  // (offset, flags): one 32-bit read
  }
  return v;
}

// Records to their slots.  TSC/PCS: a warp's 32 records are staged in shared
// memory and written 4 at a time by 28 lanes, 7 x 16 bytes each, so that a
// record's 112 bytes leave as one contiguous run (and a run of consecutive
// slots, as spatially ordered catalogues give, as whole sectors).
constexpr int kScatterWarps = 8;
__global__ void __launch_bounds__(32 * kScatterWarps, 4) k_scatter(const __grid_constant__ GatherArgs g,
                                                                   Particles p) {
  __shared__ __align__(16) WRec stage[kScatterWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t step = (size_t)gridDim.x * kScatterWarps * 32;
  for (size_t base = ((size_t)blockIdx.x * kScatterWarps + w) * 32; base < p.n; base += step) {
    const size_t i = base + lane;
    const unsigned rk = (i < p.n) ? g.rank[i] : 0xffffffffu;
    const bool valid = rk != 0xffffffffu;
    unsigned slot = 0;
    if (valid) {
      const Particle q = load_particle(p, g, i);
      Rec r;
      unsigned key;
      make_record(q, g, r, key);
      if (g.region) key /= 27u;  // one bucket per home tile (region_key)
      slot = g.hist[key] + rk;
      if (g.assign >= 2)
        stage[w][lane] = weighted_record(r, g);
      else
        reinterpret_cast<Rec*>(g.rec)[slot] = r;
    }
    if (g.assign >= 2) {
      __syncwarp();
      const int jr = lane / 7, part = lane - 7 * jr;
#pragma unroll
      for (int it = 0; it < 8; it++) {
        const int j = (it * 4 + jr) & 31;  // lanes 28-31 idle
        const unsigned sj = __shfl_sync(0xffffffffu, slot, j);
        const bool vj = __shfl_sync(0xffffffffu, valid ? 1 : 0, j) != 0;
        if (lane < 28 && vj)
          reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(g.rec) + (size_t)sj * sizeof(WRec))[part] =
              reinterpret_cast<const uint4*>(&stage[w][j])[part];
      }
      __syncwarp();  // the stage is rewritten next step
    }
  }
}

// ---- exclusive scan of nkeys counts in place (hist[nkeys] = total)
constexpr int kScanPer = 16;  // elements per thread
constexpr int kScanBlock = 256 * kScanPer;

__device__ __forceinline__ unsigned block_exclusive(unsigned v, unsigned* sh, unsigned& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned s = (lane < 8) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < 8) sh[lane] = s;
  }
  __syncthreads();
  const unsigned before = (wid ? sh[wid - 1] : 0) + x - v;
  total = sh[7];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(256) k_scan_reduce(const unsigned* hist, size_t n, unsigned* bsum) {
  __shared__ unsigned sh[8];
  const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanPer;
  unsigned s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; k++)
    if (base + k < n) s += hist[base + k];
  unsigned total;
  block_exclusive(s, sh, total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(256) k_scan_blocks(unsigned* bsum, int nb) {
  __shared__ unsigned sh[8];
  unsigned carry = 0;
  for (int c = 0; c < nb; c += 256) {
    const int i = c + threadIdx.x;
    const unsigned v = (i < nb) ? bsum[i] : 0;
    unsigned total;
    const unsigned ex = block_exclusive(v, sh, total);
    if (i < nb) bsum[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) bsum[nb] = carry;  // number of classified particles
}

__global__ void __launch_bounds__(256) k_scan_apply(unsigned* hist, size_t n, const unsigned* bsum,
                                                    int nb) {
  __shared__ unsigned sh[8];
  const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanPer;
  unsigned v[kScanPer];
  unsigned s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    v[k] = (base + k < n) ? hist[base + k] : 0;
    s += v[k];
  }
  unsigned total;
  unsigned run = block_exclusive(s, sh, total) + bsum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    if (base + k < n) hist[base + k] = run;
    run += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) hist[n] = bsum[nb];
}

// ---- gather: one CTA per tile.  TT: compile-time tile edge (0: g.T).
template <int S, bool INT64, int TT>
__global__ void __launch_bounds__(kGatherThreads, 3) k_gather(const __grid_constant__ GatherArgs g) {
  extern __shared__ __align__(16) unsigned long long acc[];  // [nmesh][T^3 + kMeshPad]
  __shared__ unsigned bstart[128];
  __shared__ unsigned boff[125];
  __shared__ unsigned rowmask[2][8];  // T = 16: touched (x, y) rows per mesh
  __shared__ float bound_sum[2];
  const int T = TT ? TT : g.T;
  const int nt = g.nt, ng = g.ng;
  const int T3 = T * T * T;
  const int nmesh = g.interlace ? 2 : 1;
  const int tx = blockIdx.z, ty = blockIdx.y, tz = blockIdx.x;  // grid (nt, nt, nt)
  const int org[3] = {tx * T, ty * T, tz * T};
  // the 125 buckets that can reach this tile (loads issued before the
  // accumulators are zeroed, so their latency overlaps the stores)
  unsigned h0 = 0, hc = 0;
  if (threadIdx.x < 125) {
    int k = threadIdx.x;
    int off[3], c[3];
    // 5 choices per axis: neighbour -1 (class 2), own (classes 0, 1, 2), +1 (class 1)
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int ch = k % 5;
      k /= 5;
      off[a] = (ch == 0) ? -1 : ((ch == 4) ? 1 : 0);
      c[a] = (ch == 0) ? 2 : ((ch == 4) ? 1 : ch - 1);
    }
    auto wrap = [nt](int v) { return v < 0 ? v + nt : (v >= nt ? v - nt : v); };
    const int nx = wrap(tx + off[0]), ny = wrap(ty + off[1]), nz = wrap(tz + off[2]);
    const unsigned key =
        ((unsigned)((nx * nt + ny) * nt + nz)) * 27u + (unsigned)(c[0] + 3 * c[1] + 9 * c[2]);
    h0 = g.hist[key];
    hc = g.hist[key + 1];
  }
  {
    // zeroed while the bucket loads are in flight
    const int nacc = nmesh * (T3 + kMeshPad);
    if constexpr (TT % 4 == 0 && TT != 0) {
      ulonglong2* a2 = reinterpret_cast<ulonglong2*>(acc);
      for (int e = threadIdx.x; e < nacc / 2; e += blockDim.x) a2[e] = make_ulonglong2(0ull, 0ull);
    } else {
      for (int e = threadIdx.x; e < nacc; e += blockDim.x) acc[e] = 0ull;
    }
  }
  if (threadIdx.x < 128) {
    if (threadIdx.x < 125) boff[threadIdx.x] = h0;
    bstart[threadIdx.x] = hc - h0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // exclusive scan of 128 entries, 4 per lane
    const int l = threadIdx.x;
    const unsigned v0 = bstart[4 * l], v1 = bstart[4 * l + 1], v2 = bstart[4 * l + 2],
                   v3 = bstart[4 * l + 3];
    const unsigned s = v0 + v1 + v2 + v3;
    unsigned x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (l >= o) x += y;
    }
    const unsigned ex = x - s;
    __syncwarp();
    bstart[4 * l] = ex;
    bstart[4 * l + 1] = ex + v0;
    bstart[4 * l + 2] = ex + v0 + v1;
    bstart[4 * l + 3] = ex + v0 + v1 + v2;
  }
  __syncthreads();
  const unsigned total = bstart[125];
  const Rec* rec = reinterpret_cast<const Rec*>(g.rec);
  const int of = first_off(g.assign);
  constexpr bool kSwz = (S >= 3 && TT == 16);
  // Local index of the first stencil node, s = base + of - org taken in
  // [-(S-1), ng-(S-1)): then s + k lies in [0, T) exactly for the nodes
  // inside the tile (T <= ng/2 < ng - S + 1).
  auto rel = [&](int base, int a) {
    int s = base + of - org[a];
    s += (s < 0) ? ng : 0;
    s -= (s >= ng - (S - 1)) ? ng : 0;
    return s;
  };
  // Sparse tiles: one pass over all records (below), which also flags the
  // (x, y) rows of 16 z cells that it touches; the write-out converts only
  // those and writes -mean elsewhere.  Dense tiles: every row is flagged.
  const bool sparse = (S >= 3) && total <= g.sparse_max;
  if (threadIdx.x < 16) rowmask[threadIdx.x >> 3][threadIdx.x & 7] = (sparse && TT == 16) ? 0u : ~0u;
  __syncthreads();
  bool split_used = false;  // the tile sums are in the split 32-bit form
  if constexpr (S >= 3) {
    // Accumulators: 64-bit adds, or (TT == 16, every tile of at most 65535
    // records) the split form of the region gather: q mod 2^32 summed at
    // word idx, q >> 16 summed at HW + idx, native 32-bit shared adds in
    // place of a 64-bit compare-and-swap loop, in the same bytes.  A tile
    // whose records' node bounds sum to 2^46 or more is redone with 64-bit
    // adds.  The cell value 2^16 H + L is the same integer either way.
    unsigned* const w32 = reinterpret_cast<unsigned*>(acc);
    const int HW = nmesh * (T3 + kMeshPad);
    auto add = [&](auto split, int idx, long long q) {
      if constexpr (decltype(split)::value) {
        atomicAdd(&w32[idx], (unsigned)q);
        atomicAdd(reinterpret_cast<int*>(&w32[HW + idx]), (int)(q >> 16));
      } else {
        atomicAdd(&acc[idx], (unsigned long long)q);
      }
    };
    auto run = [&](auto split) {
   if (sparse) {
    // Lane = (record, mesh, z node), 4 lanes per record and mesh: all the
    // records of the tile in one step.  The z = 0 lane flags the rows.
    const WRec* recs = reinterpret_cast<const WRec*>(g.rec);
    const int G = nmesh * 4;
    for (unsigned u = threadIdx.x; u < total * (unsigned)G; u += blockDim.x) {
      const unsigned i = u / (unsigned)G;
      const int sub = (int)(u - i * (unsigned)G), m = sub >> 2, kz = sub & 3;
      int b = 0;
#pragma unroll
      for (int step = 64; step > 0; step >>= 1)
        if (b + step < 126 && bstart[b + step] <= i) b += step;
      const WRec* rp = recs + boff[b] + (i - bstart[b]);
      const short4 bs = *reinterpret_cast<const short4*>(&rp->base[m][0]);
      if (decltype(split)::value && kz == 0)
        atomicAdd(&bound_sum[m], __int_as_float((min(bs.w & 0xff, 127) + 127) << 23));
      const float4 wx4 = *reinterpret_cast<const float4*>(&rp->w[m][0][0]);
      const float4 wy4 = *reinterpret_cast<const float4*>(&rp->w[m][1][0]);
      const float wz = rp->w[m][2][kz];
      const float wxs[4] = {wx4.x, wx4.y, wx4.z, wx4.w}, wys[4] = {wy4.x, wy4.y, wy4.z, wy4.w};
      const int sx = rel(bs.x, 0), sy = rel(bs.y, 1), lz = rel(bs.z, 2) + kz;
      if constexpr (TT == 16) {
        if (kz == 0) {
          const int lo = max(sy, 0), hi = min(sy + S, 16);
          if (lo < hi) {
            const unsigned ybits = ((1u << (hi - lo)) - 1u) << lo;
#pragma unroll
            for (int x = 0; x < S; x++) {
              const int lx = sx + x;
              if ((unsigned)lx < 16u) atomicOr(&rowmask[m][lx >> 1], ybits << ((lx & 1) * 16));
            }
          }
        }
      }
      if (kz >= S || (unsigned)lz >= (unsigned)T) continue;
      unsigned long long* A = acc + m * (T3 + kMeshPad);
      // node value wx * (wy * wz), in the order of the other mappings, so
      // that the mesh does not depend on which one runs
      const float wyz[4] = {wys[0] * wz, wys[1] * wz, wys[2] * wz, wys[3] * wz};
#pragma unroll
      for (int x = 0; x < S; x++) {
        const int lx = sx + x;
        if ((unsigned)lx >= (unsigned)T) continue;
#pragma unroll
        for (int y = 0; y < S; y++) {
          const int ly = sy + y;
          if ((unsigned)ly >= (unsigned)T) continue;
          const int col = kSwz ? (lz ^ ((ly & 3) << 2)) : lz;
          const float v = wxs[x] * wyz[y];
          const long long q = (bs.w & 0x100) ? round_small(v) : round_fix(v);
          add(split, (int)(A - acc) + (lx * T + ly) * T + col, q);
        }
      }
    }
   } else {
    // One record per warp.  Lane = (mesh, or x parity with one mesh; y node;
    // z node); each lane loops over the x nodes.  With the swizzle, the 16
    // (y, z) cells of one mesh and x plane sit in 16 distinct bank pairs.
    // The next record's loads are issued before this one's atomics.
    const WRec* recs = reinterpret_cast<const WRec*>(g.rec);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int half = lane >> 4, yy = (lane >> 2) & 3, zz = lane & 3;
    const int m = (nmesh == 2) ? half : 0;
    const bool act = yy < S && zz < S;
    struct Ld {
      float4 wx;
      float wy, wz;
      int b0, b1, b2, small;
      float bound;  // 2^e above every node value of the record (2^-32 units)
    };
    auto load = [&](unsigned i, int& b) {
      while (bstart[b + 1] <= i) b++;  // warp-uniform; i only grows
      const WRec* rp = recs + boff[b] + (i - bstart[b]);
      Ld L;
      L.wx = *reinterpret_cast<const float4*>(&rp->w[m][0][0]);
      L.wy = rp->w[m][1][yy];
      L.wz = rp->w[m][2][zz];
      const short4 bs = *reinterpret_cast<const short4*>(&rp->base[m][0]);
      L.b0 = bs.x;
      L.b1 = bs.y;
      L.b2 = bs.z;
      L.small = bs.w & 0x100;
      L.bound = __int_as_float((min(bs.w & 0xff, 127) + 127) << 23);
      return L;
    };
    int b = 0;
    unsigned i = warp;
    Ld nxt{};
    if (i < total) nxt = load(i, b);
    for (; i < total; i += nw) {
      const Ld cur = nxt;
      if (i + nw < total) nxt = load(i + nw, b);
      if (decltype(split)::value && yy == 0 && zz == 0 && (nmesh == 2 || half == 0))
        atomicAdd(&bound_sum[m], cur.bound);
      if (!act) continue;
      const int ly = rel(cur.b1, 1) + yy, lz = rel(cur.b2, 2) + zz;
      if ((unsigned)ly >= (unsigned)T || (unsigned)lz >= (unsigned)T) continue;
      const float wyz = cur.wy * cur.wz;
      const int col = kSwz ? (lz ^ ((ly & 3) << 2)) : lz;
      unsigned long long* A = acc + m * (T3 + kMeshPad) + ly * T + col;
      const int dx = rel(cur.b0, 0);
      const float wxs[4] = {cur.wx.x, cur.wx.y, cur.wx.z, cur.wx.w};
#pragma unroll
      for (int x = 0; x < S; x++) {
        if (nmesh == 1 && (x & 1) != half) continue;  // one mesh: the halves split x
        const int lx = dx + x;
        if ((unsigned)lx >= (unsigned)T) continue;
        const float v = wxs[x] * wyz;
        const long long q = cur.small ? round_small(v) : round_fix(v);  // warp-uniform
        add(split, (int)(A - acc) + lx * T * T, q);
      }
    }
   }
    };
    bool done = false;
    if constexpr (TT == 16) {
      if (total <= 65535u) {
        if (threadIdx.x < 2) bound_sum[threadIdx.x] = 0.f;
        __syncthreads();
        run(std::integral_constant<bool, true>());
        __syncthreads();
        done = bound_sum[0] < 70368744177664.f && bound_sum[1] < 70368744177664.f;  // 2^46
        split_used = done;
        if (!done) {
          ulonglong2* a2 = reinterpret_cast<ulonglong2*>(acc);
          for (int e = threadIdx.x; e < nmesh * (T3 + kMeshPad) / 2; e += blockDim.x)
            a2[e] = make_ulonglong2(0ull, 0ull);
          __syncthreads();
        }
      }
    }
    if (!done) run(std::integral_constant<bool, false>());
  } else {
    // Work item = (record, mesh, z node): P lanes per mesh (P = S rounded up
    // to a power of two), G = nmesh * P lanes per record, aligned within the
    // warp.  Lanes of one record hit consecutive words along z (no bank
    // conflicts); the meshes are kMeshPad words apart.
    constexpr int P = (S == 3) ? 4 : S;
    const int G = nmesh * P;
    const int lane = threadIdx.x & 31;
    const int sub = lane % G, m = sub / P, kz = sub % P;
    const unsigned nwork = total * (unsigned)G;
    for (unsigned u = threadIdx.x; u < nwork; u += blockDim.x) {
      const unsigned i = u / (unsigned)G;
      // largest b with bstart[b] <= i (bstart[0] = 0, bstart[125] = total > i)
      int b = 0;
  #pragma unroll
      for (int step = 64; step > 0; step >>= 1)
        if (b + step < 126 && bstart[b + step] <= i) b += step;
      if (kz >= S) continue;
      const Rec r = rec[boff[b] + (i - bstart[b])];
      float w[3][4];
      int loc[3][4];
  #pragma unroll
      for (int a = 0; a < 3; a++) {
        node_weights<S>(m ? r.par[1][a] : r.par[0][a], w[a]);
  #pragma unroll
        for (int k = 0; k < S; k++) {
          int node = (m ? r.base[1][a] : r.base[0][a]) + of + k;
          node += (node < 0) ? ng : 0;
          node -= (node >= ng) ? ng : 0;
          int l = node - org[a];
          l += (l < 0) ? ng : 0;
          loc[a][k] = (l < T) ? l : -1;
        }
      }
      // this lane's z node
      float wz = w[2][0];
      int lz = loc[2][0];
  #pragma unroll
      for (int k = 1; k < S; k++)
        if (kz == k) {
          wz = w[2][k];
          lz = loc[2][k];
        }
      if (lz < 0) continue;
      unsigned long long* A = acc + m * (T3 + kMeshPad) + lz;
      const float wzf = wz * r.wf;
  #pragma unroll
      for (int x = 0; x < S; x++) {
        if (loc[0][x] < 0) continue;
        const float wxz = w[0][x] * wzf;
        const int row = loc[0][x] * T;
  #pragma unroll
        for (int y = 0; y < S; y++) {
          if (loc[1][y] < 0) continue;
          const long long q = (S == 1) ? r.q : round_fix(wxz * w[1][y]);
          atomicAdd(&A[(row + loc[1][y]) * T], (unsigned long long)q);
        }
      }
    }
  }
  __syncthreads();
  // write the tile: rows of T cells along z
  const long long off = INT64 ? 0 : *g.moff;  // mean cell value (k_wsum)
  if constexpr (TT == 16) {
    // 4 consecutive z cells per thread and step; untouched rows are -mean
    const float cst = fix_to_float(-off);
    for (int e = threadIdx.x; e < nmesh * 256 * 4; e += blockDim.x) {
      const int q = e & 3, row = (e >> 2) & 255, m = e >> 10;
      const int lx = row >> 4, ly = row & 15;
      const size_t cell = ((size_t)(org[0] + lx) * ng + org[1] + ly) * ng + org[2] + 4 * q;
      const bool touched = (rowmask[m][row >> 5] >> (row & 31)) & 1u;
      ulonglong2 u0 = make_ulonglong2(0ull, 0ull), u1 = u0;
      if (touched) {
        const int pq = kSwz ? (q ^ (ly & 3)) : q;  // stored block of z cells [4q, 4q + 4)
        if (split_used) {
          const unsigned* w32 = reinterpret_cast<const unsigned*>(acc);
          const int idx = m * (T3 + kMeshPad) + row * 16 + 4 * pq;
          const uint4 lo = *reinterpret_cast<const uint4*>(w32 + idx);
          const int4 hi = *reinterpret_cast<const int4*>(w32 + nmesh * (T3 + kMeshPad) + idx);
          auto join = [](unsigned l, int h) {
            return (unsigned long long)(((long long)h << 16) +
                                        (long long)(unsigned)(l - ((unsigned)h << 16)));
          };
          u0 = make_ulonglong2(join(lo.x, hi.x), join(lo.y, hi.y));
          u1 = make_ulonglong2(join(lo.z, hi.z), join(lo.w, hi.w));
        } else {
          const ulonglong2* Ar =
              reinterpret_cast<const ulonglong2*>(acc + m * (T3 + kMeshPad) + row * 16);
          u0 = Ar[2 * pq];
          u1 = Ar[2 * pq + 1];
        }
      }
      if (INT64) {
        longlong2* o = reinterpret_cast<longlong2*>(g.out64[m] + cell);
        o[0] = make_longlong2((long long)u0.x, (long long)u0.y);
        o[1] = make_longlong2((long long)u1.x, (long long)u1.y);
      } else {
        float4 v = make_float4(cst, cst, cst, cst);
        if (touched)
          v = make_float4(fix_to_float((long long)u0.x - off), fix_to_float((long long)u0.y - off),
                          fix_to_float((long long)u1.x - off), fix_to_float((long long)u1.y - off));
        *reinterpret_cast<float4*>(g.out[m] + cell) = v;
      }
    }
  } else {
    for (int m = 0; m < nmesh; m++) {
      const unsigned long long* A = acc + m * (T3 + kMeshPad);
      for (int e = threadIdx.x; e < T3; e += blockDim.x) {
        const int lx = e / (T * T), ly = (e / T) % T, lz = e % T;
        const size_t cell = ((size_t)(org[0] + lx) * ng + org[1] + ly) * ng + org[2] + lz;
        const long long v = (long long)A[e];
        if (INT64)
          g.out64[m][cell] = v;
        else
          g.out[m][cell] = fix_to_float(v - off);
      }
    }
  }
}

// 16-byte asynchronous copy global -> shared (one group per commit).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// FP32 form of a region (the FP32 meshes): word (row, rem) of the region's
// [R][R][RG][NM] layout (row = x * R + y, rem = z * NM + mesh) as FP32, the
// mean cell value subtracted in fixed point from the tile's own cells
// (region index [1 - of, T + 1 - of) on every axis), so that a cell's sum
// over its regions carries the mean once.  NM == 2: four words per 16-byte
// store, NM == 1: two per 8-byte store.  word(row, rem) -> fixed-point sum.
template <int S, int NM, class Word>
__device__ __forceinline__ void region_out_f32(const GatherArgs& g, unsigned tile, Word word) {
  constexpr int R = RegGeom<S>::R, RG = RegGeom<S>::RG, RP = RegGeom<S>::RP;
  constexpr int T = kRegT, of = (S >= 3) ? -1 : 0, ROW = RG * NM, V = 2 * NM;
  static_assert((NM * RP) % V == 0, "whole stores per region");
  const long long off = *g.moff;
  float* o = reinterpret_cast<float*>(g.regbuf) + (size_t)tile * NM * RP;
  for (int e = threadIdx.x; e < NM * RP / V; e += blockDim.x) {
    float v[V];
#pragma unroll
    for (int j = 0; j < V; j++) {
      const int wi = V * e + j, row = wi / ROW, rem = wi - row * ROW;
      const int ux = row / R, uy = row - ux * R, uz = rem / NM;
      const bool home = (unsigned)(ux - 1 + of) < (unsigned)T && (unsigned)(uy - 1 + of) < (unsigned)T &&
                        (unsigned)(uz - 1 + of) < (unsigned)T;
      v[j] = fix_to_float(word(row, rem) - (home ? off : 0ll));
    }
    if constexpr (NM == 2)
      *reinterpret_cast<float4*>(o + V * e) = make_float4(v[0], v[1], v[2], v[3]);
    else
      *reinterpret_cast<float2*>(o + V * e) = make_float2(v[0], v[1]);
  }
}

// ---- region gather.  One CTA per home tile (the tile of the plain grid's
// base node): each record is added once, into shared-memory accumulators
// that cover every node its stencils reach, local cells [of - 1, T + of +
// S - 1] per axis.  The regions are written out and k_region_sum adds, for
// each cell, the up to 8 regions that cover it.  The integer sums are the
// tile gather's, so the mesh is the same to the bit.
template <int S, int NM>
__global__ void __launch_bounds__(NM == 2 ? 1024 : 512, 1) k_gather_region(const __grid_constant__ GatherArgs g) {
  constexpr int R = RegGeom<S>::R, RP = RegGeom<S>::RP, RZ = RegGeom<S>::RZ, SM = RegGeom<S>::SM;
  constexpr int RG = RegGeom<S>::RG;
  // 64-bit path: acc[NM][SM].  Split path, the same bytes as 32-bit words:
  // the node values q mod 2^32 summed at [c * NM + m], q >> 16 summed at
  // HW + [c * NM + m] (meshes interleaved: with two meshes the half-warps
  // use even and odd banks).
  extern __shared__ __align__(16) unsigned long long acc[];
  constexpr int HW = NM * R * R * RZ;
  unsigned* const w32 = reinterpret_cast<unsigned*>(acc);
  __shared__ float bound_sum[2];
  const int nt = g.nt;
  const unsigned tile = ((unsigned)blockIdx.z * nt + blockIdx.y) * nt + blockIdx.x;
  const unsigned beg = g.hist[tile], end = g.hist[tile + 1];  // one bucket per tile
  auto zero = [&]() {
    ulonglong2* a2 = reinterpret_cast<ulonglong2*>(acc);
    for (int e = threadIdx.x; e < NM * SM / 2; e += blockDim.x) a2[e] = make_ulonglong2(0ull, 0ull);
  };
  // the accumulators are zeroed while the bucket offsets are in flight (in
  // vain for a tile without records)
  zero();
  if (beg == end) {  // k_region_sum skips tiles without records
    if (threadIdx.x == 0) g.regflag[tile] = 0;
    return;
  }
  // Lane = (mesh, y node, z node) with two meshes, (record of a pair, y
  // node, z node) with one; each lane loops over the x nodes.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int half = lane >> 4, yy = (lane >> 2) & 3, zz = lane & 3;
  const int m = (NM == 2) ? half : 0;
  const bool act = yy < S && zz < S;
  struct Ld {
    float4 wx;
    float wy, wz;
    short2 bs;  // region word offset, flags
  };
  // This warp's records, in stages of 4 consecutive ones (with one mesh
  // the half-warps take alternate records), two stages in flight: a stage
  // is copied as 28 x 16 bytes with cp.async into the warp's ring, one
  // group per stage, and read once its group has landed.
  constexpr int Q = 4;
  unsigned char* const ring =
      reinterpret_cast<unsigned char*>(acc + NM * SM) + warp * (2 * Q * sizeof(WRec));
  const unsigned w0 = beg + (unsigned)(warp * Q), step = (unsigned)(nw * Q);
  const unsigned K = (w0 < end) ? (end - w0 + step - 1) / step : 0u;
  const int cj = lane / 7, part = lane - 7 * cj;  // copy lanes 0-27: record cj, 16-byte part
  const unsigned char* src = reinterpret_cast<const unsigned char*>(g.rec) + part * 16;
  auto issue = [&](unsigned k) {
    const unsigned i = w0 + k * step + (unsigned)cj;
    if (k < K && lane < 7 * Q && i < end)
      cp_async16(ring + ((k & 1) * Q + cj) * sizeof(WRec) + part * 16, src + (size_t)i * sizeof(WRec));
    cp_async_commit();
  };
  // primed: the first stage was issued already (before a CTA barrier)
  auto records = [&](auto&& proc, bool primed) {
    if (!primed) issue(0);
    for (unsigned k = 0; k < K; k++) {
      __syncwarp();  // the stage refilled next was read in step k - 1
      issue(k + 1);
      cp_async_wait<1>();
      __syncwarp();  // every lane's part of stage k has landed
      const unsigned i0 = w0 + k * step;
      const unsigned char* const slot = ring + (k & 1) * Q * sizeof(WRec);
      auto one = [&](int j) {
        const unsigned char* rp = slot + j * sizeof(WRec);
        Ld L;
        L.wx = *reinterpret_cast<const float4*>(rp + m * 48);
        L.wy = *reinterpret_cast<const float*>(rp + m * 48 + 16 + yy * 4);
        L.wz = *reinterpret_cast<const float*>(rp + m * 48 + 32 + zz * 4);
        L.bs = *reinterpret_cast<const short2*>(rp + 96 + m * 8);
        proc(L);
      };
      if (i0 + Q <= end) {  // a full stage
#pragma unroll
        for (int jj = 0; jj < ((NM == 2) ? Q : Q / 2); jj++) one((NM == 2) ? jj : 2 * jj + half);
      } else {
#pragma unroll
        for (int jj = 0; jj < ((NM == 2) ? Q : Q / 2); jj++) {
          const int j = (NM == 2) ? jj : 2 * jj + half;
          if (i0 + (unsigned)j < end) one(j);
        }
      }
    }
    cp_async_wait<0>();
    __syncwarp();
  };
  // Split path.  With q = 2^16 h + l (0 <= l < 2^16), H = sum h and
  // L = sum l: at most 65535 records put at most 65535 terms in a cell, so
  // 0 <= L < 2^32 and L = (sum q - 2^16 H) mod 2^32.  A record whose node
  // values are all below 2^31 (flag 0x100) adds |h| <= 2^15 to a cell; one
  // with larger values adds |h| <= 2^(e - 16), e its bound exponent.  So
  // |H| < 2^31 when n 2^31 + sum over the large records of 2^e < 2^47 (n
  // records): then the cell value is 2^16 H + L exactly.  A tile past that
  // bound is redone below.
  const unsigned nrec = end - beg;
  bool split = nrec <= 65535u;
  if (split) {
    if (threadIdx.x < 2) bound_sum[threadIdx.x] = 0.f;
    issue(0);  // the first stage's copies overlap the barrier
    __syncthreads();
    float bsum = 0.f;  // sum of 2^e over this lane's large-value records (exact: powers >= 2^31)
    const int lbase = (yy * RZ + zz) * NM + m;
    auto proc = [&](const Ld& cur) {
      if (!act) return;
      unsigned* A = w32 + lbase + cur.bs.x * NM;
      const float wyz = cur.wy * cur.wz;
      const float wxs[4] = {cur.wx.x, cur.wx.y, cur.wx.z, cur.wx.w};
      if (cur.bs.y & 0x100) {
#pragma unroll
        for (int x = 0; x < S; x++) {
          const int q = __float2int_rn(wxs[x] * wyz);
          atomicAdd(A + x * R * RZ * NM, (unsigned)q);
          atomicAdd(reinterpret_cast<int*>(A + HW) + x * R * RZ * NM, q >> 16);
        }
      } else {
        bsum += __int_as_float((min(cur.bs.y & 0xff, 127) + 127) << 23);
#pragma unroll
        for (int x = 0; x < S; x++) {
          const long long q = round_fix(wxs[x] * wyz);
          atomicAdd(A + x * R * RZ * NM, (unsigned)q);
          atomicAdd(reinterpret_cast<int*>(A + HW) + x * R * RZ * NM, (int)(q >> 16));
        }
      }
    };
    records(proc, true);
    if (lane == 0 || lane == 16) atomicAdd(&bound_sum[(NM == 2) ? half : 0], bsum);
    __syncthreads();
    const float room = 2147483648.f * (float)(65536u - nrec);  // 2^47 - n 2^31, exact
    split = bound_sum[0] < room && bound_sum[1] < room;
    if (split) {
      if constexpr (NM == 2) {
        if (g.reg_f32) {
          // FP32 regions (see region_out_f32): four words, two cells of both
          // meshes, per thread and step, from 16-byte loads of each array
          constexpr int T = kRegT, of = (S >= 3) ? -1 : 0, ROW = RG * NM;
          static_assert(ROW % 4 == 0 && (RZ * NM) % 4 == 0 && HW % 4 == 0, "16-byte groups");
          const long long off = *g.moff;
          float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(g.regbuf) + (size_t)tile * NM * RP);
          for (int e = threadIdx.x; e < NM * RP / 4; e += blockDim.x) {
            const int row = (4 * e) / ROW, rem = 4 * e - row * ROW;
            const int ux = row / R, uy = row - ux * R, uz = rem / NM;
            const bool hxy = (unsigned)(ux - 1 + of) < (unsigned)T && (unsigned)(uy - 1 + of) < (unsigned)T;
            const long long o0 = (hxy && (unsigned)(uz - 1 + of) < (unsigned)T) ? off : 0ll;
            const long long o1 = (hxy && (unsigned)(uz + of) < (unsigned)T) ? off : 0ll;
            const int w = row * RZ * NM + rem;
            const uint4 lo = *reinterpret_cast<const uint4*>(w32 + w);
            const int4 hi = *reinterpret_cast<const int4*>(w32 + HW + w);
            auto join = [](unsigned l, int h) {
              return ((long long)h << 16) + (long long)(l - ((unsigned)h << 16));
            };
            o[e] = make_float4(fix_to_float(join(lo.x, hi.x) - o0), fix_to_float(join(lo.y, hi.y) - o0),
                               fix_to_float(join(lo.z, hi.z) - o1), fix_to_float(join(lo.w, hi.w) - o1));
          }
          if (threadIdx.x == 0) g.regflag[tile] = 1;
          return;
        }
      }
      if (g.reg_f32) {
        region_out_f32<S, NM>(g, tile, [&](int row, int rem) {
          const int w = row * RZ * NM + rem;
          const unsigned lo = w32[w];
          const int hi = reinterpret_cast<const int*>(w32 + HW)[w];
          return ((long long)hi << 16) + (long long)(lo - ((unsigned)hi << 16));
        });
        if (threadIdx.x == 0) g.regflag[tile] = 1;
        return;
      }
      // out as [R][R][RG][NM] (meshes interleaved): a pair of words per
      // thread and step, one 16-byte store; the padding column z = R reads
      // zeros
      longlong2* o = reinterpret_cast<longlong2*>(g.regbuf + (size_t)tile * NM * RP);
      constexpr int ROW = RG * NM;
      for (int e = threadIdx.x; e < NM * RP / 2; e += blockDim.x) {
        const int row = (2 * e) / ROW, w = row * RZ * NM + (2 * e - row * ROW);
        const uint2 lo = *reinterpret_cast<const uint2*>(w32 + w);
        const int2 hi = *reinterpret_cast<const int2*>(w32 + HW + w);
        o[e] = make_longlong2(((long long)hi.x << 16) + (long long)(lo.x - ((unsigned)hi.x << 16)),
                              ((long long)hi.y << 16) + (long long)(lo.y - ((unsigned)hi.y << 16)));
      }
      if (threadIdx.x == 0) g.regflag[tile] = 1;
      return;
    }
    __syncthreads();  // every thread has read the bound sums
  }
  // 64-bit path
  zero();
  __syncthreads();
  {
    const int lofs = m * SM + yy * RZ + zz;
    auto proc = [&](const Ld& cur) {
      if (!act) return;
      unsigned long long* A = acc + lofs + cur.bs.x;
      const float wyz = cur.wy * cur.wz;
      const float wxs[4] = {cur.wx.x, cur.wx.y, cur.wx.z, cur.wx.w};
      if (cur.bs.y & 0x100) {
#pragma unroll
        for (int x = 0; x < S; x++)
          atomicAdd(A + x * R * RZ, (unsigned long long)round_small(wxs[x] * wyz));
      } else {
#pragma unroll
        for (int x = 0; x < S; x++)
          atomicAdd(A + x * R * RZ, (unsigned long long)round_fix(wxs[x] * wyz));
      }
    };
    records(proc, false);
  }
  __syncthreads();
  if (g.reg_f32) {
    region_out_f32<S, NM>(g, tile, [&](int row, int rem) {
      return (long long)acc[(rem % NM) * SM + row * RZ + rem / NM];
    });
    if (threadIdx.x == 0) g.regflag[tile] = 1;
    return;
  }
  // out as [R][R][RG][NM], as above
  longlong2* o = reinterpret_cast<longlong2*>(g.regbuf + (size_t)tile * NM * RP);
  constexpr int ROW = RG * NM;
  for (int e = threadIdx.x; e < NM * RP / 2; e += blockDim.x) {
    const int row = (2 * e) / ROW, rem = 2 * e - row * ROW;
    long long v[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int c = (rem + j) / NM, mm = (rem + j) % NM;
      v[j] = (long long)acc[mm * SM + row * RZ + c];
    }
    o[e] = make_longlong2(v[0], v[1]);
  }
  if (threadIdx.x == 0) g.regflag[tile] = 1;
}

// Regions covering cell c along one axis: the home tile t0 = c / T at
// region index u - of + 1 (u = c - t0 T), the tile before for u < S + of,
// the tile after for u >= T + of - 1 (never both: S < T).
template <int S>
__device__ __forceinline__ int region_sources(int c, int nt, int* t, int* idx) {
  constexpr int T = kRegT, of = (S >= 3) ? -1 : 0;
  const int t0 = c / T, u = c - t0 * T;
  t[0] = t0;
  idx[0] = u - of + 1;
  if (u < S + of) {
    t[1] = (t0 == 0) ? nt - 1 : t0 - 1;
    idx[1] = u + T - of + 1;
    return 2;
  }
  if (u >= T + of - 1) {
    t[1] = (t0 == nt - 1) ? 0 : t0 + 1;
    idx[1] = u - T - of + 1;
    return 2;
  }
  return 1;
}

// Two consecutive cells of every mesh from a region row: words [c NM + m]
// (cell-major, mesh-minor), one 32- or 16-byte load.
template <int NM>
__device__ __forceinline__ void load_pair(const unsigned long long* p, long long (&v)[2 * NM]) {
  if constexpr (NM == 2) {
    const longlong4_32a q = *reinterpret_cast<const longlong4_32a*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else {
    const longlong2 q = *reinterpret_cast<const longlong2*>(p);
    v[0] = q.x;
    v[1] = q.y;
  }
}

template <int NM>
__device__ __forceinline__ void load_pair_f32(const float* p, float (&v)[2 * NM]) {
  if constexpr (NM == 2) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else {
    const float2 q = *reinterpret_cast<const float2*>(p);
    v[0] = q.x;
    v[1] = q.y;
  }
}

// Mesh from the regions: a pair of consecutive z cells of every mesh per
// thread (a warp reads 32 consecutive pairs: whole sectors), the FP32 sum
// of the FP32 regions (F32R), or from int64 regions the exact fixed-point
// sum (INT64) or its FP32 value minus the mean.  Regions are [R][R][RG][NM]
// words; a cell pair starts on an even region cell.  A tile
// without records wrote neither its region nor a flag of 1, and its words
// (loaded alongside the flag) are dropped.
template <int S, int NM, bool INT64, bool F32R>
__global__ void __launch_bounds__(256) k_region_sum(const __grid_constant__ GatherArgs g) {
  constexpr int T = kRegT, R = RegGeom<S>::R, RG = RegGeom<S>::RG, RP = RegGeom<S>::RP;
  constexpr int of = (S >= 3) ? -1 : 0;
  constexpr int NB = S + of;      // cells u < NB also take the tile before (cell u + T - of + 1)
  constexpr int NA = T + of - 1;  // cells u >= NA also take the tile after (cell u - T - of + 1)
  static_assert((1 - of) % 2 == 0 && RG % 2 == 0 && NA % 2 == 0,
                "cell pairs start on even region cells; a pair never straddles NA");
  static_assert(NB % 2 == 0 || (NB + T - of + 1 == R && RG > R),
                "a pair straddling NB reads the padding column as its second cell");
  const int ng = g.ng, nt = g.nt, nh = ng >> 1;
  const size_t work = (size_t)ng * ng * nh;
  const long long off = INT64 ? 0 : *g.moff;  // mean cell value (k_wsum)
  const unsigned long long* const rb = g.regbuf;
  const float* const rbf = reinterpret_cast<const float*>(g.regbuf);  // FP32 regions
  const float mean_neg = fix_to_float(-off);  // a cell whose home tile has no records
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < work;
       e += (size_t)gridDim.x * blockDim.x) {
    const int zh = (int)(e % (size_t)nh);
    const size_t r = e / (size_t)nh;
    const int y = (int)(r % (size_t)ng), x = (int)(r / (size_t)ng);
    int tx[2], ix[2], ty[2], iy[2];
    const int nx = region_sources<S>(x, nt, tx, ix), ny = region_sources<S>(y, nt, ty, iy);
    const int z = 2 * zh, tz = z / T, uz = z - tz * T;  // uz even
    // the second z source: the tile before for uz < NB (for PCS the pair
    // (2, 3) reads its cells (R - 1, R): cell 3 gets the zero padding
    // column), the tile after for uz >= NA
    int tz2 = -1, cz2 = 0;
    if (uz < NB) {
      tz2 = (tz == 0) ? nt - 1 : tz - 1;
      cz2 = uz + T - of + 1;
    } else if (uz >= NA) {
      tz2 = (tz == nt - 1) ? 0 : tz + 1;
      cz2 = uz - T - of + 1;
    }
    if constexpr (F32R) {
      // FP32 regions: the (x, y) sources q = 2a + b (a < nx, b < ny), the
      // home tile's (which carries the mean) first; every source's flags
      // and words are loaded before any is added, so that a thread has all
      // its loads in flight at once
      unsigned t0q[4], t1q[4];
      int rowq[4];
      bool onq[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int a = q >> 1, b = q & 1;
        onq[q] = a < nx && b < ny;
        const unsigned tb = onq[q] ? ((unsigned)tx[a] * nt + (unsigned)ty[b]) * nt : 0u;
        rowq[q] = onq[q] ? (ix[a] * R + iy[b]) * RG : 0;
        t0q[q] = tb + tz;
        t1q[q] = tb + (tz2 >= 0 ? tz2 : 0);
      }
      float v0[4][2 * NM], v1[4][2 * NM];
      bool f0[4], f1[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        f0[q] = f1[q] = false;
        if (onq[q]) {
          f0[q] = g.regflag[t0q[q]] != 0;
          load_pair_f32<NM>(rbf + ((size_t)t0q[q] * RP + (size_t)(rowq[q] + uz - of + 1)) * NM, v0[q]);
          if (tz2 >= 0) {
            f1[q] = g.regflag[t1q[q]] != 0;
            load_pair_f32<NM>(rbf + ((size_t)t1q[q] * RP + (size_t)(rowq[q] + cz2)) * NM, v1[q]);
          }
        }
      }
      float s[2 * NM];
#pragma unroll
      for (int k = 0; k < 2 * NM; k++) s[k] = 0.f;
#pragma unroll
      for (int q = 0; q < 4; q++) {
#pragma unroll
        for (int k = 0; k < 2 * NM; k++) s[k] += f0[q] ? v0[q][k] : ((q == 0) ? mean_neg : 0.f);
        if (f1[q]) {
#pragma unroll
          for (int k = 0; k < 2 * NM; k++) s[k] += v1[q][k];
        }
      }
      const size_t cell = ((size_t)x * ng + y) * ng + z;
#pragma unroll
      for (int m = 0; m < NM; m++)
        *reinterpret_cast<float2*>(g.out[m] + cell) = make_float2(s[m], s[NM + m]);
    } else {
      long long s[2 * NM];
#pragma unroll
      for (int k = 0; k < 2 * NM; k++) s[k] = 0;
      // int64 regions, one source after another (the exact sums, in 98
      // registers with every load in flight, ran slower)
      for (int a = 0; a < nx; a++)
        for (int b = 0; b < ny; b++) {
          const unsigned tb = ((unsigned)tx[a] * nt + (unsigned)ty[b]) * nt;
          const int row = (ix[a] * R + iy[b]) * RG;
          const unsigned t0 = tb + tz;
          const bool f0 = g.regflag[t0] != 0;
          long long v0[2 * NM], v1[2 * NM];
          load_pair<NM>(rb + ((size_t)t0 * RP + (size_t)(row + uz - of + 1)) * NM, v0);
          bool f1 = false;
          if (tz2 >= 0) {
            const unsigned t1 = tb + tz2;
            f1 = g.regflag[t1] != 0;
            load_pair<NM>(rb + ((size_t)t1 * RP + (size_t)(row + cz2)) * NM, v1);
          }
          if (f0) {
#pragma unroll
            for (int k = 0; k < 2 * NM; k++) s[k] += v0[k];
          }
          if (f1) {
#pragma unroll
            for (int k = 0; k < 2 * NM; k++) s[k] += v1[k];
          }
        }
      const size_t cell = ((size_t)x * ng + y) * ng + z;
#pragma unroll
      for (int m = 0; m < NM; m++) {
        if (INT64)
          *reinterpret_cast<longlong2*>(g.out64[m] + cell) = make_longlong2(s[m], s[NM + m]);
        else
          *reinterpret_cast<float2*>(g.out[m] + cell) =
              make_float2(fix_to_float(s[m] - off), fix_to_float(s[NM + m] - off));
      }
    }
  }
}

}  // namespace

bool gather_region_ok(int ng, int T, int assign) {
  return assign >= 2 && T == kRegT && ng >= kRegT + width(assign) + 1;
}

size_t gather_region_words(int assign) {
  return assign == 2 ? (size_t)RegGeom<3>::RP : (size_t)RegGeom<4>::RP;
}

size_t gather_region_smem(int assign, int interlace) {
  // accumulators + a ring of 2 stages x 4 records per warp (1024 threads
  // with two meshes, 512 with one)
  const size_t acc = (size_t)(interlace ? 2 : 1) * (assign == 2 ? RegGeom<3>::SM : RegGeom<4>::SM) *
                     sizeof(unsigned long long);
  return acc + (size_t)(interlace ? 32 : 16) * 2 * 4 * sizeof(WRec);
}

int gather_tile(int ng) {
  int best = 0;
  for (int t = 4; t <= 16; t++)
    if (ng % t == 0 && ng / t >= 2) best = t;
  return best;
}

size_t gather_record_bytes() { return kRecBytes; }

size_t gather_keys(int ng) {
  const int T = gather_tile(ng);
  if (!T) return 0;
  const size_t nt = (size_t)(ng / T);
  return nt * nt * nt * 27;
}

namespace {
// The same for nkeys <= kScanBlock (the region gather's one bucket per
// tile): one block, the total into hist[n].
__global__ void __launch_bounds__(256) k_scan_one(unsigned* hist, size_t n) {
  __shared__ unsigned sh[8];
  const size_t base = (size_t)threadIdx.x * kScanPer;
  unsigned v[kScanPer];
  unsigned s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    v[k] = (base + k < n) ? hist[base + k] : 0;
    s += v[k];
  }
  unsigned total;
  unsigned run = block_exclusive(s, sh, total);
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    if (base + k < n) hist[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) hist[n] = total;
}
}  // namespace

namespace {
// CTAs of a grid-stride assignment kernel over n particles: the resident
// CTAs of all SMs (the occupancy query; 2048 without a device), at most one
// per 256 particles and at most kAssignMaxBlocks (the weight partials).
size_t assign_grid(size_t n, const void* kernel, int threads, size_t smem) {
  size_t cap = kAssignMaxBlocks;
  int dev = 0, nsm = 0, per = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) == cudaSuccess &&
      nsm > 0 && per > 0)
    cap = std::min(cap, (size_t)nsm * (size_t)per);
  else
    cudaGetLastError();
  return std::max<size_t>(1, std::min(cap, (n + 255) / 256));
}
}  // namespace

int launch_gather_assign(const Particles& p, GatherArgs g, cudaStream_t s, bool int64_out) {
  int n = 0;
  // FP32 regions for the FP32 meshes of a periodic box; exact int64 ones for
  // the int64 meshes and for survey meshes (data minus alpha randoms), whose
  // cells cancel to a small fraction of their terms
  g.reg_f32 = (int64_out || g.nomean) ? 0 : 1;
  // buckets: (tile, reach class) for the tile gather, one per tile for the region gather
  const size_t nkeys = g.region ? gather_keys(g.ng) / 27 : gather_keys(g.ng);
  if (!int64_out) {
    cudaMemsetAsync(g.hist, 0, (nkeys + 1) * sizeof(unsigned), s);
    // grid-stride kernels: one wave of resident CTAs (a partial last wave
    // of a larger grid would run at part occupancy)
    const size_t blocks = assign_grid(p.n, reinterpret_cast<const void*>(k_classify), 256, 0);
    k_classify<<<(unsigned)blocks, 256, 0, s>>>(g, p);
    n++;
    k_wsum<<<1, kWsumThreads, 0, s>>>(reinterpret_cast<const float4*>(g.wpart), (int)blocks, g.wsum,
                                      g.moff, g.moff_scale, g.nomean);
    n++;
    const int nb = (int)((nkeys + kScanBlock - 1) / kScanBlock);
    if (nb == 1) {
      k_scan_one<<<1, 256, 0, s>>>(g.hist, nkeys);
      n++;
    } else {
      k_scan_reduce<<<nb, 256, 0, s>>>(g.hist, nkeys, g.bsum);
      k_scan_blocks<<<1, 256, 0, s>>>(g.bsum, nb);
      k_scan_apply<<<nb, 256, 0, s>>>(g.hist, nkeys, g.bsum, nb);
      n += 3;
    }
    const size_t scatter_blocks = assign_grid(p.n, reinterpret_cast<const void*>(k_scatter), 32 * kScatterWarps, 0);
    k_scatter<<<(unsigned)scatter_blocks, 32 * kScatterWarps, 0, s>>>(g, p);
    n++;
  }
  if (g.region) {
    const dim3 ntile((unsigned)g.nt, (unsigned)g.nt, (unsigned)g.nt);
    const int nm = g.interlace ? 2 : 1;
    const size_t smem = gather_region_smem(g.assign, g.interlace);
    // two waves of the resident CTAs
    const size_t work = (size_t)g.ng * g.ng * (g.ng / 2), cap = (size_t)152 * 12;
    const unsigned sblocks = (unsigned)((work + 255) / 256 < cap ? (work + 255) / 256 : cap);
#define PS_REGION(SS)                                                                          \
  if (nm == 2) {                                                                               \
    cudaFuncSetAttribute(k_gather_region<SS, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                         (int)smem);                                                           \
    k_gather_region<SS, 2><<<ntile, 1024, smem, s>>>(g);                                       \
  } else {                                                                                     \
    cudaFuncSetAttribute(k_gather_region<SS, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                         (int)smem);                                                           \
    k_gather_region<SS, 1><<<ntile, 512, smem, s>>>(g);                                        \
  }                                                                                            \
  if (int64_out && nm == 2)                                                                    \
    k_region_sum<SS, 2, true, false><<<sblocks, 256, 0, s>>>(g);                               \
  else if (int64_out)                                                                          \
    k_region_sum<SS, 1, true, false><<<sblocks, 256, 0, s>>>(g);                               \
  else if (nm == 2 && g.reg_f32)                                                               \
    k_region_sum<SS, 2, false, true><<<sblocks, 256, 0, s>>>(g);                               \
  else if (nm == 2)                                                                            \
    k_region_sum<SS, 2, false, false><<<sblocks, 256, 0, s>>>(g);                              \
  else if (g.reg_f32)                                                                          \
    k_region_sum<SS, 1, false, true><<<sblocks, 256, 0, s>>>(g);                               \
  else                                                                                         \
    k_region_sum<SS, 1, false, false><<<sblocks, 256, 0, s>>>(g);
    if (g.assign == 2) {
      PS_REGION(3)
    } else {
      PS_REGION(4)
    }
#undef PS_REGION
    return n + 2;
  }
  const int T = g.T;
  const size_t smem = (size_t)(g.interlace ? 2 : 1) * (T * T * T + kMeshPad) * sizeof(unsigned long long);
  const dim3 ntile((unsigned)g.nt, (unsigned)g.nt, (unsigned)g.nt);
  // Few particles per tile: 8 warps per CTA (a CTA's accumulators are held
  // until its last warp ends); many: 16 warps to hide the record latency.
  const unsigned nthr = g.threads ? (unsigned)g.threads
                                   : ((double)p.n >= 64.0 * g.nt * g.nt * g.nt) ? kGatherThreads
                                                                                : kGatherThreads / 2;
#define PS_GATHER_T(SS, TV)                                                                    \
  if (int64_out) {                                                                             \
    cudaFuncSetAttribute(k_gather<SS, true, TV>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                         (int)smem);                                                           \
    k_gather<SS, true, TV><<<ntile, nthr, smem, s>>>(g);                             \
  } else {                                                                                     \
    cudaFuncSetAttribute(k_gather<SS, false, TV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                         (int)smem);                                                           \
    k_gather<SS, false, TV><<<ntile, nthr, smem, s>>>(g);                            \
  }
#define PS_GATHER(SS)          \
  if (T == 16) {               \
    PS_GATHER_T(SS, 16)        \
  } else {                     \
    PS_GATHER_T(SS, 0)         \
  }
  switch (g.assign) {
    case 0: PS_GATHER(1); break;
    case 1: PS_GATHER(2); break;
    case 2: PS_GATHER(3); break;
    default: PS_GATHER(4); break;
  }
#undef PS_GATHER_T
#undef PS_GATHER
  n++;
  return n;
}

}  // namespace ps
