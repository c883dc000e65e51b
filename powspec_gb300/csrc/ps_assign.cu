// ps_assign.cu -- particle assignment (NGP / CIC / TSC / PCS) with optional
// half-cell interlacing, into deterministic int64 fixed-point meshes.
//
// Reference: ngp/cic/tsc/pcs (src/genr_mesh.c:50-412), the interlace shift
// (src/genr_mesh.c:590-602, :815-833) and the sim-box bound check
// (src/genr_mesh.c:523-531).
//
// Grid coordinate and branch decisions follow the reference's FP64
// expression x = (pos - bmin) * Ng / L with correctly rounded intrinsics (no
// FMA contraction), so cell indices and the NGP/TSC branches are the
// reference's.  The 1-D stencil weights and their products are FP32; each
// node value is rounded once to 2^-32 fixed point and added with an integer
// atomic, which makes the mesh independent of the order of the atomics.
#include "ps_internal.h"

namespace ps {
namespace {

constexpr int kAssignThreads = 256;

struct Stencil {
  int node[4];
  float w[4];
  int big;  // index of the largest weight (>= 1/2 CIC, 1/2 TSC, 0.48 PCS)
};

// Reference FP64 grid coordinate of one axis; returns the truncated cell and
// the fraction.  shift selects the interlaced grid (lower corner -H/2, and
// positions at or above smin + L moved by -L first).
__device__ __forceinline__ void grid_coord(double pos, double L, int ng, bool shift,
                                          int& i0, double& d) {
  double bmin = 0.0;
  if (shift) {
    bmin = __dsub_rn(0.0, __ddiv_rn(__dmul_rn(0.5, L), (double)ng));
    if (pos >= __dadd_rn(bmin, L)) pos = __dsub_rn(pos, L);
  }
  const double x = __ddiv_rn(__dmul_rn(__dsub_rn(pos, bmin), (double)ng), L);
  i0 = (int)x;
  d = __dsub_rn(x, (double)i0);
  // x can round up to exactly Ng for pos just below L; the reference has no
  // guard there (src/genr_mesh.c:60).  Wrap periodically instead.
  if (i0 >= ng) i0 -= ng;
}

template <int S>
__device__ __forceinline__ void stencil_1d(int i0, double d, int ng, Stencil& st) {
  if (S == 1) {  // NGP: round up at d >= 0.5 (src/genr_mesh.c:64-66)
    st.node[0] = (d >= 0.5) ? ((i0 == ng - 1) ? 0 : i0 + 1) : i0;
    st.w[0] = 1.f;
    st.big = 0;
  } else if (S == 2) {  // CIC (src/genr_mesh.c:98-108)
    const float f = (float)d;
    st.node[0] = i0;
    st.node[1] = (i0 == ng - 1) ? 0 : i0 + 1;
    st.w[0] = 1.f - f;
    st.w[1] = f;
    st.big = (f < 0.5f) ? 0 : 1;
  } else if (S == 3) {  // TSC (src/genr_mesh.c:153-173)
    if (d < 0.5) {
      const float f = (float)d;
      st.node[1] = i0;
      st.node[0] = (i0 == 0) ? ng - 1 : i0 - 1;
      st.node[2] = (i0 == ng - 1) ? 0 : i0 + 1;
      const float a = 0.5f - f;
      st.w[0] = 0.5f * a * a;
      st.w[1] = 0.75f - f * f;
    } else {
      const float f = (float)__dsub_rn(1.0, d);
      st.node[0] = i0;
      st.node[1] = (i0 == ng - 1) ? 0 : i0 + 1;
      st.node[2] = (st.node[1] == ng - 1) ? 0 : st.node[1] + 1;
      const float a = 0.5f + f;
      st.w[0] = 0.5f * a * a;
      st.w[1] = 0.75f - f * f;
    }
    st.w[2] = 1.f - st.w[0] - st.w[1];
    st.big = 1;
  } else {  // PCS: cubic B-spline on nodes i0-1 .. i0+2 (src/genr_mesh.c:257-270)
    const float f = (float)d;
    st.node[1] = i0;
    st.node[0] = (i0 == 0) ? ng - 1 : i0 - 1;
    st.node[2] = (i0 == ng - 1) ? 0 : i0 + 1;
    st.node[3] = (st.node[2] == ng - 1) ? 0 : st.node[2] + 1;
    const float f2 = f * f, f3 = f2 * f;
    const float s = 1.f / 6.f;
    st.w[3] = f3 * s;
    st.w[2] = (1.f + 3.f * (f + f2 - f3)) * s;
    st.w[1] = (4.f - 6.f * f2 + 3.f * f3) * s;
    st.w[0] = 1.f - st.w[1] - st.w[2] - st.w[3];
    st.big = (f < 0.5f) ? 1 : 2;
  }
}

__device__ __forceinline__ void red_add(unsigned long long* cell, long long v) {
  atomicAdd(cell, (unsigned long long)v);
}

template <int S, bool AOS>
__global__ void __launch_bounds__(kAssignThreads)
    k_assign(Particles p, int ng, double L0, double L1, double L2,
             unsigned long long* __restrict__ mesh, int shift, double* wpart, int* err) {
  const double L[3] = {L0, L1, L2};
  double ws = 0.0, wa = 0.0;
  int bad = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += stride) {
    double pos[3], w;
    if (AOS) {
      const double4 r = reinterpret_cast<const double4*>(p.aos)[i];
      pos[0] = r.x; pos[1] = r.y; pos[2] = r.z; w = r.w;
    } else {
      pos[0] = (double)p.x[i];
      pos[1] = (double)p.y[i];
      pos[2] = (double)p.z[i];
      w = p.w ? (double)p.w[i] : 1.0;
    }
    if (!(pos[0] >= 0.0 && pos[0] < L0 && pos[1] >= 0.0 && pos[1] < L1 &&
          pos[2] >= 0.0 && pos[2] < L2)) {
      bad = 1;
      continue;
    }
    if (!shift) {
      ws += w;
      wa += fabs(w);
    }
    Stencil st[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      int i0;
      double d;
      grid_coord(pos[a], L[a], ng, shift != 0, i0, d);
      stencil_1d<S>(i0, d, ng, st[a]);
    }
    if (S == 1) {
      const size_t cell = ((size_t)st[0].node[0] * ng + st[1].node[0]) * ng + st[2].node[0];
      red_add(mesh + cell, __double2ll_rn(w * 4294967296.0));
      continue;
    }
    // Every node gets its FP32 share rounded to fixed point, except the
    // stencil's largest node, which gets the remainder: the particle's
    // quantised weight llrint(w 2^32) is conserved exactly.
    const long long qtot = __double2ll_rn(w * 4294967296.0);
    const float wf = (float)w * kFixScale;
    long long qsum = 0;
    size_t acell = 0;
    int anc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) anc[d] = st[d].big;
#pragma unroll
    for (int a = 0; a < S; a++) {
      const float wx = st[0].w[a] * wf;
#pragma unroll
      for (int b = 0; b < S; b++) {
        const float wxy = wx * st[1].w[b];
        const size_t row = ((size_t)st[0].node[a] * ng + st[1].node[b]) * ng;
#pragma unroll
        for (int c = 0; c < S; c++) {
          const size_t cell = row + st[2].node[c];
          if (a == anc[0] && b == anc[1] && c == anc[2]) {
            acell = cell;
            continue;
          }
          const long long q = __float2ll_rn(wxy * st[2].w[c]);
          qsum += q;
          red_add(mesh + cell, q);
        }
      }
    }
    red_add(mesh + acell, qtot - qsum);
  }
  // Block reduction of the weight sums (plain grid only).
  if (!shift) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ws += __shfl_down_sync(0xffffffffu, ws, o);
      wa += __shfl_down_sync(0xffffffffu, wa, o);
    }
    __shared__ double sws[kAssignThreads / 32], swa[kAssignThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
      sws[wid] = ws;
      swa[wid] = wa;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t0 = 0, t1 = 0;
      for (int k = 0; k < kAssignThreads / 32; k++) {
        t0 += sws[k];
        t1 += swa[k];
      }
      // per-block partials, summed in block order by k_wsum: deterministic
      wpart[2 * blockIdx.x] = t0;
      wpart[2 * blockIdx.x + 1] = t1;
    }
  }
  if (bad) atomicOr(err, 1);
}

__global__ void k_wsum(const double* __restrict__ wpart, int nblocks, double* wsum) {
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0;
    for (int b = 0; b < nblocks; b++) {
      t0 += wpart[2 * b];
      t1 += wpart[2 * b + 1];
    }
    wsum[0] = t0;
    wsum[1] = t1;
  }
}

template <int S>
int launch_s(const Particles& p, const AssignArgs& a, cudaStream_t s) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  size_t blocks = (p.n + kAssignThreads - 1) / kAssignThreads;
  const size_t cap = (size_t)kAssignMaxBlocks;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  int n = 0;
  for (int m = 0; m < (a.mesh1 ? 2 : 1); m++) {
    unsigned long long* mesh = m ? a.mesh1 : a.mesh0;
    if (p.aos)
      k_assign<S, true><<<(unsigned)blocks, kAssignThreads, 0, s>>>(
          p, a.ng, a.box[0], a.box[1], a.box[2], mesh, m, a.wpart, a.err);
    else
      k_assign<S, false><<<(unsigned)blocks, kAssignThreads, 0, s>>>(
          p, a.ng, a.box[0], a.box[1], a.box[2], mesh, m, a.wpart, a.err);
    n++;
    if (m == 0) {
      k_wsum<<<1, 32, 0, s>>>(a.wpart, (int)blocks, a.wsum);
      n++;
    }
  }
  return n;
}

}  // namespace

int launch_assign(const Particles& p, const AssignArgs& a, cudaStream_t s) {
  switch (a.assign) {
    case PS_ASSIGN_NGP: return launch_s<1>(p, a, s);
    case PS_ASSIGN_CIC: return launch_s<2>(p, a, s);
    case PS_ASSIGN_TSC: return launch_s<3>(p, a, s);
    default: return launch_s<4>(p, a, s);
  }
}

}  // namespace ps
