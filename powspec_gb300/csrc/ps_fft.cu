// ps_fft.cu -- the first two passes of the hand-written FP32 r2c 3-D FFT.
//
// Replaces FFT_EXEC_R2C (src/fftw_define.h:56, called at
// src/multipole.c:444,459).  The transform is split into three passes, each
// of which reads long contiguous lines, transforms them in shared memory and
// writes them transposed so that the next pass again reads contiguous lines:
//
//   pass A  mesh[x][y][z] (FP32)               ->  A[x][kz][y]   (z, r2c)
//   pass B  A[x][kz][y]                        ->  B[kz][ky][x]  (y)
//   pass C  B[kz][ky][x] -> x transform, then binned in place (ps_bin.cu)
//
// The meshes arrive as FP32 with the mean cell value already subtracted
// (ps_gather.cu): only the k = 0 mode changes, which the periodic-box
// estimator never uses (src/multipole.c:806), while FP32 round-off of every
// other mode scales with the norm of the input.
#include "ps_internal.h"

namespace ps {
namespace {

// Harmonic weight of real cell (i, j, k) for the survey multipoles.
__device__ __forceinline__ float cell_harmonic(const PassAArgs& a, int i, int j, int k) {
  return (i == 0 && j == 0) ? 1.f
                            : ylm_eval(a.yc, (i + a.org[0]) * a.len[0], (j + a.org[1]) * a.len[1],
                                       (k + a.org[2]) * a.len[2]);
}

template <bool P2>
__global__ void __launch_bounds__(kFftThreads, 2) k_pass_a(const __grid_constant__ PassAArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, M = ng >> 1, ngk = M + 1;
  const int ls = line_stride(M + 1, P2);
  const int nty = (ng + a.ty - 1) / a.ty;
  const int x = blockIdx.x / nty;
  const int y0 = (blockIdx.x - x * nty) * a.ty;
  const int nl = min(a.ty, ng - y0);

  const float* base = a.fgrid + ((size_t)x * ng + y0) * ng;
  for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
    const int r = e / M, m = e - r * M;
    float2 v = __ldcs(reinterpret_cast<const float2*>(base + (size_t)r * ng) + m);
    if (a.yw) {
      v.x *= cell_harmonic(a, x, y0 + r, 2 * m);
      v.y *= cell_harmonic(a, x, y0 + r, 2 * m + 1);
    }
    sm[r * ls + lidx<P2>(m)] = v;
  }
  __syncthreads();
  if (P2)
    fft2_lines(sm, a.plan_half.logn, nl, ls, a.tw_half);
  else
    fft_lines(sm, a.plan_half, nl, ls, a.tw_half);

  // Real-to-complex split of each line: Z = FFT_M(x[2m] + i x[2m+1]);
  // X[k] = E + W^k O with E = (Z[k] + conj Z[M-k]) / 2,
  // O = -i (Z[k] - conj Z[M-k]) / 2, W = exp(-2 pi i / ng), k = 0..M.
  const int half = (M >> 1) + 1;
  for (int e = threadIdx.x; e < nl * half; e += blockDim.x) {
    const int r = e / half, k = e - r * half;
    float2* L = sm + r * ls;
    if (k == 0) {
      const float2 z = L[0];
      L[0] = make_float2(z.x + z.y, 0.f);
      L[lidx<P2>(M)] = make_float2(z.x - z.y, 0.f);
    } else {
      const int ik = lidx<P2>(k), imk = lidx<P2>(M - k);
      const float2 A = L[ik], B = L[imk];
      const float2 E = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
      const float2 O = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
      const float2 W = __ldg(&a.tw_full[k]);
      const float2 WO = cmul(W, O);
      // W^(M-k) = -conj(W)
      const float2 W2O = cmul(make_float2(-W.x, W.y), make_float2(O.x, -O.y));
      L[ik] = cadd(E, WO);
      L[imk] = make_float2(E.x + W2O.x, -E.y + W2O.y);
    }
  }
  __syncthreads();

  float2* ob = a.out + (size_t)x * ngk * ng + y0;
  for (int e = threadIdx.x; e < ngk * nl; e += blockDim.x) {
    const int kz = e / nl, r = e - kz * nl;
    ob[(size_t)kz * ng + r] = sm[r * ls + lidx<P2>(kz)];
  }
}

template <bool P2>
__global__ void __launch_bounds__(kFftThreads, 2) k_pass_b(const __grid_constant__ PassBArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, ngk = (ng >> 1) + 1;
  const int ls = line_stride(ng, P2);
  const int ntx = (ng + a.tx - 1) / a.tx;
  const int kz = blockIdx.x / ntx;
  const int x0 = (blockIdx.x - kz * ntx) * a.tx;
  const int nl = min(a.tx, ng - x0);
  const int h = ng >> 1;
  for (int e = threadIdx.x; e < nl * h; e += blockDim.x) {
    const int r = e / h, m = e - r * h;
    const float4 v = __ldcs(reinterpret_cast<const float4*>(
                               a.in + ((size_t)(x0 + r) * ngk + kz) * ng) + m);
    sm[r * ls + lidx<P2>(2 * m)] = make_float2(v.x, v.y);
    sm[r * ls + lidx<P2>(2 * m + 1)] = make_float2(v.z, v.w);
  }
  __syncthreads();
  if (P2)
    fft2_lines(sm, a.plan_full.logn, nl, ls, a.tw_full);
  else
    fft_lines(sm, a.plan_full, nl, ls, a.tw_full);
  float2* ob = a.out + (size_t)kz * ng * ng + x0;
  for (int e = threadIdx.x; e < ng * nl; e += blockDim.x) {
    const int ky = e / nl, r = e - ky * nl;
    ob[(size_t)ky * ng + r] = sm[r * ls + lidx<P2>(ky)];
  }
}

// ---------------------------------------------------------------------------
// Pipelined power-of-two passes.  Persistent CTAs (one per SM); thread 0
// issues the bulk copies of tile t+1's input rows into the other half of a
// double-buffered staging area while all threads transform tile t.  The
// first radix pass reads the staging buffer, later passes work in place on
// the padded FFT buffer.  Waits are bounded: on time-out the CTA raises
// err[0] |= 2 and stops.

struct Pipe {
  uint64_t* bar;  // [2]
  int it;
};

// MAXLOG 4: radix-16 passes on 4096-value tiles, two CTAs per SM; MAXLOG 5:
// radix-32 passes on 8192-value tiles, one CTA per SM.
template <int MAXLOG>
__global__ void __launch_bounds__(kFftThreads, MAXLOG == 4 ? 2 : 1) k_pass_a_tma(const __grid_constant__ PassAArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int s_abort;
  const int ng = a.ng, M = ng >> 1, ngk = M + 1;
  const int logm = a.plan_half.logn;
  const int ls = line_stride(M + 1, true);
  const int nty = (ng + a.ty - 1) / a.ty;
  const int ntile = ng * nty;
  const size_t selems = ((size_t)a.ty * ls + 1) & ~(size_t)1;  // 16-byte aligned
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  float2* stage[2];
  stage[0] = reinterpret_cast<float2*>(smraw + 128);
  stage[1] = stage[0] + selems;
  float2* F = stage[1] + selems;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  // real rows of ng floats, staged as M complex values (x[2m], x[2m+1])
  int nissued = 0;  // copies issued (thread 0)
  auto issue = [&](int tile, int s) {
    nissued++;
    const int x = tile / nty, y0 = (tile - x * nty) * a.ty;
    const int nl = min(a.ty, ng - y0);
    mbar_expect_tx(&bar[s], (uint32_t)(nl * ng * 4));
    if (a.stall && blockIdx.x == 0 && nissued == 2) return;  // test hook: no copy
    const float* src = a.fgrid + ((size_t)x * ng + y0) * ng;
    for (int r = 0; r < nl; r++)
      bulk_g2s(stage[s] + (size_t)r * M, src + (size_t)r * ng, (uint32_t)(ng * 4), &bar[s]);
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < ntile) issue(blockIdx.x, 0);
  int it = 0;
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x, it++) {
    const int s = it & 1;
    if (threadIdx.x == 0 && tile + (int)gridDim.x < ntile) {
      fence_proxy_async();
      issue(tile + gridDim.x, s ^ 1);
    }
    if (!pipe_wait(bar, it, a.err, &s_abort, wait_limit(a.wait_limit))) break;
    const int x = tile / nty, y0 = (tile - x * nty) * a.ty;
    const int nl = min(a.ty, ng - y0);
    if (a.yw) {  // weight the staged rows in place; the buffer is refilled
                 // by the async proxy only after the fence and two barriers.
                 // tpr threads per row, so the (x, y) part is done per row.
      const int tpr = max(1, (int)blockDim.x / nl);
      const int rstep = (int)blockDim.x / tpr;
      for (int r = threadIdx.x / tpr; r < nl; r += rstep) {
        float* row = reinterpret_cast<float*>(stage[s] + (size_t)r * M);
        const int j = y0 + r;
        if (x == 0 && j == 0) continue;  // the row i = j = 0 keeps weight 1
        const YlmRow w = ylm_row(a.yc, (x + a.org[0]) * a.len[0], (j + a.org[1]) * a.len[1]);
        for (int k = threadIdx.x % tpr; k < ng; k += tpr)
          row[k] *= ylm_cell(a.yc, w, (k + a.org[2]) * a.len[2]);
      }
      fence_proxy_async();
      __syncthreads();
    }
    float2* X = fft2_pp_from<false, MAXLOG>(stage[s], M, 0, F, logm, nl, ls, a.tw_half);
    const int half = (M >> 1) + 1;
    for (int e = threadIdx.x; e < nl * half; e += blockDim.x) {
      const int r = e / half, k = e - r * half;
      float2* L = X + r * ls;
      if (k == 0) {
        const float2 z = L[0];
        L[0] = make_float2(z.x + z.y, 0.f);
        L[pidx(M)] = make_float2(z.x - z.y, 0.f);
      } else {
        const int ik = pidx(k), imk = pidx(M - k);
        const float2 A = L[ik], B = L[imk];
        const float2 E = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        const float2 O = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
        const float2 Wk = __ldg(&a.tw_full[k]);
        const float2 WO = cmul(Wk, O);
        const float2 W2O = cmul(make_float2(-Wk.x, Wk.y), make_float2(O.x, -O.y));
        L[ik] = cadd(E, WO);
        L[imk] = make_float2(E.x + W2O.x, -E.y + W2O.y);
      }
    }
    __syncthreads();
    float2* ob = a.out + (size_t)x * ngk * ng + y0;
    for (int e = threadIdx.x; e < ngk * nl; e += blockDim.x) {
      const int kz = e / nl, r = e - kz * nl;
      ob[(size_t)kz * ng + r] = X[r * ls + pidx(kz)];
    }
    __syncthreads();
  }
  // drain: never exit with a bulk copy in flight into this CTA's memory
  if (threadIdx.x == 0 && s_abort) pipe_drain(bar, nissued, wait_limit(a.wait_limit));
}

// MAXLOG 5: radix-32 passes, 8192-value tiles, one CTA per SM (long lines);
// MAXLOG 4: radix-16 passes, 4096-value tiles, two CTAs per SM.
template <int MAXLOG>
__global__ void __launch_bounds__(kFftThreads, MAXLOG == 4 ? 2 : 1) k_pass_b_tma(const __grid_constant__ PassBArgs a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int s_abort;
  const int ng = a.ng, ngk = (ng >> 1) + 1;
  const int logn = a.plan_full.logn;
  const int ls = line_stride(ng, true);
  const int ntx = (ng + a.tx - 1) / a.tx;
  const int ntile = ngk * ntx;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  const size_t selems = ((size_t)a.tx * ls + 1) & ~(size_t)1;  // 16-byte aligned
  float2* stage[2];
  stage[0] = reinterpret_cast<float2*>(smraw + 128);
  stage[1] = stage[0] + selems;
  float2* F = stage[1] + selems;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  int nissued = 0;  // copies issued (thread 0)
  auto issue = [&](int tile, int s) {
    nissued++;
    const int kz = tile / ntx, x0 = (tile - kz * ntx) * a.tx;
    const int nl = min(a.tx, ng - x0);
    mbar_expect_tx(&bar[s], (uint32_t)(nl * ng * 8));
    if (a.stall && blockIdx.x == 0 && nissued == 2) return;  // test hook: no copy
    for (int r = 0; r < nl; r++)
      bulk_g2s(stage[s] + (size_t)r * ng, a.in + ((size_t)(x0 + r) * ngk + kz) * ng,
               (uint32_t)(ng * 8), &bar[s]);
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < ntile) issue(blockIdx.x, 0);
  int it = 0;
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x, it++) {
    const int s = it & 1;
    if (threadIdx.x == 0 && tile + (int)gridDim.x < ntile) {
      fence_proxy_async();
      issue(tile + gridDim.x, s ^ 1);
    }
    if (!pipe_wait(bar, it, a.err, &s_abort, wait_limit(a.wait_limit))) break;
    const int kz = tile / ntx, x0 = (tile - kz * ntx) * a.tx;
    const int nl = min(a.tx, ng - x0);
    const float2* X = fft2_pp_from<false, MAXLOG>(stage[s], ng, 0, F, logn, nl, ls, a.tw_full);
    float2* ob = a.out + (size_t)kz * ng * ng + x0;
    for (int e = threadIdx.x; e < ng * nl; e += blockDim.x) {
      const int ky = e / nl, r = e - ky * nl;
      ob[(size_t)ky * ng + r] = X[r * ls + pidx(ky)];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && s_abort) pipe_drain(bar, nissued, wait_limit(a.wait_limit));
}

}  // namespace

int launch_pass_a(const PassAArgs& a, cudaStream_t s) {
  if (a.twl && launch_pass_a_w(a, s)) return 1;
  const int M = a.ng / 2;
  const bool p2 = a.plan_half.logn >= 0;
  const size_t smem = (size_t)a.ty * line_stride(M + 1, p2) * sizeof(float2);
  const int nty = (a.ng + a.ty - 1) / a.ty;
  const unsigned grid = (unsigned)(a.ng * nty);
  if (p2 && a.pipe_grid > 0) {
    const size_t sm2 = 128 + 3 * ((((size_t)a.ty * line_stride(M + 1, true)) + 1) & ~(size_t)1) * 8;
    if (a.radix32) {
      cudaFuncSetAttribute(k_pass_a_tma<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
      k_pass_a_tma<5><<<(unsigned)a.pipe_grid, kFftThreads, sm2, s>>>(a);
    } else {
      cudaFuncSetAttribute(k_pass_a_tma<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
      k_pass_a_tma<4><<<(unsigned)a.pipe_grid, kFftThreads, sm2, s>>>(a);
    }
  } else if (p2) {
    cudaFuncSetAttribute(k_pass_a<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pass_a<true><<<grid, kFftThreads, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(k_pass_a<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pass_a<false><<<grid, kFftThreads, smem, s>>>(a);
  }
  return 1;
}

int launch_pass_b(const PassBArgs& a, cudaStream_t s) {
  if (a.twl && launch_pass_b_w(a, s)) return 1;
  const bool p2 = a.plan_full.logn >= 0;
  const size_t smem = (size_t)a.tx * line_stride(a.ng, p2) * sizeof(float2);
  const int ntx = (a.ng + a.tx - 1) / a.tx;
  const int ngk = a.ng / 2 + 1;
  const unsigned grid = (unsigned)(ngk * ntx);
  if (p2 && a.pipe_grid > 0) {
    const size_t sm2 = 128 + 3 * ((((size_t)a.tx * line_stride(a.ng, true)) + 1) & ~(size_t)1) * 8;
    if (a.radix32) {
      cudaFuncSetAttribute(k_pass_b_tma<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
      k_pass_b_tma<5><<<(unsigned)a.pipe_grid, kFftThreads, sm2, s>>>(a);
    } else {
      cudaFuncSetAttribute(k_pass_b_tma<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
      k_pass_b_tma<4><<<(unsigned)a.pipe_grid, kFftThreads, sm2, s>>>(a);
    }
  } else if (p2) {
    cudaFuncSetAttribute(k_pass_b<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pass_b<true><<<grid, kFftThreads, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(k_pass_b<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_pass_b<false><<<grid, kFftThreads, smem, s>>>(a);
  }
  return 1;
}

}  // namespace ps
