// ps_fft.cu -- the first two passes of the hand-written FP32 r2c 3-D FFT.
//
// Replaces FFT_EXEC_R2C (src/fftw_define.h:56, called at
// src/multipole.c:444,459).  The transform is split into three passes, each
// of which reads long contiguous lines, transforms them in shared memory and
// writes them transposed so that the next pass again reads contiguous lines:
//
//   pass A  grid[x][y][z] (int64 fixed point)  ->  A[x][kz][y]   (z, r2c)
//   pass B  A[x][kz][y]                        ->  B[kz][ky][x]  (y)
//   pass C  B[kz][ky][x] -> x transform, then binned in place (ps_bin.cu)
//
// Pass A fuses the fixed-point -> FP32 conversion and subtracts the mean
// cell value: only the k = 0 mode changes, and the periodic-box estimator
// never uses it (src/multipole.c:806), while FP32 round-off of every other
// mode scales with the norm of the input.
#include "ps_internal.h"

namespace ps {
namespace {

__device__ __forceinline__ int odd_stride(int n) { return (n & 1) ? n : n + 1; }

__global__ void __launch_bounds__(kFftThreads) k_pass_a(const __grid_constant__ PassAArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, M = ng >> 1, ngk = M + 1;
  const int ls = odd_stride(M + 1);
  const int nty = (ng + a.ty - 1) / a.ty;
  const int x = blockIdx.x / nty;
  const int y0 = (blockIdx.x - x * nty) * a.ty;
  const int nl = min(a.ty, ng - y0);

  if (a.grid) {
    // Mean cell value in fixed point (any constant works: it only moves k = 0).
    const double W = *a.wsum;
    const long long off = __double2ll_rn(W * 4294967296.0 / ((double)ng * ng * ng));
    const long long* base = a.grid + ((size_t)x * ng + y0) * ng;
    for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
      const int r = e / M, m = e - r * M;
      const longlong2 q = __ldcs(reinterpret_cast<const longlong2*>(base + (size_t)r * ng) + m);
      sm[r * ls + m] = make_float2(fix_to_float(q.x - off), fix_to_float(q.y - off));
    }
  } else {
    const float* base = a.fgrid + ((size_t)x * ng + y0) * ng;
    for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
      const int r = e / M, m = e - r * M;
      sm[r * ls + m] = __ldcs(reinterpret_cast<const float2*>(base + (size_t)r * ng) + m);
    }
  }
  __syncthreads();
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
      L[M] = make_float2(z.x - z.y, 0.f);
    } else {
      const float2 A = L[k], B = L[M - k];
      const float2 E = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
      const float2 O = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
      const float2 W = __ldg(&a.tw_full[k]);
      const float2 WO = cmul(W, O);
      // W^(M-k) = -conj(W)
      const float2 W2O = cmul(make_float2(-W.x, W.y), make_float2(O.x, -O.y));
      L[k] = cadd(E, WO);
      L[M - k] = make_float2(E.x + W2O.x, -E.y + W2O.y);
    }
  }
  __syncthreads();

  float2* ob = a.out + (size_t)x * ngk * ng + y0;
  for (int e = threadIdx.x; e < ngk * nl; e += blockDim.x) {
    const int kz = e / nl, r = e - kz * nl;
    ob[(size_t)kz * ng + r] = sm[r * ls + kz];
  }
}

__global__ void __launch_bounds__(kFftThreads) k_pass_b(const __grid_constant__ PassBArgs a) {
  extern __shared__ float2 sm[];
  const int ng = a.ng, ngk = (ng >> 1) + 1;
  const int ls = ng + 1;
  const int ntx = (ng + a.tx - 1) / a.tx;
  const int kz = blockIdx.x / ntx;
  const int x0 = (blockIdx.x - kz * ntx) * a.tx;
  const int nl = min(a.tx, ng - x0);
  const int h = ng >> 1;
  for (int e = threadIdx.x; e < nl * h; e += blockDim.x) {
    const int r = e / h, m = e - r * h;
    const float4 v = __ldcs(reinterpret_cast<const float4*>(
                               a.in + ((size_t)(x0 + r) * ngk + kz) * ng) + m);
    sm[r * ls + 2 * m] = make_float2(v.x, v.y);
    sm[r * ls + 2 * m + 1] = make_float2(v.z, v.w);
  }
  __syncthreads();
  fft_lines(sm, a.plan_full, nl, ls, a.tw_full);
  float2* ob = a.out + (size_t)kz * ng * ng + x0;
  for (int e = threadIdx.x; e < ng * nl; e += blockDim.x) {
    const int ky = e / nl, r = e - ky * nl;
    ob[(size_t)ky * ng + r] = sm[r * ls + ky];
  }
}

}  // namespace

int launch_pass_a(const PassAArgs& a, cudaStream_t s) {
  const int M = a.ng / 2;
  const int ls = ((M + 1) & 1) ? M + 1 : M + 2;
  const size_t smem = (size_t)a.ty * ls * sizeof(float2);
  const int nty = (a.ng + a.ty - 1) / a.ty;
  cudaFuncSetAttribute(k_pass_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_pass_a<<<(unsigned)(a.ng * nty), kFftThreads, smem, s>>>(a);
  return 1;
}

int launch_pass_b(const PassBArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)a.tx * (a.ng + 1) * sizeof(float2);
  const int ntx = (a.ng + a.tx - 1) / a.tx;
  const int ngk = a.ng / 2 + 1;
  cudaFuncSetAttribute(k_pass_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_pass_b<<<(unsigned)(ngk * ntx), kFftThreads, smem, s>>>(a);
  return 1;
}

}  // namespace ps
