// ps_mlp.cu -- the learned alias/window correction: a 6 -> 64 -> 64 -> 64 -> 1
// GELU MLP with BF16 weights and activations on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation), trained on the GPU by a fused
// forward + loss + backward kernel and an Adam kernel.  No counterpart in
// the reference (it extends the window compensation of src/multipole.c:46-100).
//
// The network maps the features of a (k, |mu|) cell of a coarse mesh --
// (k/k_Nyq, (k/k_Nyq)^2, mu^2, scheme/3, interlace, shot/(shot + P_0)) -- to
// y; c = exp(y) multiplies the raw power of every mode of the cell.  Training
// rows come in groups of 16 |mu| cells of one k bin of one coarse
// measurement; a group's corrected multipoles are
//   Pc_l = (2l+1) (sum_j c_j A_jl - B_l),   l = 0, 2, 4
// (A: the cell's raw sums / (norm cnt), B: the shot-noise term) and its loss
// is sum_l ((Pc_l - Pf_l) / sigma)^2 against the fine-mesh label Pf.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "powspec_gpu.h"
#include "ps_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kIn = 6;       // features
constexpr int kK1 = 16;      // padded input width
constexpr int kH = 64;       // hidden width
constexpr int kGroup = 16;   // |mu| cells per group (one warp's 16 rows)
constexpr int kWarps = 8;    // groups per CTA
constexpr int kRows = kGroup * kWarps;  // 128 rows per CTA
constexpr int kGroupF = 8;   // floats per group record: B0 B2 B4 Pf0 Pf2 Pf4 1/sigma^2 mask

// flat FP32 parameter layout
constexpr int oW1 = 0;                 // [16][64] (in, out)
constexpr int ob1 = oW1 + kK1 * kH;    // [64]
constexpr int oW2 = ob1 + kH;          // [64][64]
constexpr int ob2 = oW2 + kH * kH;
constexpr int oW3 = ob2 + kH;
constexpr int ob3 = oW3 + kH * kH;
constexpr int ow4 = ob3 + kH;          // [64]
constexpr int ob4 = ow4 + kH;          // [1]
constexpr int kNParam = ob4 + 1;       // 9473

// BF16 weight images: transposed (out, in) for the forward B operand and
// plain (in, out) for the backward one.
struct BfWeights {
  bf16 w1t[kH * kK1], w1[kK1 * kH];
  bf16 w2t[kH * kH], w2[kH * kH];
  bf16 w3t[kH * kH], w3[kH * kH];
};

__device__ __forceinline__ uint32_t ld32(const bf16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}
__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  __nv_bfloat162 v = __halves2bfloat162(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragment loads (g = lane / 4, t = lane % 4).
// A tile (rows r0.., cols k0..) of a row-major [rows][ld] matrix.
__device__ __forceinline__ void frag_a(const bf16* M, int ld, int r0, int k0, uint32_t (&a)[4]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  a[0] = ld32(M + (r0 + g) * ld + k0 + 2 * t);
  a[1] = ld32(M + (r0 + g + 8) * ld + k0 + 2 * t);
  a[2] = ld32(M + (r0 + g) * ld + k0 + 2 * t + 8);
  a[3] = ld32(M + (r0 + g + 8) * ld + k0 + 2 * t + 8);
}
// A(m, k) = M[k][m] (transposed view of a row-major [K][ld] matrix).
__device__ __forceinline__ void frag_at(const bf16* M, int ld, int m0, int k0, uint32_t (&a)[4]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const int k = k0 + 2 * t;
  a[0] = pack2(M[k * ld + m0 + g], M[(k + 1) * ld + m0 + g]);
  a[1] = pack2(M[k * ld + m0 + g + 8], M[(k + 1) * ld + m0 + g + 8]);
  a[2] = pack2(M[(k + 8) * ld + m0 + g], M[(k + 9) * ld + m0 + g]);
  a[3] = pack2(M[(k + 8) * ld + m0 + g + 8], M[(k + 9) * ld + m0 + g + 8]);
}
// B(k, n) = BT[n][k] (n-major storage).
__device__ __forceinline__ void frag_b(const bf16* BT, int ld, int n0, int k0, uint32_t (&b)[2]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  b[0] = ld32(BT + (n0 + g) * ld + k0 + 2 * t);
  b[1] = ld32(BT + (n0 + g) * ld + k0 + 2 * t + 8);
}
// B(k, n) = M[k][n] (row-major [K][ld] storage).
__device__ __forceinline__ void frag_bk(const bf16* M, int ld, int n0, int k0, uint32_t (&b)[2]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const int k = k0 + 2 * t;
  b[0] = pack2(M[k * ld + n0 + g], M[(k + 1) * ld + n0 + g]);
  b[1] = pack2(M[(k + 8) * ld + n0 + g], M[(k + 9) * ld + n0 + g]);
}

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

struct Smem {
  BfWeights w;
  bf16 x[kRows * kK1];
  bf16 h[3][kRows * kH];   // activations of the three hidden layers
  float z[3][kRows * kH];  // pre-activations
  bf16 dz[kRows * kH];     // gradient w.r.t. the current layer's pre-activation
  float y[kRows];
  float dy[kRows];
  float w4[kH];
  float b[3][kH];
  float b4;
};

// One layer forward for this warp's 16 rows: z = in * W + b, h = gelu(z).
template <int KIN>
__device__ __forceinline__ void layer_fwd(Smem& s, const bf16* in, const bf16* wt, int layer,
                                          int r0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < KIN; k0 += 16) {
    uint32_t a[4];
    frag_a(in, KIN, r0, k0, a);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      uint32_t b[2];
      frag_b(wt, KIN, nt * 8, k0, b);
      mma16816(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int n = nt * 8 + 2 * t;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int row = r0 + g + ((q & 2) ? 8 : 0);
      const int col = n + (q & 1);
      const float zz = acc[nt][q] + s.b[layer][col];
      s.z[layer][row * kH + col] = zz;
      s.h[layer][row * kH + col] = __float2bfloat16(gelu(zz));
    }
  }
}

// Weight gradient of one layer: dW[in][out] += sum_rows act[row][in] dz[row][out],
// all 8 warps share the (KIN/16) x 8 output tiles; FP32 atomics into global.
template <int KIN>
__device__ __forceinline__ void layer_dw(const bf16* act, const bf16* dz, float* gW) {
  const int warp = threadIdx.x >> 5;
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  constexpr int MT = KIN / 16;
  for (int tile = warp; tile < MT * 8; tile += kWarps) {
    const int m0 = (tile / 8) * 16, n0 = (tile % 8) * 8;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k0 = 0; k0 < kRows; k0 += 16) {
      uint32_t a[4], b[2];
      frag_at(act, KIN, m0, k0, a);
      frag_bk(dz, kH, n0, k0, b);
      mma16816(acc, a, b);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int row = m0 + g + ((q & 2) ? 8 : 0), col = n0 + 2 * t + (q & 1);
      atomicAdd(&gW[row * kH + col], acc[q]);
    }
  }
}

// dh_prev = dz * W^T for this warp's rows, then dz_prev = dh_prev * gelu'(z_prev),
// written (BF16) over s.dz after a warp barrier; bias gradients of the previous layer.
__device__ __forceinline__ void layer_bwd_input(Smem& s, const bf16* w, int prev, int r0,
                                                float* gb_prev) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < kH; k0 += 16) {
    uint32_t a[4];
    frag_a(s.dz, kH, r0, k0, a);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      uint32_t b[2];
      frag_b(w, kH, nt * 8, k0, b);  // B(k=out, n=in) = W[in][out]
      mma16816(acc[nt], a, b);
    }
  }
  __syncwarp();
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int n = nt * 8 + 2 * t;
    float bsum[2] = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int row = r0 + g + ((q & 2) ? 8 : 0);
      const int col = n + (q & 1);
      const float d = acc[nt][q] * gelu_grad(s.z[prev][row * kH + col]);
      s.dz[row * kH + col] = __float2bfloat16(d);
      bsum[q & 1] += d;
    }
#pragma unroll
    for (int c = 0; c < 2; c++) {
      float v = bsum[c];
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (g == 0) atomicAdd(&gb_prev[n + c], v);
    }
  }
  __syncwarp();
}

struct TrainArgs {
  const bf16* x;        // [nrows][16]
  const float* a;       // [nrows][3]
  const float* grp;     // [ngroups][8]
  const int* idx;       // [batch] group indices of this step
  int batch;            // groups in this step (multiple of 8)
  const float* params;  // FP32 master
  const BfWeights* bw;  // BF16 images
  float* grad;          // [kNParam], accumulated (already scaled by 1/batch)
  float* loss;          // [1] accumulated
  int train;            // 0: inference (c = exp(y) into out)
  float* out;           // inference output [nrows]
  int nrows;            // inference rows
};

__global__ void __launch_bounds__(256, 1) k_mlp(const __grid_constant__ TrainArgs p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Smem& s = *reinterpret_cast<Smem*>(smraw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // weights, in 16-byte pieces (all loads of a thread in flight at once);
  // inference needs only the forward images (w1t, w2t, w3t)
  {
    static_assert(sizeof(BfWeights) % 16 == 0 && offsetof(BfWeights, w2t) % 16 == 0 &&
                      offsetof(BfWeights, w3t) % 16 == 0 && (kH * kK1 * sizeof(bf16)) % 16 == 0 &&
                      (kH * kH * sizeof(bf16)) % 16 == 0,
                  "16-byte weight pieces");
    auto copy = [&](const bf16* g, bf16* d, int n) {
      const uint4* src = reinterpret_cast<const uint4*>(g);
      uint4* dst = reinterpret_cast<uint4*>(d);
      for (int e = threadIdx.x; e < n * (int)sizeof(bf16) / 16; e += blockDim.x) dst[e] = src[e];
    };
    if (p.train) {
      copy(reinterpret_cast<const bf16*>(p.bw), reinterpret_cast<bf16*>(&s.w),
           (int)(sizeof(BfWeights) / sizeof(bf16)));
    } else {
      copy(p.bw->w1t, s.w.w1t, kH * kK1);
      copy(p.bw->w2t, s.w.w2t, kH * kH);
      copy(p.bw->w3t, s.w.w3t, kH * kH);
    }
    for (int e = threadIdx.x; e < kH; e += blockDim.x) {
      s.w4[e] = p.params[ow4 + e];
      s.b[0][e] = p.params[ob1 + e];
      s.b[1][e] = p.params[ob2 + e];
      s.b[2][e] = p.params[ob3 + e];
    }
    if (threadIdx.x == 0) s.b4 = p.params[ob4];
  }
  // rows: training -> the 8 groups of this CTA; inference -> 128 consecutive rows
  const int r0 = warp * kGroup;
  int grow = -1;  // global row of (r0 + lane) for lanes < 16
  if (p.train) {
    const int gi = blockIdx.x * kWarps + warp;
    if (gi < p.batch && lane < kGroup) grow = p.idx[gi] * kGroup + lane;
  } else {
    const int row = blockIdx.x * kRows + r0 + lane;
    if (lane < kGroup && row < p.nrows) grow = row;
  }
  for (int e = lane; e < kGroup * kK1; e += 32) {
    const int rl = e / kK1, c = e % kK1;
    const int gr = __shfl_sync(0xffffffffu, grow, rl);
    s.x[(r0 + rl) * kK1 + c] = (gr >= 0) ? p.x[(size_t)gr * kK1 + c] : __float2bfloat16(0.f);
  }
  __syncthreads();

  layer_fwd<kK1>(s, s.x, s.w.w1t, 0, r0);
  __syncwarp();
  layer_fwd<kH>(s, s.h[0], s.w.w2t, 1, r0);
  __syncwarp();
  layer_fwd<kH>(s, s.h[1], s.w.w3t, 2, r0);
  __syncwarp();
  // output layer (FP32 dot of the BF16 activations)
  if (lane < kGroup) {
    const int row = r0 + lane;
    float y = s.b4;
#pragma unroll 8
    for (int n = 0; n < kH; n++) y += __bfloat162float(s.h[2][row * kH + n]) * s.w4[n];
    s.y[row] = y;
  }
  __syncwarp();
  if (!p.train) {
    if (lane < kGroup && grow >= 0) p.out[grow] = __expf(s.y[r0 + lane]);
    return;
  }

  // ---- loss of this warp's group and dL/dy
  {
    const int gi = blockIdx.x * kWarps + warp;
    const bool valid = gi < p.batch;
    const int G = valid ? p.idx[gi] : 0;
    float ca[3] = {0.f, 0.f, 0.f}, c = 0.f, av[3] = {0.f, 0.f, 0.f};
    if (valid && lane < kGroup) {
      c = __expf(s.y[r0 + lane]);
#pragma unroll
      for (int l = 0; l < 3; l++) {
        av[l] = p.a[(size_t)grow * 3 + l];
        ca[l] = c * av[l];
      }
    }
#pragma unroll
    for (int l = 0; l < 3; l++)
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) ca[l] += __shfl_xor_sync(0xffffffffu, ca[l], o);
    float dy = 0.f;
    if (valid) {
      const float* gr = p.grp + (size_t)G * kGroupF;
      const float inv = gr[6] * gr[7] / (float)p.batch;
      float lsum = 0.f;
#pragma unroll
      for (int l = 0; l < 3; l++) {
        const float f = (float)(4 * l + 1);
        const float r = f * (ca[l] - gr[l]) - gr[3 + l];
        lsum += r * r * inv;
        dy += 2.f * r * inv * f * av[l] * c;
      }
      if (lane == 0) atomicAdd(p.loss, lsum);
    }
    if (lane < kGroup) s.dy[r0 + lane] = dy;
  }
  __syncwarp();

  // ---- backward
  {
    const int g = (lane >> 2), t = lane & 3;
    // dz3 = dy * w4 * gelu'(z3); db3; dw4; db4
    for (int e = lane; e < kGroup * kH; e += 32) {
      const int rl = e / kH, col = e % kH, row = r0 + rl;
      const float d = s.dy[row] * s.w4[col] * gelu_grad(s.z[2][row * kH + col]);
      s.dz[row * kH + col] = __float2bfloat16(d);
    }
    (void)g;
    (void)t;
    if (lane < kH / 2) {
      for (int c2 = 0; c2 < 2; c2++) {
        const int col = lane * 2 + c2;
        float db = 0.f, dw = 0.f;
        for (int rl = 0; rl < kGroup; rl++) {
          const int row = r0 + rl;
          db += s.dy[row] * s.w4[col] * gelu_grad(s.z[2][row * kH + col]);
          dw += __bfloat162float(s.h[2][row * kH + col]) * s.dy[row];
        }
        atomicAdd(&p.grad[ob3 + col], db);
        atomicAdd(&p.grad[ow4 + col], dw);
      }
    }
    if (lane == 0) {
      float d4 = 0.f;
      for (int rl = 0; rl < kGroup; rl++) d4 += s.dy[r0 + rl];
      atomicAdd(&p.grad[ob4], d4);
    }
  }
  __syncthreads();
  layer_dw<kH>(s.h[1], s.dz, p.grad + oW3);  // dW3 = h2^T dz3
  __syncthreads();
  layer_bwd_input(s, s.w.w3, 1, r0, p.grad + ob2);  // dz2
  __syncthreads();
  layer_dw<kH>(s.h[0], s.dz, p.grad + oW2);  // dW2 = h1^T dz2
  __syncthreads();
  layer_bwd_input(s, s.w.w2, 0, r0, p.grad + ob1);  // dz1
  __syncthreads();
  layer_dw<kK1>(s.x, s.dz, p.grad + oW1);  // dW1 = x^T dz1
}

// Adam on the FP32 master parameters, then refresh the BF16 images and clear
// the gradients.  Rows 6..15 of W1 (input padding) stay zero.
__global__ void k_adam(float* params, float* m, float* v, float* grad, BfWeights* bw, float lr,
                       float b1, float b2, float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNParam) return;
  const bool pad = (i < ob1) && ((i / kH) >= kIn);
  float p = params[i];
  if (!pad) {
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    p -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    params[i] = p;
  }
  grad[i] = 0.f;
  const bf16 pb = __float2bfloat16(p);
  if (i < ob1) {
    const int in = i / kH, out = i % kH;
    bw->w1[in * kH + out] = pb;
    bw->w1t[out * kK1 + in] = pb;
  } else if (i >= oW2 && i < ob2) {
    const int in = (i - oW2) / kH, out = (i - oW2) % kH;
    bw->w2[in * kH + out] = pb;
    bw->w2t[out * kH + in] = pb;
  } else if (i >= oW3 && i < ob3) {
    const int in = (i - oW3) / kH, out = (i - oW3) % kH;
    bw->w3[in * kH + out] = pb;
    bw->w3t[out * kH + in] = pb;
  }
}

// Inference only (the learned evaluation's c = exp(y) per cell): 4 warps
// of 16 rows per CTA, the forward weight images and two activation buffers
// in 35 KB of shared memory (no pre-activations kept), so many CTAs share
// an SM; the same arithmetic as k_mlp's forward.
constexpr int kInfWarps = 4;
struct SmemInf {
  bf16 w1t[kH * kK1], w2t[kH * kH], w3t[kH * kH];
  bf16 x[kInfWarps * kGroup * kK1];
  bf16 h[2][kInfWarps * kGroup * kH];
  float w4[kH];
  float b[3][kH];
  float b4;
};
template <int KIN>
__device__ __forceinline__ void layer_fwd_inf(const bf16* in, const bf16* wt, const float* bias,
                                              bf16* out, int r0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  float acc[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < KIN; k0 += 16) {
    uint32_t a[4];
    frag_a(in, KIN, r0, k0, a);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      uint32_t b[2];
      frag_b(wt, KIN, nt * 8, k0, b);
      mma16816(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int n = nt * 8 + 2 * t;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int row = r0 + g + ((q & 2) ? 8 : 0);
      const int col = n + (q & 1);
      out[row * kH + col] = __float2bfloat16(gelu(acc[nt][q] + bias[col]));
    }
  }
}
__global__ void __launch_bounds__(32 * kInfWarps) k_mlp_infer(const __grid_constant__ TrainArgs p) {
  __shared__ __align__(16) SmemInf s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto copy = [&](const bf16* g, bf16* d, int n) {
    const uint4* src = reinterpret_cast<const uint4*>(g);
    uint4* dst = reinterpret_cast<uint4*>(d);
    for (int e = threadIdx.x; e < n * (int)sizeof(bf16) / 16; e += blockDim.x) dst[e] = src[e];
  };
  copy(p.bw->w1t, s.w1t, kH * kK1);
  copy(p.bw->w2t, s.w2t, kH * kH);
  copy(p.bw->w3t, s.w3t, kH * kH);
  for (int e = threadIdx.x; e < kH; e += blockDim.x) {
    s.w4[e] = p.params[ow4 + e];
    s.b[0][e] = p.params[ob1 + e];
    s.b[1][e] = p.params[ob2 + e];
    s.b[2][e] = p.params[ob3 + e];
  }
  if (threadIdx.x == 0) s.b4 = p.params[ob4];
  const int r0 = warp * kGroup;
  const int row0 = blockIdx.x * (kInfWarps * kGroup) + r0;
  for (int e = lane; e < kGroup * kK1; e += 32) {
    const int rl = e / kK1, c = e % kK1;
    const int gr = row0 + rl;
    s.x[(r0 + rl) * kK1 + c] = (gr < p.nrows) ? p.x[(size_t)gr * kK1 + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  layer_fwd_inf<kK1>(s.x, s.w1t, s.b[0], s.h[0], r0);
  __syncwarp();
  layer_fwd_inf<kH>(s.h[0], s.w2t, s.b[1], s.h[1], r0);
  __syncwarp();
  layer_fwd_inf<kH>(s.h[1], s.w3t, s.b[2], s.h[0], r0);
  __syncwarp();
  if (lane < kGroup && row0 + lane < p.nrows) {
    const int row = r0 + lane;
    float y = s.b4;
#pragma unroll 8
    for (int n = 0; n < kH; n++) y += __bfloat162float(s.h[0][row * kH + n]) * s.w4[n];
    p.out[row0 + lane] = __expf(y);
  }
}

__global__ void k_to_bf16(const float* x, bf16* y, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

}  // namespace

struct ps_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr, *d_loss = nullptr;
  BfWeights* d_bw = nullptr;
  bf16* d_x = nullptr;
  float *d_a = nullptr, *d_grp = nullptr;
  int* d_idx = nullptr;
  int ngroups = 0, idx_cap = 0;
  float* d_inf_x = nullptr;   // inference buffers, grown on demand
  bf16* d_inf_xb = nullptr;
  float* d_inf_c = nullptr;
  int inf_cap = 0;
  long long step = 0;
  float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  char err[256] = {0};
};

namespace {

int mfail(ps_mlp* m, int code, const char* msg, cudaError_t e) {
  if (m) snprintf(m->err, sizeof m->err, "%s: %s", msg, cudaGetErrorString(e));
  return code;
}
#define MCU(call)                                                         \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) return mfail(m, PS_GPU_ERR_CUDA, #call, e_);   \
  } while (0)

int refresh_bf16(ps_mlp* m) {
  // zero-lr Adam step: refreshes the BF16 images and clears gradients
  k_adam<<<(kNParam + 255) / 256, 256, 0, m->stream>>>(m->d_params, m->d_m, m->d_v, m->d_grad,
                                                       m->d_bw, 0.f, m->beta1, m->beta2, m->eps,
                                                       1.f, 1.f);
  MCU(cudaGetLastError());
  return 0;
}

int launch_mlp(ps_mlp* m, TrainArgs& a, int grid) {
  const size_t smem = sizeof(Smem);
  MCU(cudaFuncSetAttribute(k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_mlp<<<grid, 256, smem, m->stream>>>(a);
  MCU(cudaGetLastError());
  return 0;
}

// Learned correction of one measurement (one CTA per k bin).  Features
// (k/k_Nyq, (k/k_Nyq)^2, mu^2, scheme/3, interlace, shot ratio) of the
// (k, |mu|) cells from the raw sums: A_jl = sums_l / (norm cnt), shot ratio
// = clip(shot / sum_j A_j0, 0, 1), with norm = W^2 / V, shot = V / W
// (src/genr_mesh.c:904-910); the FP64 values are rounded to FP32 as the
// host feature builder does.
__global__ void k_learned_features(const ps::LearnedArgs a) {
  const int b = blockIdx.x;
  __shared__ double s_a0[64];
  __shared__ double s_ratio;
  const double W = a.wsum[0], norm = W * W / a.volume, shot = a.volume / W;
  const double cb = a.cnt[b], safe = fmax(cb, 1.0);
  for (int j = threadIdx.x; j < a.nmu; j += blockDim.x)
    s_a0[j] = (cb > 0) ? a.sums[(size_t)b * a.nmu + j] / (norm * safe) : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double raw0 = 0.0;  // in j order
    for (int j = 0; j < a.nmu; j++) raw0 += s_a0[j];
    s_ratio = fmin(fmax(shot / fmax(raw0, 1e-30), 0.0), 1.0);
  }
  __syncthreads();
  const double q = a.kcen[b] / a.kny;
  // the rows as the network reads them: FP32 features rounded to BF16
  for (int j = threadIdx.x; j < a.nmu; j += blockDim.x) {
    const double mu = (j + 0.5) / a.nmu;
    bf16* xr = reinterpret_cast<bf16*>(a.xb) + ((size_t)b * a.nmu + j) * kK1;
    xr[0] = __float2bfloat16((float)q);
    xr[1] = __float2bfloat16((float)(q * q));
    xr[2] = __float2bfloat16((float)(mu * mu));
    xr[3] = __float2bfloat16(a.assign3);
    xr[4] = __float2bfloat16(a.interlace);
    xr[5] = __float2bfloat16((float)s_ratio);
#pragma unroll
    for (int k = kIn; k < kK1; k++) xr[k] = __float2bfloat16(0.f);
  }
}

// P_l = (2l + 1) (sum_j c_j A_jl - shot lcnt_l / cnt), l = 0, 2, 4, the
// cells summed in j order.
// One thread per (pole, bin): the per-cell sums times the corrections in
// FP64, then one division by the bin's normalisation (FP64 division is slow
// on this GPU: one per pole and bin, not per cell).
__global__ void k_learned_combine(const ps::LearnedArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.npole * a.nbin) return;
  const int l = e / a.nbin, b = e - l * a.nbin;
  const double W = a.wsum[0], norm = W * W / a.volume, shot = a.volume / W;
  const double cb = a.cnt[b], safe = fmax(cb, 1.0);
  const int nkey = a.nbin * a.nmu;
  double s = 0.0, B = 0.0;
  if (cb > 0) {
    const float* c = a.c + (size_t)b * a.nmu;
    const double* sm = a.sums + (size_t)l * nkey + (size_t)b * a.nmu;
    for (int j = 0; j < a.nmu; j++) s = fma((double)c[j], sm[j], s);
    s /= norm * safe;
    B = shot * a.lcnt[(size_t)l * a.nbin + b] / safe;
  }
  a.out[(size_t)l * a.nbin + b] = (4.0 * l + 1.0) * (s - B);
}

}  // namespace

namespace ps {

int learned_feature_width() { return kK1; }

// Features, network and combination on stream s (the caller's context
// stream); the network's weights are only read.
int learned_enqueue(::ps_mlp* m, const LearnedArgs& a, cudaStream_t s) {
  if (!m || a.nmu < 1 || a.nmu > 64 || a.npole != 3) return PS_GPU_ERR_ARG;
  const int n = a.nbin * a.nmu;
  k_learned_features<<<a.nbin, 64, 0, s>>>(a);
  TrainArgs t{};
  t.x = (bf16*)a.xb;
  t.params = m->d_params;
  t.bw = m->d_bw;
  t.train = 0;
  t.out = a.c;
  t.nrows = n;
  k_mlp_infer<<<(n + kInfWarps * kGroup - 1) / (kInfWarps * kGroup), 32 * kInfWarps, 0, s>>>(t);
  k_learned_combine<<<(a.npole * a.nbin + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : PS_GPU_ERR_CUDA;
}

}  // namespace ps

extern "C" {

int ps_mlp_nparam(void) { return kNParam; }

int ps_mlp_create(int device, ps_mlp** out) {
  if (!out) return PS_GPU_ERR_ARG;
  ps_mlp* m = new (std::nothrow) ps_mlp();
  if (!m) return PS_GPU_ERR_MEMORY;
  *out = m;
  m->device = device;
  ps::DeviceScope dev_scope_(device);
  MCU(dev_scope_.err);
  MCU(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  MCU(cudaMalloc(&m->d_params, kNParam * sizeof(float)));
  MCU(cudaMalloc(&m->d_m, kNParam * sizeof(float)));
  MCU(cudaMalloc(&m->d_v, kNParam * sizeof(float)));
  MCU(cudaMalloc(&m->d_grad, kNParam * sizeof(float)));
  MCU(cudaMalloc(&m->d_loss, sizeof(float)));
  MCU(cudaMalloc(&m->d_bw, sizeof(BfWeights)));
  MCU(cudaMemset(m->d_params, 0, kNParam * sizeof(float)));
  MCU(cudaMemset(m->d_m, 0, kNParam * sizeof(float)));
  MCU(cudaMemset(m->d_v, 0, kNParam * sizeof(float)));
  MCU(cudaMemset(m->d_grad, 0, kNParam * sizeof(float)));
  MCU(cudaMemset(m->d_bw, 0, sizeof(BfWeights)));
  return refresh_bf16(m);
}

void ps_mlp_destroy(ps_mlp* m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* bufs[] = {m->d_params, m->d_m, m->d_v, m->d_grad, m->d_loss, m->d_bw,
                  m->d_x, m->d_a, m->d_grp, m->d_idx, m->d_inf_x, m->d_inf_xb, m->d_inf_c};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

const char* ps_mlp_last_error(const ps_mlp* m) { return m ? m->err : "null"; }

int ps_mlp_set_params(ps_mlp* m, const float* params) {
  if (!m || !params) return PS_GPU_ERR_ARG;
  MCU(cudaMemcpyAsync(m->d_params, params, kNParam * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  int rc = refresh_bf16(m);
  if (rc) return rc;
  MCU(cudaStreamSynchronize(m->stream));
  return 0;
}

int ps_mlp_get_params(ps_mlp* m, float* params) {
  if (!m || !params) return PS_GPU_ERR_ARG;
  MCU(cudaMemcpyAsync(params, m->d_params, kNParam * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCU(cudaStreamSynchronize(m->stream));
  return 0;
}

int ps_mlp_set_data(ps_mlp* m, const float* x, const float* a, const float* grp, int ngroups) {
  if (!m || !x || !a || !grp || ngroups < 1) return PS_GPU_ERR_ARG;
  const size_t nrows = (size_t)ngroups * kGroup;
  if (m->d_x) cudaFree(m->d_x);
  if (m->d_a) cudaFree(m->d_a);
  if (m->d_grp) cudaFree(m->d_grp);
  m->d_x = nullptr;
  m->d_a = nullptr;
  m->d_grp = nullptr;
  std::vector<float> xp(nrows * kK1, 0.f);
  for (size_t r = 0; r < nrows; r++)
    for (int c = 0; c < kIn; c++) xp[r * kK1 + c] = x[r * kIn + c];
  float* d_xf = nullptr;
  MCU(cudaMalloc(&d_xf, xp.size() * sizeof(float)));
  MCU(cudaMalloc(&m->d_x, xp.size() * sizeof(bf16)));
  MCU(cudaMalloc(&m->d_a, nrows * 3 * sizeof(float)));
  MCU(cudaMalloc(&m->d_grp, (size_t)ngroups * kGroupF * sizeof(float)));
  MCU(cudaMemcpy(d_xf, xp.data(), xp.size() * sizeof(float), cudaMemcpyHostToDevice));
  k_to_bf16<<<(unsigned)((xp.size() + 255) / 256), 256, 0, m->stream>>>(d_xf, m->d_x, xp.size());
  MCU(cudaGetLastError());
  MCU(cudaMemcpy(m->d_a, a, nrows * 3 * sizeof(float), cudaMemcpyHostToDevice));
  MCU(cudaMemcpy(m->d_grp, grp, (size_t)ngroups * kGroupF * sizeof(float), cudaMemcpyHostToDevice));
  MCU(cudaStreamSynchronize(m->stream));
  cudaFree(d_xf);
  m->ngroups = ngroups;
  return 0;
}

// Gradient (and loss) of one batch of groups at the current parameters, no update.
int ps_mlp_grad(ps_mlp* m, const int* idx, int batch, float* grad, float* loss) {
  if (!m || !idx || batch < 1 || !m->d_x) return PS_GPU_ERR_ARG;
  for (int i = 0; i < batch; i++)
    if (idx[i] < 0 || idx[i] >= m->ngroups) return PS_GPU_ERR_ARG;
  if (batch > m->idx_cap) {
    if (m->d_idx) cudaFree(m->d_idx);
    MCU(cudaMalloc(&m->d_idx, (size_t)batch * sizeof(int)));
    m->idx_cap = batch;
  }
  MCU(cudaMemcpyAsync(m->d_idx, idx, (size_t)batch * sizeof(int), cudaMemcpyHostToDevice, m->stream));
  MCU(cudaMemsetAsync(m->d_grad, 0, kNParam * sizeof(float), m->stream));
  MCU(cudaMemsetAsync(m->d_loss, 0, sizeof(float), m->stream));
  TrainArgs a{};
  a.x = m->d_x;
  a.a = m->d_a;
  a.grp = m->d_grp;
  a.idx = m->d_idx;
  a.batch = batch;
  a.params = m->d_params;
  a.bw = m->d_bw;
  a.grad = m->d_grad;
  a.loss = m->d_loss;
  a.train = 1;
  int rc = launch_mlp(m, a, (batch + kWarps - 1) / kWarps);
  if (rc) return rc;
  if (grad) MCU(cudaMemcpyAsync(grad, m->d_grad, kNParam * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  if (loss) MCU(cudaMemcpyAsync(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCU(cudaStreamSynchronize(m->stream));
  return refresh_bf16(m);
}

// nsteps Adam steps; step s uses groups idx[s * batch .. (s + 1) * batch).
// loss[s] receives each step's loss (may be NULL).
int ps_mlp_train(ps_mlp* m, const int* idx, int nsteps, int batch, float lr, float* loss) {
  if (!m || !idx || batch < 1 || nsteps < 1 || !m->d_x) return PS_GPU_ERR_ARG;
  const size_t n = (size_t)nsteps * batch;
  for (size_t i = 0; i < n; i++)
    if (idx[i] < 0 || idx[i] >= m->ngroups) return PS_GPU_ERR_ARG;
  if ((int)n > m->idx_cap) {
    if (m->d_idx) cudaFree(m->d_idx);
    MCU(cudaMalloc(&m->d_idx, n * sizeof(int)));
    m->idx_cap = (int)n;
  }
  float* d_losses = nullptr;
  MCU(cudaMalloc(&d_losses, (size_t)nsteps * sizeof(float)));
  MCU(cudaMemsetAsync(d_losses, 0, (size_t)nsteps * sizeof(float), m->stream));
  MCU(cudaMemcpyAsync(m->d_idx, idx, n * sizeof(int), cudaMemcpyHostToDevice, m->stream));
  MCU(cudaMemsetAsync(m->d_grad, 0, kNParam * sizeof(float), m->stream));
  const size_t smem = sizeof(Smem);
  MCU(cudaFuncSetAttribute(k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (int s = 0; s < nsteps; s++) {
    TrainArgs a{};
    a.x = m->d_x;
    a.a = m->d_a;
    a.grp = m->d_grp;
    a.idx = m->d_idx + (size_t)s * batch;
    a.batch = batch;
    a.params = m->d_params;
    a.bw = m->d_bw;
    a.grad = m->d_grad;
    a.loss = d_losses + s;
    a.train = 1;
    k_mlp<<<(batch + kWarps - 1) / kWarps, 256, smem, m->stream>>>(a);
    m->step++;
    const float bc1 = 1.f - powf(m->beta1, (float)m->step);
    const float bc2 = 1.f - powf(m->beta2, (float)m->step);
    k_adam<<<(kNParam + 255) / 256, 256, 0, m->stream>>>(m->d_params, m->d_m, m->d_v, m->d_grad,
                                                         m->d_bw, lr, m->beta1, m->beta2, m->eps,
                                                         bc1, bc2);
  }
  MCU(cudaGetLastError());
  if (loss) MCU(cudaMemcpyAsync(loss, d_losses, (size_t)nsteps * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCU(cudaStreamSynchronize(m->stream));
  cudaFree(d_losses);
  return 0;
}

// c = exp(y) for n feature rows x[n][6] (host memory).
int ps_mlp_infer(ps_mlp* m, const float* x, int n, float* c) {
  if (!m || !x || !c || n < 1) return PS_GPU_ERR_ARG;
  if (n > m->inf_cap) {
    if (m->d_inf_x) cudaFree(m->d_inf_x);
    if (m->d_inf_xb) cudaFree(m->d_inf_xb);
    if (m->d_inf_c) cudaFree(m->d_inf_c);
    m->d_inf_x = nullptr;
    m->d_inf_xb = nullptr;
    m->d_inf_c = nullptr;
    m->inf_cap = 0;
    MCU(cudaMalloc(&m->d_inf_x, (size_t)n * kK1 * sizeof(float)));
    MCU(cudaMalloc(&m->d_inf_xb, (size_t)n * kK1 * sizeof(bf16)));
    MCU(cudaMalloc(&m->d_inf_c, (size_t)n * sizeof(float)));
    m->inf_cap = n;
  }
  // features padded to 16 on the device: copy rows of 6 into a zeroed buffer
  MCU(cudaMemsetAsync(m->d_inf_x, 0, (size_t)n * kK1 * sizeof(float), m->stream));
  MCU(cudaMemcpy2DAsync(m->d_inf_x, kK1 * sizeof(float), x, kIn * sizeof(float), kIn * sizeof(float),
                        (size_t)n, cudaMemcpyHostToDevice, m->stream));
  k_to_bf16<<<(unsigned)(((size_t)n * kK1 + 255) / 256), 256, 0, m->stream>>>(m->d_inf_x, m->d_inf_xb,
                                                                              (size_t)n * kK1);
  TrainArgs a{};
  a.x = m->d_inf_xb;
  a.params = m->d_params;
  a.bw = m->d_bw;
  a.train = 0;
  a.out = m->d_inf_c;
  a.nrows = n;
  k_mlp_infer<<<(n + kInfWarps * kGroup - 1) / (kInfWarps * kGroup), 32 * kInfWarps, 0, m->stream>>>(a);
  MCU(cudaGetLastError());
  MCU(cudaMemcpyAsync(c, m->d_inf_c, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCU(cudaStreamSynchronize(m->stream));
  return 0;
}

// Checkpoint: parameters, Adam moments and the step counter (resume-able).
int ps_mlp_save(ps_mlp* m, const char* path) {
  if (!m || !path) return PS_GPU_ERR_ARG;
  std::vector<float> buf(3 * (size_t)kNParam);
  MCU(cudaMemcpy(buf.data(), m->d_params, kNParam * sizeof(float), cudaMemcpyDeviceToHost));
  MCU(cudaMemcpy(buf.data() + kNParam, m->d_m, kNParam * sizeof(float), cudaMemcpyDeviceToHost));
  MCU(cudaMemcpy(buf.data() + 2 * kNParam, m->d_v, kNParam * sizeof(float), cudaMemcpyDeviceToHost));
  FILE* f = fopen(path, "wb");
  if (!f) return PS_GPU_ERR_ARG;
  const char magic[8] = {'P', 'S', 'M', 'L', 'P', '0', '0', '1'};
  const int np = kNParam;
  bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(&np, sizeof np, 1, f) == 1 &&
            fwrite(&m->step, sizeof m->step, 1, f) == 1 &&
            fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  fclose(f);
  return ok ? 0 : PS_GPU_ERR_ARG;
}

int ps_mlp_load(ps_mlp* m, const char* path) {
  if (!m || !path) return PS_GPU_ERR_ARG;
  FILE* f = fopen(path, "rb");
  if (!f) return PS_GPU_ERR_ARG;
  char magic[8];
  int np = 0;
  long long step = 0;
  std::vector<float> buf(3 * (size_t)kNParam);
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "PSMLP001", 8) == 0 &&
            fread(&np, sizeof np, 1, f) == 1 && np == kNParam &&
            fread(&step, sizeof step, 1, f) == 1 &&
            fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  fclose(f);
  if (!ok) return PS_GPU_ERR_ARG;
  MCU(cudaMemcpy(m->d_params, buf.data(), kNParam * sizeof(float), cudaMemcpyHostToDevice));
  MCU(cudaMemcpy(m->d_m, buf.data() + kNParam, kNParam * sizeof(float), cudaMemcpyHostToDevice));
  MCU(cudaMemcpy(m->d_v, buf.data() + 2 * kNParam, kNParam * sizeof(float), cudaMemcpyHostToDevice));
  m->step = step;
  int rc = refresh_bf16(m);
  if (rc) return rc;
  MCU(cudaStreamSynchronize(m->stream));
  return 0;
}

}  // extern "C"
