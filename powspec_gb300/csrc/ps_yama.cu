// ps_yama.cu -- survey multipoles l > 0 by the spherical-harmonic
// decomposition of the Legendre polynomial (Hand et al. 2017; the
// reference's src/mp_template.c:48-149):
//   F_l(k) = sum_m Y_lm(k^) FFT[ F(r) Y_lm(r^) ](k),
//   P_l ~ sum_k Re[F_0(k) F_l(k)*],
// with F the data - alpha x randoms mesh and r^ the direction from the
// observer (the coordinate origin).  Any orthonormal real basis of the
// degree-l harmonics gives the same sum over m (the addition theorem,
// sum_m Y_lm(a) Y_lm(b) = (2l + 1) / (4 pi) L_l(a . b)); the one here is
// Y_l0 = K_l0 P_l(cos t), Y_lm = sqrt(2) K_lm P_l^m(cos t) cos(m p),
// Y_l,-m = sqrt(2) K_lm P_l^m(cos t) sin(m p), K_lm^2 = (2l + 1) / (4 pi)
// (l - m)! / (l + m)!, with P_l^m by the standard recurrences.
//
// Two conventions of the reference are kept: the first mesh row
// (i = j = 0) and the modes on the k_z axis (k_x = k_y = 0) take the
// harmonic as 1 for every m (src/mp_template.c:71-74, :118-121).
#include "ps_internal.h"

namespace ps {
namespace {

// Y_lm of the direction (x, y, z) (need not be normalised); l <= 6.
__device__ __forceinline__ float ylm(int l, int m, float kl, float x, float y, float z) {
  const float rxy2 = x * x + y * y, r = sqrtf(rxy2 + z * z);
  const float ct = z / r, st = sqrtf(rxy2) / r;
  const int am = abs(m);
  // P_am^am = (2 am - 1)!! st^am, then up to P_l^am (Condon-Shortley sign
  // dropped: the sum over m does not depend on it)
  float pmm = 1.f;
  for (int i = 1; i <= am; i++) pmm *= (2 * i - 1) * st;
  float p = pmm;
  if (l > am) {
    float p1 = ct * (2 * am + 1) * pmm, p0 = pmm;
    p = p1;
    for (int ll = am + 2; ll <= l; ll++) {
      p = ((2 * ll - 1) * ct * p1 - (ll + am - 1) * p0) / (ll - am);
      p0 = p1;
      p1 = p;
    }
  }
  if (m == 0) return kl * p;
  // cos(am phi), sin(am phi) from cos phi = x / rxy, sin phi = y / rxy
  const float ri = rsqrtf(rxy2), cp = x * ri, sp = y * ri;
  float c = 1.f, s = 0.f;
  for (int i = 0; i < am; i++) {
    const float c2 = c * cp - s * sp;
    s = s * cp + c * sp;
    c = c2;
  }
  return kl * p * (m > 0 ? c : s);
}

// out = in * Y_lm(r^) over the real mesh [x][y][z]; cell (i, j, k) sits at
// (i + o0, j + o1, k + o2) cells from the observer, o = box corner * Ng / L,
// and directions are taken as cells * L (src/mp_template.c:60-70).
__global__ void k_ylm_real(const float* __restrict__ in, float* __restrict__ out, int ng, int l,
                           int m, float kl, float o0, float o1, float o2, float L0, float L1,
                           float L2) {
  const size_t n = (size_t)ng * ng * ng;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % ng);
    const size_t row = e / ng;
    const int j = (int)(row % ng), i = (int)(row / ng);
    float y = 1.f;
    if (row != 0) y = ylm(l, m, kl, (i + o0) * L0, (j + o1) * L1, (k + o2) * L2);
    out[e] = in[e] * y;
  }
}

// acc (+)= f * Y_lm(k^) over the stored half-complex field [x][y][z/2+1];
// k = (signed i / L0, signed j / L1, k / L2).
__global__ void k_ylm_acc(const float2* __restrict__ f, float2* __restrict__ acc, int ng, int l,
                          int m, float kl, float iL0, float iL1, float iL2, int first) {
  const int ngk = ng / 2 + 1;
  const size_t n = (size_t)ng * ng * ngk;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % ngk);
    const size_t row = e / ngk;
    const int j = (int)(row % ng), i = (int)(row / ng);
    const int ip = (2 * i <= ng) ? i : i - ng, jp = (2 * j <= ng) ? j : j - ng;
    float y = 1.f;
    if (ip != 0 || jp != 0) y = ylm(l, m, kl, ip * iL0, jp * iL1, k * iL2);
    const float2 v = f[e];
    float2 a = first ? make_float2(0.f, 0.f) : acc[e];
    a.x += v.x * y;
    a.y += v.y * y;
    acc[e] = a;
  }
}

}  // namespace

int launch_ylm_real(const float* in, float* out, int ng, int l, int m, double kl,
                    const double origin[3], const double box[3], cudaStream_t s) {
  const size_t n = (size_t)ng * ng * ng;
  const unsigned blocks = (unsigned)((n + 255) / 256 < 152 * 32 ? (n + 255) / 256 : 152 * 32);
  k_ylm_real<<<blocks, 256, 0, s>>>(in, out, ng, l, m, (float)kl, (float)(origin[0] * ng / box[0]),
                                     (float)(origin[1] * ng / box[1]),
                                     (float)(origin[2] * ng / box[2]), (float)box[0],
                                     (float)box[1], (float)box[2]);
  return 1;
}

int launch_ylm_acc(const float2* f, float2* acc, int ng, int l, int m, double kl,
                   const double box[3], bool first, cudaStream_t s) {
  const size_t n = (size_t)ng * ng * (ng / 2 + 1);
  const unsigned blocks = (unsigned)((n + 255) / 256 < 152 * 32 ? (n + 255) / 256 : 152 * 32);
  k_ylm_acc<<<blocks, 256, 0, s>>>(f, acc, ng, l, m, (float)kl, (float)(1.0 / box[0]),
                                    (float)(1.0 / box[1]), (float)(1.0 / box[2]), first ? 1 : 0);
  return 1;
}

}  // namespace ps
