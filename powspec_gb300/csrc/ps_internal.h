// ps_internal.h -- launch wrappers shared by the translation units of
// libpowspec_gpu.so.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "powspec_gpu.h"
#include "powspec_learned.h"
#include "ps_common.cuh"

namespace ps {

// Particle source for the assignment kernels.
struct Particles {
  const double* aos;  // {x, y, z, w} records, or NULL
  const float* x;     // SoA arrays when aos == NULL
  const float* y;
  const float* z;
  const float* w;     // NULL: unit weights
  size_t n;
};

constexpr int kAssignMaxBlocks = 2048;  // per-block weight partials

// Tile assignment (ps_gather.cu).
struct GatherArgs {
  int ng, assign, interlace;
  int T, nt;               // tile edge (cells) and tiles per axis
  int tshift;              // log2 T when T is a power of two, else -1
  double box[3];
  double bmin[3], bmax[3]; // shifted grid's edges: -(L / 2) / Ng and that + L (FP64)
  float s_hi[3], s_lo[3];  // Ng / L as a double-float pair per axis
  long long box_bits[3];   // bit pattern of L (AoS FP64 bound check)
  float box_f[3];          // smallest float >= L (SoA FP32 bound check)
  unsigned* hist;          // [nkeys + 1] counts, then offsets
  unsigned* bsum;          // [ceil(nkeys / 4096) + 1]
  unsigned* rank;          // [n]
  void* rec;               // [n] records, gather_record_bytes() each
  float* out[2];           // FP32 meshes minus the mean cell value
  long long* out64[2];     // or exact fixed-point meshes (diagnostics)
  double* wsum;            // [2]
  long long* moff;         // mean cell value in fixed point (0 with nomean), set by k_wsum
  double* wpart;           // [2 * kAssignMaxBlocks]: per block (sum w as an FP32 pair, sum |w|, 0)
  double moff_scale;       // 2^32 / Ng^3: the mean cell value in fixed point per unit of W
  int* err;                // bit 0: particle outside [0, L); bit 1: region index out of range
  int threads;             // CTA size of the gather: 256, 512 or 0 (by density)
  unsigned sparse_max;     // tiles with at most this many records: lane groups, rows flagged;
                           // more: one record per warp (TSC/PCS)
  int region;              // 1: each record once, into its home tile's region (TSC/PCS, T = 16)
  unsigned long long* regbuf;  // [tiles][gather_region_words()][meshes] region sums
  int reg_f32;                 // 1: regions as FP32 words (home cells minus the mean);
                               // 0: exact int64 words (int64 meshes, survey meshes)
  unsigned char* regflag;      // [tiles] 1: the tile wrote its region (it has records)
  int nomean;                  // 1: FP32 meshes keep their mean (survey catalogues)
};
// Learned correction on the device (ps_mlp.cu), after a binning pass with
// |mu| sub-bins: cell features, network, corrected multipoles.
struct LearnedArgs {
  const double* sums;  // [npole][nbin * nmu] raw sums of p L_l (one auto spectrum)
  const double* wsum;  // W at [0]
  const double* kcen;  // [nbin] bin centres
  const double* cnt;   // [nbin] mode counts
  const double* lcnt;  // [npole][nbin] sums of w L_l
  double volume, kny;
  float assign3, interlace;  // features: scheme / 3, 0 or 1
  int nbin, nmu, npole;      // npole 3: l = 0, 2, 4
  float* x;                  // [nbin * nmu][16] feature rows (FP32; not written on the device path)
  void* xb;                  // [nbin * nmu][16] BF16 copy
  float* c;                  // [nbin * nmu] corrections exp(y)
  double* out;               // [npole][nbin] corrected P_l
};
int learned_enqueue(::ps_mlp* m, const LearnedArgs& a, cudaStream_t s);
int learned_feature_width();

// Survey multipoles l > 0 (ps_yama.cu): the coefficients of one harmonic
// (ylm_eval).
YlmCoef ylm_coef(int l, int m);
void ylm_poly(int l, int am, double* q);  // FP64 polynomial of Y_l,+-am in cos(theta)
// F_l(0) into *out (device): sum_r F(r) sum_m Y_lm(r^) of an FP32 mesh
// [ng][ng][ng] in FP64 (harmonics included), through `grid` CTA partials
// in `part` (grid + 1 doubles), when some catalogue's |sum w| exceeds kDcGate
// times its sum |w| (wsum: [ncat][2] on the device); else the FP32
// transform's DC *dc32.  Returns the launches made, or < 0 for l outside 0..6.
constexpr double kDcGate = 1e-4;
int launch_dc_sum(const float* mesh, int ng, int ell, const double* org, const double* len,
                  const double* wsum, int ncat, const float2* dc32, double* part, int grid,
                  double* out, cudaStream_t s);
// The interlaced field's c2r (ps_yama.cu): inverse along the leading axis
// of [l][p][kz] into [p][l][kz] (with in2: over the interlace combination,
// also written back to in), then half-complex z rows -> real rows / Ng^3.
int launch_inv_lead(float2* in, const float2* in2, float2* out, int ng, const float2* phase,
                    const float2* tw_full, const FftPlan& plan_full, cudaStream_t s);
int launch_c2r_z(const float2* in, float* out, int ng, int ty, const float2* tw_half,
                 const float2* tw_full, const FftPlan& plan_half, cudaStream_t s);

int gather_tile(int ng);    // tile edge for this mesh size, 0 if unsupported
// Region path: possible for this mesh and scheme; words per tile and mesh.
bool gather_region_ok(int ng, int T, int assign);
size_t gather_region_words(int assign);
size_t gather_region_smem(int assign, int interlace);  // shared bytes of a region CTA
size_t gather_keys(int ng);  // number of (tile, class) keys
size_t gather_record_bytes();  // bytes per particle record
// int64_out: only the gather step, into out64 (records must be in place).
int launch_gather_assign(const Particles& p, GatherArgs g, cudaStream_t s, bool int64_out);

// z transform: fixed-point grid [x][y][z] -> A[x][kz][y] (complex).
struct PassAArgs {
  int ng;
  int ty;                       // y rows per CTA
  const float* fgrid;           // FP32 input mesh
  float2* out;
  const float2* tw_half;        // length ng/2 twiddles
  const float2* tw_full;        // length ng twiddles (r2c split)
  FftPlan plan_half;
  int pipe_grid;                // > 0: pipelined persistent kernel with this grid
  int radix32;                  // pipelined kernel: radix-32 passes on 8192-value tiles
  const float2* twl;            // non-NULL: the warp transform (ps_wfft.cu), its table
  int* err;                     // bit 1: pipeline wait timed out
  // survey harmonics (yw != 0): cell (i, j, k) of the FP32 input is weighted
  // by Y_lm of ((i, j, k) + org) * len on the way in, 1 on the row i = j = 0
  // (src/mp_template.c:60-74)
  int yw;
  YlmCoef yc;
  float org[3], len[3];
  // test hook (ps_gpu_debug_stall_pipeline): CTA 0 of a pipelined kernel
  // arms its second copy but issues none, and every wait gives up after
  // wait_limit polls (0: the default bound)
  int stall;
  int wait_limit;
};
int launch_pass_a(const PassAArgs& a, cudaStream_t s);

// y transform: A[x][kz][y] -> B[kz][ky][x].
struct PassBArgs {
  int ng;
  int tx;
  const float2* in;
  float2* out;
  const float2* tw_full;
  FftPlan plan_full;
  int pipe_grid;
  int radix32;  // pipelined kernel: radix-32 passes on 8192-value tiles
  const float2* twl;            // non-NULL: the warp transform (ps_wfft.cu), its table
  int* err;
  // test hook (ps_gpu_debug_stall_pipeline): CTA 0 of a pipelined kernel
  // arms its second copy but issues none, and every wait gives up after
  // wait_limit polls (0: the default bound)
  int stall;
  int wait_limit;
};
int launch_pass_b(const PassBArgs& a, cudaStream_t s);

// x transform of B[kz][ky][x] rows, then either stored in the FFTW layout
// [x][y][kz] (store mode) or combined, windowed and binned (bin mode).
struct PassCArgs {
  int ng;
  int ty;
  int nfield;                   // 1, 2 (interlace or 2 catalogues) or 4
  int interlace;
  int ncat;
  int nspec;                    // spectra accumulated: pairs (sa, sb)
  int spec_a[3], spec_b[3];     // catalogue indices of each spectrum
  const float2* in[4];          // field f = cat * (interlace ? 2 : 1) + mesh
  float2* store;                // store mode target (FFTW layout), or NULL
  int acc_mode;                 // store mode: 0 store; 1 store x Y(k^); 2 add x Y(k^)
  YlmCoef yk;                   // acc_mode > 0: the harmonic; 1 on the k_z axis
  float kinv[3];                // 1 / L per axis (wave-vector direction)
  const float2* tw_full;
  FftPlan plan_full;
  ModeGeom geom;
  float2* partials;             // [grid][nspec*npole*nbin] FP32 pairs (hi + lo)
  int grid;                     // persistent CTAs (bin mode)
  int pipe;                     // power-of-two Ng: the cp.async.bulk-pipelined kernel
  int mom;                      // 0: pole sums; 2..4: mu^2 moments (even poles, lmax = 2 (mom - 1))
  const float2* twl;            // bin mode, non-NULL: the warp transform (ps_wfft.cu)
  int wpc;                      // warp x pass: warps per CTA (4, 8 or 16)
  int* err;                     // bit 1: a pipeline wait timed out
  // test hook (ps_gpu_debug_stall_pipeline): CTA 0 of a pipelined kernel
  // arms its second copy but issues none, and every wait gives up after
  // wait_limit polls (0: the default bound)
  int stall;
  int wait_limit;
};
// mu^2 moments the binning pass accumulates for a pole set (0: a Horner sum
// per pole, for sets with odd multipoles), and its FP32 tile accumulators
// per spectrum.
int pass_c_moments(const int* poles, int npole);
inline int pass_c_accs(int npole, int mom) { return mom > 0 ? (mom > npole ? mom : npole) : npole; }
int launch_pass_c(const PassCArgs& a, cudaStream_t s);
// Dynamic shared memory of the pipelined pass C (barriers, 2 stages + FFT
// buffer, tile sums); complex elements of one of its buffers.
size_t pass_c_tma_smem(int ng, int ty, int nfield, int nacc, int nkey);
__host__ __device__ inline size_t pass_c_tma_elems(int ng, int ty, int nfield) {
  return ((size_t)nfield * ty * line_stride(ng, true) + 1) & ~(size_t)1;  // 16-byte multiple
}

// Warp-register transforms (ps_wfft.cu) for power-of-two meshes: pass 0
// (z, Ng = 256..2048), passes 1 and 2 (y, x + binning; Ng = 256..1024).
// Line length n is held as L lanes x V values; the table of a length-n
// transform is twl[k1 L + l] = exp(-2 pi i l k1 / n), n entries.
bool wfft_supported(int ng, int pass);
void wfft_shape(int n, int* L, int* V);
int launch_pass_a_w(const PassAArgs& a, cudaStream_t s);  // 0: shape not supported
int launch_pass_b_w(const PassBArgs& a, cudaStream_t s);
int launch_pass_c_w(const PassCArgs& a, cudaStream_t s);
// Resident CTAs per SM of the warp x pass launch_pass_c_w would run for these
// arguments (ng, nfield, nspec, mom, wpc, geom.npole/nbin/nmu/los), by the
// chosen instance's registers and shared memory; 0 without a warp form.
int pass_c_w_per_sm(const PassCArgs& a);
// The store-mode x pass (one field, survey harmonic terms); 0 without a warp form.
int launch_pass_c_ws(const PassCArgs& a, cudaStream_t s);
// Dynamic shared memory and block size of the warp x pass (persistent CTAs).
size_t pass_c_w_smem(int ng, int nfield, int nacc, int nkey, int wpc);

// Binning of standard-layout half-complex fields [x][y][kz].
struct BinFieldArgs {
  int ng;
  const float2* f1;
  const float2* f2;
  ModeGeom geom;
  float2* partials;             // [grid][npole*nbin] FP32 pairs (hi + lo)
  int grid;
};
int launch_bin_fields(const BinFieldArgs& a, cudaStream_t s);

// Geometry-only sweep: mode counts, sum of |k| and sum of w L_l(mu) per bin
// (FP64), accumulated into cnt[nbin], ksum[nbin], lcnt[npole*nbin].
struct GeomArgs {
  int ng;
  ModeGeom geom;
  double vec[3];
  double los[3];
  unsigned long long* cnt;
  double* ksum;
  double* lcnt;
};
int launch_geometry(const GeomArgs& a, cudaStream_t s);

// Deterministic reduction of per-CTA partials: out[j] = sum_g part[g][j].
int launch_reduce(const float2* part, int grid, int width, double* out, cudaStream_t s);
int launch_reduce_f64(const double* part, int grid, int width, double* out, cudaStream_t s);

// Minimum shared memory per CTA the passes need (bytes).
size_t pass_c_smem(int ng, int ty, int nfield, int nacc, int nbin, bool pow2);

// Makes `dev` the current device for the scope of one entry point and gives
// the caller's current device back on every return path, so that a call on
// a context never changes the device the calling thread works on.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) err = cudaSetDevice(dev);
    else prev = -1;  // already current: nothing to give back
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// Loads the no-allocation entry point's static scratch array on the current
// device (ps_noalloc.cu).
cudaError_t noalloc_prepare(int dev);

// Read-only view of a context for entry points outside ps_capi.cu.
struct CtxView {
  int ng, device;
  ModeGeom geom;  // device tables owned by the context
};
int ctx_view(const ps_gpu_ctx* c, CtxView* v);  // nonzero if c is NULL
// Records the message as the context's last error; returns code.
int ctx_fail(ps_gpu_ctx* c, int code, const char* fmt, ...);

}  // namespace ps
