/*
 * powspec_gpu.h -- C ABI of the GB300 (sm_103a) periodic-box P_l(k) path.
 *
 * Drop-in boundary for powspec's hot path.  The reference computes it in two
 * calls from main (src/powspec.c:47,55):
 *
 *   MESH *genr_mesh(const CONF *conf, CATA *cat);          src/genr_mesh.c:874
 *   PK   *powspec(const CONF *conf, const CATA *cat, MESH *mesh);
 *                                                          src/multipole.c:1179
 *
 * Here the same work is an opaque context driven by plain pointers and sizes:
 * ps_gpu_create (mesh_init + powspec_init + powspec_precomp),
 * ps_gpu_assign_* (one catalogue's part of gen_dens), ps_gpu_execute
 * (dens_k0 + count_mode + normalisation) and ps_gpu_destroy (mesh_destroy +
 * powspec_destroy).  Every entry point returns 0 or a negative status whose
 * values extend the reference's POWSPEC_ERR_* codes (src/define.h:112-124);
 * none of them exits the process.  One context per host thread; each
 * context owns one CUDA stream.  There is no CPU fallback: without a usable
 * GPU every call that needs one fails with PS_GPU_ERR_CUDA.
 */
#ifndef POWSPEC_GPU_H
#define POWSPEC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PS_GPU_ABI_VERSION 1

/* Status codes.  The first block mirrors src/define.h:112-124. */
#define PS_GPU_OK 0
#define PS_GPU_ERR_MEMORY (-1)  /* POWSPEC_ERR_MEMORY: host or device allocation */
#define PS_GPU_ERR_ARG (-2)     /* POWSPEC_ERR_ARG: invalid argument */
#define PS_GPU_ERR_CATA (-11)   /* POWSPEC_ERR_CATA: particle outside [0, BOX_SIZE) */
#define PS_GPU_ERR_MESH (-13)   /* POWSPEC_ERR_MESH */
#define PS_GPU_ERR_PK (-14)     /* POWSPEC_ERR_PK: bin definition (src/multipole.c:344-356) */
#define PS_GPU_ERR_CUDA (-20)   /* CUDA runtime error or no usable device */
#define PS_GPU_ERR_STATE (-21)  /* call order: execute before every catalogue was assigned */
#define PS_GPU_ERR_RANGE (-22)  /* total |weight| too large for the fixed-point mesh */

/* Particle assignment schemes (src/genr_mesh.h:37-42). */
#define PS_ASSIGN_NGP 0
#define PS_ASSIGN_CIC 1
#define PS_ASSIGN_TSC 2
#define PS_ASSIGN_PCS 3

/* Estimator settings.  Every field has the meaning of the CONF field of the
 * same role after load_conf (src/load_conf.h:40-117); in particular kmin and
 * kmax are log10 values when logscale is set (src/load_conf.c:1352-1354) and
 * kmax <= 0 means "unset" (POWSPEC_KMAX_ISSET, src/define.h:68). */
typedef struct {
  int ng;            /* GRID_SIZE: even, with ng/2 a product of 2, 3 and 5 */
  double box[3];     /* BOX_SIZE */
  int assign;        /* PARTICLE_ASSIGN */
  int interlace;     /* GRID_INTERLACE */
  int ncat;          /* number of data catalogues: 1 or 2 */
  int isauto[2];     /* auto spectra wanted (OUTPUT_AUTO set) */
  int iscross;       /* cross spectrum wanted (OUTPUT_CROSS set, ncat == 2) */
  double los[3];     /* LINE_OF_SIGHT */
  double kmin, kmax; /* KMIN, KMAX */
  double dk;         /* BIN_SIZE */
  int logscale;      /* LOG_SCALE */
  int npole;         /* number of multipoles */
  int poles[7];      /* MULTIPOLE: sorted, unique, 0..6 */
  int device;        /* CUDA device ordinal */
} ps_gpu_params;

/* Outputs of ps_gpu_execute; arrays are caller-owned and sized with
 * ps_gpu_nbin().  Field names follow PK (src/multipole.h:38-61). */
typedef struct {
  int nbin;          /* out */
  double *k;         /* [nbin]   bin centres */
  double *kedge;     /* [nbin+1] bin edges */
  double *km;        /* [nbin]   mean |k| of the modes in each bin */
  uint64_t *cnt;     /* [nbin]   mode counts (bit-exact with the reference) */
  double *lcnt;      /* [npole*nbin] sum of weight * L_l(mu) per bin */
  double *pl;        /* [2][npole][nbin] auto multipoles (NULL: not copied) */
  double *xpl;       /* [npole][nbin] cross multipoles (NULL: not copied) */
  double shot[2];    /* out: V / W (src/genr_mesh.c:907) */
  double norm[2];    /* out: W^2 / V (src/genr_mesh.c:908) */
  double wdata[2];   /* out: W = sum of weights */
} ps_gpu_result;

typedef struct ps_gpu_ctx ps_gpu_ctx;

/* Validates the settings, defines the bins (src/multipole.c:334-394),
 * allocates the device meshes, and builds the geometry tables: bin of every
 * squared lattice vector, mode counts, mean |k| and the multipole mode
 * weights (src/multipole.c:111-257, which depend on the geometry only). */
int ps_gpu_create(const ps_gpu_params *params, ps_gpu_ctx **ctx);

/* Frees everything the context owns (src/genr_mesh.c:615, src/multipole.c:270). */
void ps_gpu_destroy(ps_gpu_ctx *ctx);

/* Number of k bins; < 0 on error. */
int ps_gpu_nbin(const ps_gpu_ctx *ctx);

/* Assigns catalogue `cat` (0 or 1) to its mesh(es) with the configured
 * scheme (src/genr_mesh.c:793-848 for CUBIC_SIM).  Positions must lie in
 * [0, BOX_SIZE) (src/genr_mesh.c:523-531).
 *   _aos:  xyzw = n records {double x, y, z, w} -- the reference DATA
 *          layout (src/read_cata.h:42-45).
 *   _soa:  four float arrays x[n], y[n], z[n], w[n] (w may be NULL: unit
 *          weights).
 * on_device = 0: host pointers (copied through a pinned staging buffer);
 * on_device = 1: pointers already in this device's memory.  Asynchronous on
 * the context stream; errors from out-of-range particles are reported by
 * ps_gpu_execute. */
int ps_gpu_assign_aos(ps_gpu_ctx *ctx, int cat, const double *xyzw, size_t n,
                      int on_device);
int ps_gpu_assign_soa(ps_gpu_ctx *ctx, int cat, const float *x,
                      const float *y, const float *z, const float *w,
                      size_t n, int on_device);

/* Survey catalogue `cat` (CUBIC_SIM = F), set before its assign: the
 * context's catalogue holds the data with weights w and the randoms with
 * weights -alpha w, positions minus the box's lower corner `origin`
 * (src/genr_mesh.c:797-809, :541-566); its FP32 mesh keeps its mean.
 * P_0 = (sum / cnt - shot) / norm with the given shot noise and
 * normalisation (src/read_cata.c:173-183, src/multipole.c:1108-1116); the
 * k = 0 mode is summed when it lies in the first bin (src/multipole.c:593).
 * Multipoles l > 0 (origin needed, the observer at 0) come from the
 * spherical-harmonic decomposition of L_l (src/mp_template.c:48-149):
 * P_l = 4 pi sum Re[F_0 F_l*] / (norm cnt); with interlacing the harmonics
 * weight the c2r of the combined field (src/multipole.c:489-500).
 * The result reports shot / norm as its shot noise (src/save_res.c:89).
 * Survey catalogues take no |mu| sub-bins (PS_GPU_ERR_ARG here and from
 * ps_gpu_set_mu_bins), and ps_gpu_execute refuses (PS_GPU_ERR_STATE) a
 * two-catalogue context with one survey catalogue. */
int ps_gpu_set_survey(ps_gpu_ctx *ctx, int cat, double shot, double norm, const double *origin);

/* Staged input (no counterpart in the reference): ps_gpu_stage_aos starts
 * copying n AoS records from pinned host memory into device slot `slot`
 * (0 or 1) on the context's copy stream and returns at once;
 * ps_gpu_assign_staged(ctx, cat, slot) then assigns them, its kernels
 * waiting for that copy.  With two slots the copy of the next catalogue
 * overlaps the evaluation of this one.  The host records must stay
 * unchanged until the catalogue's execute returns; a slot is refilled only
 * after the kernels that read its previous catalogue. */
int ps_gpu_stage_aos(ps_gpu_ctx *ctx, int slot, const double *xyzw, size_t n);
int ps_gpu_assign_staged(ps_gpu_ctx *ctx, int cat, int slot);

/* FFTs, interlace combine, window compensation, binning and normalisation
 * (src/multipole.c:435-505, :778-1087, :1267-1274).  Blocks until the
 * results are on the host. */
int ps_gpu_execute(ps_gpu_ctx *ctx, ps_gpu_result *res);

/* Last error message of this context (never NULL). */
const char *ps_gpu_last_error(const ps_gpu_ctx *ctx);

/* Device time in milliseconds of the phases of the last execute, measured
 * with CUDA events on the context stream: [0] assignment (all catalogues),
 * [1] z transform, [2] y transform, [3] x transform + combine + binning,
 * [4] reduction, [5] total.  Returns the number of entries written. */
int ps_gpu_last_timings(const ps_gpu_ctx *ctx, float *ms, int nmax);

/* Number of kernel launches issued by the last assign+execute cycle. */
int ps_gpu_last_launches(const ps_gpu_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), so that callers can order
 * their own work or record CUDA events around the context's launches. */
void *ps_gpu_stream(const ps_gpu_ctx *ctx);

/* Splits every k bin of the binning sweep into nmu bins of |mu| in [0, 1]
 * (1 restores the plain binning; at most 64).  ps_gpu_execute still returns
 * the usual P_l(k); the raw per-(k, |mu|) sums sum p L_l(mu) of its spectra
 * (autos, then the cross) are kept for ps_gpu_read_kmu.  Used by the learned
 * alias correction.  No counterpart in the reference. */
int ps_gpu_set_mu_bins(ps_gpu_ctx *ctx, int nmu);

/* Copies the last execute's raw sums, [nspec][npole][nbin][nmu]. */
int ps_gpu_read_kmu(const ps_gpu_ctx *ctx, double *out);

/* ---- Stage-level entry points (checked against the oracle stage by stage) */

/* Copies mesh m (0: Fr, 1: Frl) of catalogue cat to the host as doubles,
 * row-major [ng][ng][ng]: the exact fixed-point cell sums (2^-32 units),
 * re-accumulated from the catalogue's sorted records.  Valid between the
 * assign of `cat` and the next assign or execute. */
int ps_gpu_read_mesh(ps_gpu_ctx *ctx, int cat, int m, double *out);

/* Standalone r2c 3-D FFT of a real FP32 cube [ng][ng][ng] (host memory)
 * into the FFTW half-complex layout [ng][ng][ng/2+1] of interleaved FP32
 * (re, im) (host memory).  Uses ctx's device buffers of mesh 0 of
 * catalogue 0. */
int ps_gpu_fft_r2c_host(ps_gpu_ctx *ctx, const float *in, float *out);

/* Binning sweep alone over given half-complex FP32 field(s) in FFTW layout
 * (host memory), with the window of the configured scheme: f1 == f2 gives
 * an auto spectrum.  Writes the unnormalised sums
 * pl[npole][nbin] = sum p L_l(mu) (src/multipole.c:815-880). */
int ps_gpu_bin_fields_host(ps_gpu_ctx *ctx, const float *f1, const float *f2,
                           double *pl);

/* The same binning over DEVICE fields, allocating nothing: no counterpart in
 * the reference.  For callers that hold the device memory in their own pool
 * (in-situ measurement inside a simulation step), where cudaMalloc would
 * synchronise the device or fail.  f1, f2: device half-complex FP32 fields
 * [ng][ng][ng/2+1] (re, im); pl: device output [npole][nbin] doubles, written
 * asynchronously on `stream` (a cudaStream_t; NULL = legacy default stream).
 * The per-CTA partial sums live in one static device array per GPU (4,096,000
 * bytes): npole * nbin must be <= 3200, else PS_GPU_ERR_RANGE.  ps_gpu_create
 * makes the array resident on the context's device (the module load that
 * places it), so the per-step call does not; should that fail there, the
 * first call of this entry point does it, and that call should come before
 * any stream capture.  Every call looks the array's address up anew
 * (cudaGetSymbolAddress) and gives the caller's current device back on
 * return.  All calls on one device share the array: calls whose stream work
 * can overlap race and corrupt each other's sums, so order them on one
 * stream. */
int ps_gpu_bin_fields_noalloc(ps_gpu_ctx *ctx, const float *f1, const float *f2,
                              double *pl, void *stream);

/* ---- Ensembles of catalogues (mock ensembles for covariances).  No
 * counterpart in the reference, which evaluates one catalogue per run. ---- */
typedef struct ps_gpu_batch ps_gpu_batch;

/* Records, once, every launch of ncat single-catalogue evaluations through
 * ctx (assignment, FFT passes, binning, reduction into a result slot per
 * catalogue, one copy of all slots to pinned host memory) as one CUDA graph.
 * ctx must hold one catalogue (ncat == 1); xyzw[i] are device AoS records
 * {x, y, z, w} (32-byte aligned) of n[i] objects, which must stay in place
 * while the batch exists.  Catalogues with different meshes or schemes go to
 * different contexts (and batches, which may run concurrently). */
int ps_gpu_batch_create(ps_gpu_ctx *ctx, int ncat, const double *const *xyzw,
                        const size_t *n, ps_gpu_batch **batch);
/* One graph launch on the context's stream; wait != 0 blocks until done. */
int ps_gpu_batch_launch(ps_gpu_batch *batch, int wait);
int ps_gpu_batch_wait(ps_gpu_batch *batch);
/* Result of catalogue i of the last completed launch (as ps_gpu_execute). */
int ps_gpu_batch_result(ps_gpu_batch *batch, int i, ps_gpu_result *r);
/* Kernel launches recorded in the graph. */
int ps_gpu_batch_launches(const ps_gpu_batch *batch);
void ps_gpu_batch_destroy(ps_gpu_batch *batch);

/* One CUDA graph over several batches (no counterpart in the reference):
 * each batch's graph becomes a child node with no dependency on the
 * others, so batches of different contexts run concurrently from a single
 * graph launch on the ensemble's own stream.  The batches (one per context)
 * must outlive the ensemble; their results are read with
 * ps_gpu_batch_result after ps_gpu_ensemble_wait. */
typedef struct ps_gpu_ensemble ps_gpu_ensemble;
int ps_gpu_ensemble_create(ps_gpu_batch *const *batches, int nbatch, ps_gpu_ensemble **ens);
int ps_gpu_ensemble_launch(ps_gpu_ensemble *ens, int wait);
int ps_gpu_ensemble_wait(ps_gpu_ensemble *ens);
void ps_gpu_ensemble_destroy(ps_gpu_ensemble *ens);

/* Autotuner (no counterpart in the reference): times the alternative launch
 * configurations on one catalogue -- region or tile gather, gather CTA size
 * and dense-tile mapping, radix-16 / radix-32 z and y passes, pipelined or
 * plain last pass -- with `reps` evaluations each, and keeps the fastest for
 * the context.  choice[6] (if not NULL): gather threads, z radix-32,
 * y radix-32, pipelined pass C, lane groups on dense tiles, region gather. */
int ps_gpu_autotune(ps_gpu_ctx *ctx, const double *xyzw, size_t n, int reps, int *choice);
/* Sets the configurations ps_gpu_autotune chooses (no counterpart in the
 * reference), in its choice[6] order; -1 keeps an entry.  choice[5] = 2
 * returns the region gather to its default: on when there is a particle
 * for every 32 cells or more. */
int ps_gpu_set_tuning(ps_gpu_ctx *ctx, const int *choice);

/* Warp-register transforms of power-of-two meshes (no counterpart in the
 * reference): each warp transforms whole lines in registers, with no block
 * barrier inside a transform.  mask bit 0: the z pass (Ng = 256..2048), bit
 * 1: the y pass, bit 2: the x pass with the combine and binning (Ng = 256..
 * 1024); bits without a warp form for the mesh size are dropped.  They are
 * on by default, and ps_gpu_autotune times both forms of each pass.
 * mask < 0 only reads the setting.  Returns the mask in effect, or a status
 * < 0. */
int ps_gpu_set_warp_fft(ps_gpu_ctx *ctx, int mask);

/* ---- Test hook (no counterpart in the reference) */

/* Fake of an out-of-memory allocation: n > 0 makes the n-th next device or
 * pinned-host allocation made by this library's context and batch entry
 * points fail as cudaErrorMemoryAllocation without calling CUDA; n <= 0
 * disarms it.  The entry point that hits it returns PS_GPU_ERR_MEMORY, where
 * the reference exits with POWSPEC_ERR_MEMORY (src/multipole.c:121-126). */
void ps_gpu_debug_fail_alloc(int n);

/* Bounded-wait check: in the next evaluation, CTA 0 of each bulk-copy
 * pipelined pass (the block-tiled z, y and x passes) arms the barrier of
 * its second tile but issues no copy for it, and every barrier wait of
 * those passes gives up after `polls` polls.  The wait runs out, the CTA
 * drains its copies in flight and stops, and ps_gpu_execute returns
 * PS_GPU_ERR_CUDA; the context stays usable.  No fault is involved. */
int ps_gpu_debug_stall_pipeline(ps_gpu_ctx *ctx, int polls);

#ifdef __cplusplus
}
#endif

#endif
