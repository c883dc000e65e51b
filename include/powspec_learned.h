/*
 * powspec_learned.h -- C ABI of the learned alias/window correction.
 *
 * No counterpart in the reference: it extends the analytic window/alias
 * compensation of src/multipole.c:46-100 with a small network trained on
 * pairs of coarse- and fine-mesh spectra that the plain estimator produces.
 *
 * Network: 6 -> 64 -> 64 -> 64 -> 1, GELU, BF16 weights and activations on
 * the tensor cores (mma.sync m16n8k16), FP32 accumulation; output y,
 * correction c = exp(y).  Features of a (k bin, |mu| bin) cell of a coarse
 * mesh: k/k_Nyq, (k/k_Nyq)^2, mu^2, scheme/3, interlace, shot/(shot + P_0).
 *
 * Training data: groups of 16 |mu| cells of one k bin of one coarse
 * measurement.  Per row: features x[6] and A[3] (the cell's raw sums of
 * p L_l, l = 0, 2, 4, divided by norm * cnt of the bin).  Per group 8
 * floats: B_0, B_2, B_4 (shot-noise terms shot * lcnt_l / cnt), the
 * fine-mesh labels Pf_0, Pf_2, Pf_4, 1 / sigma^2, and a 0/1 mask.  The
 * group's loss is sum_l ((2l+1) (sum_j c_j A_jl - B_l) - Pf_l)^2 / sigma^2.
 */
#ifndef POWSPEC_LEARNED_H
#define POWSPEC_LEARNED_H

#include "powspec_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ps_mlp ps_mlp;

/* Number of FP32 parameters (W1[16][64] with input rows 6..15 zero, b1[64],
 * W2[64][64], b2, W3[64][64], b3, w4[64], b4). */
int ps_mlp_nparam(void);

/* Network on `device` with all parameters zero (c = 1 everywhere). */
int ps_mlp_create(int device, ps_mlp **out);
void ps_mlp_destroy(ps_mlp *m);
const char *ps_mlp_last_error(const ps_mlp *m);

int ps_mlp_set_params(ps_mlp *m, const float *params);
int ps_mlp_get_params(ps_mlp *m, float *params);

/* Uploads the training set: x[ngroups * 16][6], a[ngroups * 16][3],
 * grp[ngroups][8] (host memory). */
int ps_mlp_set_data(ps_mlp *m, const float *x, const float *a, const float *grp,
                    int ngroups);

/* Gradient of the mean loss over `batch` groups (indices idx) at the
 * current parameters; no update.  grad: [ps_mlp_nparam()] or NULL. */
int ps_mlp_grad(ps_mlp *m, const int *idx, int batch, float *grad, float *loss);

/* nsteps Adam steps (beta 0.9, 0.999, eps 1e-8) with learning rate lr;
 * step s uses groups idx[s * batch .. (s + 1) * batch).  loss[s] (optional)
 * receives each step's mean loss. */
int ps_mlp_train(ps_mlp *m, const int *idx, int nsteps, int batch, float lr,
                 float *loss);

/* c[i] = exp(y(x[i])) for n feature rows x[n][6] (host memory). */
int ps_mlp_infer(ps_mlp *m, const float *x, int n, float *c);

/* One learned evaluation, all on the GPU: the context's passes (one
 * catalogue assigned; poles 0, 2, 4; linear bins; |mu| sub-bins set with
 * ps_gpu_set_mu_bins to the network's 16), then on the context's stream the
 * cell features, the network's c = exp(y) per (k, |mu|) cell and
 * Pc_l = (2l+1) (sum_j c_j A_jl - B_l), with one copy back.  res is filled
 * as by ps_gpu_execute (the uncorrected multipoles); pl_corr receives the
 * corrected ones, [3][nbin].  The network's weights are only read: do not
 * train it meanwhile. */
int ps_gpu_execute_learned(ps_gpu_ctx *ctx, ps_mlp *m, ps_gpu_result *res, double *pl_corr);

/* ps_gpu_execute_learned in two halves (no counterpart in the reference),
 * for evaluating many catalogues back to back: launch enqueues the passes,
 * the network and the copy back, and returns; the next catalogue may then
 * be assigned (its assignment runs on the GPU after this evaluation) before
 * finish waits for this evaluation's results and fills res and pl_corr as
 * ps_gpu_execute_learned does.  One evaluation may be pending at a time;
 * ps_gpu_execute is refused meanwhile. */
int ps_gpu_learned_launch(ps_gpu_ctx *ctx, ps_mlp *m);
int ps_gpu_learned_finish(ps_gpu_ctx *ctx, ps_gpu_result *res, double *pl_corr);

/* Checkpoint with parameters, Adam moments and step count; load resumes. */
int ps_mlp_save(ps_mlp *m, const char *path);
int ps_mlp_load(ps_mlp *m, const char *path);

#ifdef __cplusplus
}
#endif

#endif
