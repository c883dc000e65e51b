/*
 * ps_oracle.c -- CPU restatement (FP64, OpenMP) of powspec's periodic-box
 * estimator path.  TEST INFRASTRUCTURE ONLY: the oracle that the GPU path is
 * checked against and the CPU baseline that bench.py times.  The GPU product
 * never links or calls this file.
 *
 * The arithmetic of every step is written so that, with one thread, it
 * performs the same floating-point operations in the same order as the
 * reference (cited per function), which tests/test_oracle_ref.py checks
 * bit-for-bit against the reference compiled from source.  The stencils are
 * written separably (1-D node/weight lists per axis, then the product
 * (wx*wy)*wz), which is the order the reference's unrolled node lists use.
 */
#define _POSIX_C_SOURCE 200112L
#include "ps_oracle.h"

#include <fftw3.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PS_PI 3.14159265358979323846264338327950288
#define PS_ERR_MEMORY (-1)
#define PS_ERR_ARG (-2)
#define PS_ERR_PK (-14)

static double wall(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0;
#endif
}

void ps_oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
  fftw_plan_with_nthreads(n);
}

int ps_oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* math/legpoly.h:47-62 */
double ps_oracle_legpoly(int ell, double x) {
  if (ell == 0) return 1;
  const double x2 = x * x;
  switch (ell) {
    case 1: return x;
    case 2: return 1.5 * x2 - 0.5;
    case 3: return 2.5 * x * (x2 - 0.6);
    case 4: return 4.375 * x2 * x2 - 3.75 * x2 + 0.375;
    case 5: return 8.75 * x * (0.9 * x2 * x2 - x2 + 0x1.b6db6db6db6dbp-3);
    case 6:
      return 14.4375 * x2 * x2 * x2 - 19.6875 * x2 * x2 + 6.5625 * x2 - 0.3125;
    default: return 0;
  }
}

/* src/multipole.c:46-100: Jing (2005) window / alias factor per dimension.
 * Interlaced: (x/sin x)^(2p) with p = assign+1; otherwise the inverse of the
 * aliased window sum for each scheme.  Taylor series below x = 0.01 with the
 * same coefficients (1/6, 7/360, 31/15120 and 1/6, 1/120, 1/5040). */
double ps_oracle_alias_corr(int interlace, int assign, double pik) {
  double fac;
  if (interlace) {
    if (pik > 0.01) {
      fac = pik / sin(pik);
    } else {
      double t = pik * pik;
      fac = 1 + 0x1.5555555555555p-3 * t + 0x1.3e93e93e93e94p-6 * t * t +
            0x1.0cbb766210cbbp-9 * t * t * t;
    }
    fac *= fac;
    switch (assign) {
      case 0: return fac;
      case 1: return fac * fac;
      case 2: return fac * fac * fac;
      case 3: fac *= fac; return fac * fac;
      default: return 1;
    }
  }
  if (pik > 0.01) {
    fac = sin(pik);
  } else {
    double t = pik * pik;
    fac = (1 - 0x1.5555555555555p-3 * t + 0x1.1111111111111p-7 * t * t -
           0x1.a01a01a01a01ap-13 * t * t * t) * pik;
  }
  fac *= fac;
  switch (assign) {
    case 0: return 1;
    case 1: return 1 / (1 - 0x1.5555555555555p-1 * fac);
    case 2: return 1 / (1 - fac + 0x1.1111111111111p-3 * fac * fac);
    case 3:
      return 1 / (1 - 0x1.5555555555555p+0 * fac + 0.4 * fac * fac -
                  0x1.a01a01a01a01ap-7 * fac * fac * fac);
    default: return 1;
  }
}

/* 1-D stencil of one coordinate: nodes and weights.  Grid coordinate
 * x = (pos - bmin) * Ng / L (src/genr_mesh.c:57,91,152,256).  The index is
 * wrapped into [0, Ng) when x rounds up to Ng, where the reference would
 * index one cell past the mesh (src/genr_mesh.c:60, no guard). */
static int stencil_1d(int assign, double x, int ng, int *node, double *w) {
  int i0 = (int)x;
  double d = x - i0;
  if (i0 >= ng) i0 -= ng;
  switch (assign) {
    case 0: /* NGP, src/genr_mesh.c:60-66 */
      if (d >= 0.5) i0 = (i0 == ng - 1) ? 0 : i0 + 1;
      node[0] = i0;
      w[0] = 1;
      return 1;
    case 1: /* CIC, src/genr_mesh.c:94-108 */
      node[0] = i0;
      node[1] = (i0 == ng - 1) ? 0 : i0 + 1;
      w[1] = d;
      w[0] = 1 - d;
      return 2;
    case 2: /* TSC, src/genr_mesh.c:153-173 */
      if (d < 0.5) {
        node[1] = i0;
        node[0] = (i0 == 0) ? ng - 1 : i0 - 1;
        node[2] = (i0 == ng - 1) ? 0 : i0 + 1;
        w[0] = 0.5 - d;
        w[0] *= w[0] * 0.5;
        w[1] = 0.75 - d * d;
      } else {
        node[0] = i0;
        node[1] = (i0 == ng - 1) ? 0 : i0 + 1;
        node[2] = (node[1] == ng - 1) ? 0 : node[1] + 1;
        d = 1 - d;
        w[0] = 0.5 + d;
        w[0] *= w[0] * 0.5;
        w[1] = 0.75 - d * d;
      }
      w[2] = 1 - w[0] - w[1];
      return 3;
    default: { /* PCS, src/genr_mesh.c:256-270 (weights x6, /6^3 later) */
      node[1] = i0;
      node[0] = (i0 == 0) ? ng - 1 : i0 - 1;
      node[2] = (i0 == ng - 1) ? 0 : i0 + 1;
      node[3] = (node[2] == ng - 1) ? 0 : node[2] + 1;
      double d2 = d * d;
      w[3] = d2 * d;
      w[2] = 1 + 3 * (d + d2 - w[3]);
      w[1] = 4 - 6 * d2 + 3 * w[3];
      w[0] = 6 - w[1] - w[2] - w[3];
      return 4;
    }
  }
}

/* One mesh: every particle's stencil added with an atomic FP64 add per node,
 * x-node outermost (src/genr_mesh.c:50-412). shift != 0 selects the
 * interlaced grid: lower corner smin = -H/2 and particles at x >= smin + L
 * moved by -L first (src/genr_mesh.c:590-602, :815-833). */
static void assign_mesh(const double *xyzw, size_t n, int ng,
                        const double box[3], int assign, int shift,
                        double *rho) {
  double bmin[3] = {0, 0, 0};
  if (shift)
    for (int d = 0; d < 3; d++) bmin[d] = 0.0 - 0.5 * box[d] / ng;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (size_t i = 0; i < n; i++) {
    const double *p = xyzw + 4 * i;
    int node[3][4];
    double wt[3][4];
    int s = 1;
    for (int d = 0; d < 3; d++) {
      double pos = p[d];
      if (shift && pos >= bmin[d] + box[d]) pos -= box[d];
      double x = (pos - bmin[d]) * ng / box[d];
      s = stencil_1d(assign, x, ng, node[d], wt[d]);
    }
    double wfac = p[3];
    if (assign == 3) wfac = p[3] * 0x1.2f684bda12f68p-8; /* 1/6^3 */
    for (int a = 0; a < s; a++) wt[0][a] *= wfac;
    for (int a = 0; a < s; a++) {
      for (int b = 0; b < s; b++) {
        size_t row = ((size_t)node[0][a] * ng + node[1][b]) * ng;
        double wab = wt[0][a] * wt[1][b];
        for (int c = 0; c < s; c++) {
          double v = wab * wt[2][c];
#ifdef _OPENMP
#pragma omp atomic
#endif
          rho[row + node[2][c]] += v;
        }
      }
    }
  }
}

int ps_oracle_assign(const double *xyzw, size_t n, int ng, const double box[3],
                     int assign, int interlace, double *mesh0, double *mesh1) {
  if (ng < 1 || assign < 0 || assign > 3 || !mesh0) return PS_ERR_ARG;
  size_t ntot = (size_t)ng * ng * ng;
  memset(mesh0, 0, sizeof(double) * ntot);
  assign_mesh(xyzw, n, ng, box, assign, 0, mesh0);
  if (interlace) {
    if (!mesh1) return PS_ERR_ARG;
    memset(mesh1, 0, sizeof(double) * ntot);
    assign_mesh(xyzw, n, ng, box, assign, 1, mesh1);
  }
  return 0;
}

/* src/multipole.c:334-394 */
int ps_oracle_bins(int ng, const double box[3], double kmin, double kmax,
                   double dk, int logscale, int maxbin, int *nbin,
                   double *kedge, double *k) {
  double bmax = (box[0] > box[1]) ? box[0] : box[1];
  if (bmax < box[2]) bmax = box[2];
  double kny = PS_PI * ng / bmax;
  if (logscale) kny = log10(kny);
  double kupper = kny;
  if (kmax > 0 && kupper > kmax) kupper = kmax;
  double nb = round((kupper - kmin) / dk);
  if (!(nb < INT_MAX)) return PS_ERR_PK;
  int nbn = (int)nb;
  if (kmin + dk * nbn > kny) nbn -= 1;
  if (nbn < 1) return PS_ERR_PK;
  *nbin = nbn;
  if (nbn > maxbin) return PS_ERR_ARG;
  for (int i = 0; i <= nbn; i++) kedge[i] = kmin + dk * i;
  for (int i = 0; i < nbn; i++) k[i] = (kedge[i] + kedge[i + 1]) * 0.5;
  return 0;
}

/* Bin of a squared wave number, or -1 (src/multipole.c:147-158). */
static inline int kbin_of(double kmod2, int logscale, int nbin,
                          const double *kedge, double dk, double *kmod_out) {
  double kmod = logscale ? 0.5 * log10(kmod2) : sqrt(kmod2);
  *kmod_out = kmod;
  if (kmod < kedge[0] || kmod >= kedge[nbin]) return -1;
  int b = (int)((kmod - kedge[0]) / dk);
  if (b < 0 || b >= nbin) return -1;
  return b;
}

/* src/multipole.c:111-257: window table over the half-complex mesh (0 marks
 * modes outside the k range), mode counts with weight 1 on the k=0 and
 * Nyquist planes and 2 between, and the mean |k| per bin. */
int ps_oracle_precomp(int ng, const double box[3], int assign, int interlace,
                      int logscale, int nbin, const double *kedge, double dk,
                      double *alias, size_t *cnt, double *km) {
  const int ngk = ng / 2 + 1;
  const double fac = PS_PI / ng;
  double vec[3];
  for (int d = 0; d < 3; d++) vec[d] = 2 * PS_PI / box[d];
  memset(cnt, 0, sizeof(size_t) * nbin);
  memset(km, 0, sizeof(double) * nbin);
  int fail = 0;
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    double *kc = calloc(nbin, sizeof(double));
    size_t *cc = calloc(nbin, sizeof(size_t));
    if (!kc || !cc) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
      fail = 1;
    }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int i = 0; i < ng; i++) {
      if (!kc || !cc) continue;
      size_t idx_i = (size_t)i * ng * ngk;
      double ki = (i <= (ng >> 1)) ? i : i - ng;
      double ai = ps_oracle_alias_corr(interlace, assign, ki * fac);
      ki *= vec[0];
      double kmi = ki * ki;
      for (int j = 0; j < ng; j++) {
        size_t idx_j = idx_i + (size_t)j * ngk;
        double kj = (j <= (ng >> 1)) ? j : j - ng;
        double aj = ps_oracle_alias_corr(interlace, assign, kj * fac);
        kj *= vec[1];
        double kmj = kmi + kj * kj;
        for (int k = 0; k < ngk; k++) {
          /* planes k = 0 and k = Ng/2 (even Ng) count once, others twice */
          int wmode = (k == 0 || (2 * k == ng)) ? 1 : 2;
          double kk = k * vec[2];
          double km2 = (k == 0) ? kmj : kmj + kk * kk;
          double kmod;
          int b = kbin_of(km2, logscale, nbin, kedge, dk, &kmod);
          if (b < 0) {
            alias[idx_j + k] = 0;
            continue;
          }
          if (k == 0)
            alias[idx_j] = ai * aj;
          else
            alias[idx_j + k] =
                ai * aj * ps_oracle_alias_corr(interlace, assign, k * fac);
          kc[b] += (wmode == 2) ? 2 * kmod : kmod;
          cc[b] += wmode;
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    if (kc && cc) {
      for (int b = 0; b < nbin; b++) {
        km[b] += kc[b];
        cnt[b] += cc[b];
      }
    }
    free(kc);
    free(cc);
  }
  if (fail) return PS_ERR_MEMORY;
  for (int b = 0; b < nbin; b++)
    if (cnt[b]) km[b] /= cnt[b];
  return 0;
}

int ps_oracle_r2c(int ng, double *mesh, double *fk) {
  fftw_plan p = fftw_plan_dft_r2c_3d(ng, ng, ng, mesh, (fftw_complex *)fk,
                                     FFTW_ESTIMATE);
  if (!p) return PS_ERR_MEMORY;
  fftw_execute_dft_r2c(p, mesh, (fftw_complex *)fk);
  fftw_destroy_plan(p);
  return 0;
}

/* src/multipole.c:462-487: F0 <- (F0 + exp(i theta) F1) / 2 with
 * theta = (pi/Ng) (i' + j' + k), i', j' signed. */
int ps_oracle_combine(int ng, double *fk0, const double *fk1) {
  const int ngk = ng / 2 + 1;
  const double fac = PS_PI / ng;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < ng; i++) {
    size_t idx_i = (size_t)i * ng * ngk;
    double ki = fac * ((i <= (ng >> 1)) ? i : i - ng);
    for (int j = 0; j < ng; j++) {
      size_t idx_j = idx_i + (size_t)j * ngk;
      double kj = fac * ((j <= (ng >> 1)) ? j : j - ng);
      for (int k = 0; k < ngk; k++) {
        size_t idx = 2 * (idx_j + k);
        double ks = ki + kj + fac * k;
        double c = cos(ks), s = sin(ks);
        double a0 = fk0[idx], a1 = fk0[idx + 1];
        double b0 = fk1[idx], b1 = fk1[idx + 1];
        fk0[idx] = 0.5 * (a0 + c * b0 - s * b1);
        fk0[idx + 1] = 0.5 * (a1 + s * b0 + c * b1);
      }
    }
  }
  return 0;
}

/* src/multipole.c:778-1031.  DC skipped; odd ell skipped on the planes
 * that count twice; mu = (k . los) / |k|. */
int ps_oracle_count_sim(int ng, const double box[3], const double *alias,
                        const double *f1, const double *f2, int logscale,
                        int nbin, const double *kedge, double dk,
                        const double los[3], int npole, const int *poles,
                        double *pl, double *lcnt) {
  const int ngk = ng / 2 + 1;
  double vec[3];
  for (int d = 0; d < 3; d++) vec[d] = 2 * PS_PI / box[d];
  const size_t nacc = (size_t)npole * nbin;
  memset(lcnt, 0, sizeof(double) * nacc);
  int fail = 0;
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    double *ps = calloc(nacc, sizeof(double));
    double *ls = calloc(nacc, sizeof(double));
    if (!ps || !ls) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
      fail = 1;
    }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int i = 0; i < ng; i++) {
      if (!ps || !ls) continue;
      size_t idx_i = (size_t)i * ng * ngk;
      double ki = vec[0] * ((i <= (ng >> 1)) ? i : i - ng);
      double kmi = ki * ki;
      for (int j = 0; j < ng; j++) {
        size_t idx_j = idx_i + (size_t)j * ngk;
        double kj = vec[1] * ((j <= (ng >> 1)) ? j : j - ng);
        double kmj = kmi + kj * kj;
        for (int k = 0; k < ngk; k++) {
          size_t idx = idx_j + k;
          if (!alias[idx]) continue;
          if (k == 0 && !kmj) continue; /* DC */
          int twice = !(k == 0 || 2 * k == ng);
          double kk = vec[2] * k;
          double km2 = (k == 0) ? kmj : kmj + kk * kk;
          double kmod = sqrt(km2);
          double kl = logscale ? 0.5 * log10(km2) : kmod;
          int b = (int)((kl - kedge[0]) / dk);
          double mu = (k == 0) ? (ki * los[0] + kj * los[1]) / kmod
                               : (ki * los[0] + kj * los[1] + kk * los[2]) / kmod;
          double p = (f1[2 * idx] * f2[2 * idx] + f1[2 * idx + 1] * f2[2 * idx + 1]) *
                     alias[idx];
          double num = 1;
          if (twice) { p *= 2; num = 2; }
          for (int l = 0; l < npole; l++) {
            if (twice && (poles[l] & 1)) continue;
            double leg = ps_oracle_legpoly(poles[l], mu);
            ps[(size_t)l * nbin + b] += p * leg;
            ls[(size_t)l * nbin + b] += num * leg;
          }
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    if (ps && ls) {
      for (size_t t = 0; t < nacc; t++) {
        pl[t] += ps[t];
        lcnt[t] += ls[t];
      }
    }
    free(ps);
    free(ls);
  }
  return fail ? PS_ERR_MEMORY : 0;
}

int ps_oracle_run(const ps_oracle_params *p, const double *const *xyzw,
                  const size_t *n, ps_oracle_result *r) {
  const int ng = p->ng, nc = p->ncat;
  if (ng < 2 || nc < 1 || nc > 2 || p->npole < 1 || p->npole > 7) return PS_ERR_ARG;
  const int ngk = ng / 2 + 1;
  const size_t ntot = (size_t)ng * ng * ng, ncx = (size_t)ng * ng * ngk;
  const int npole = p->npole;
  int rc = 0;
  double *fr[2] = {0, 0}, *frl[2] = {0, 0}, *fk0[2] = {0, 0}, *fkl[2] = {0, 0};
  double *alias = NULL;

  double t0 = wall();
  for (int c = 0; c < nc; c++) {
    double w = 0;
    for (size_t i = 0; i < n[c]; i++) w += xyzw[c][4 * i + 3];
    r->wdata[c] = w;
    fr[c] = fftw_malloc(sizeof(double) * ntot);
    fk0[c] = fftw_malloc(sizeof(double) * 2 * ncx);
    if (!fr[c] || !fk0[c]) { rc = PS_ERR_MEMORY; goto done; }
    if (p->interlace) {
      frl[c] = fftw_malloc(sizeof(double) * ntot);
      fkl[c] = fftw_malloc(sizeof(double) * 2 * ncx);
      if (!frl[c] || !fkl[c]) { rc = PS_ERR_MEMORY; goto done; }
    }
    rc = ps_oracle_assign(xyzw[c], n[c], ng, p->box, p->assign, p->interlace,
                          fr[c], frl[c]);
    if (rc) goto done;
  }
  /* src/genr_mesh.c:904-910 */
  for (int c = 0; c < nc; c++) {
    double vol = p->box[0] * p->box[1] * p->box[2];
    r->shot[c] = vol / r->wdata[c];
    r->norm[c] = r->wdata[c] * r->wdata[c] / vol;
  }
  double t1 = wall();

  int nbin = 0;
  rc = ps_oracle_bins(ng, p->box, p->kmin, p->kmax, p->dk, p->logscale,
                      r->maxbin, &nbin, r->kedge, r->k);
  r->nbin = nbin;
  if (rc) goto done;
  alias = malloc(sizeof(double) * ncx);
  if (!alias) { rc = PS_ERR_MEMORY; goto done; }
  rc = ps_oracle_precomp(ng, p->box, p->assign, p->interlace, p->logscale, nbin,
                         r->kedge, p->dk, alias, r->cnt, r->km);
  if (rc) goto done;

  /* src/multipole.c:435-505 */
  for (int c = 0; c < nc; c++) {
    if ((rc = ps_oracle_r2c(ng, fr[c], fk0[c]))) goto done;
    if (p->interlace) {
      if ((rc = ps_oracle_r2c(ng, frl[c], fkl[c]))) goto done;
      ps_oracle_combine(ng, fk0[c], fkl[c]);
      if (p->with_c2r) {
        memcpy(fkl[c], fk0[c], sizeof(double) * 2 * ncx);
        fftw_plan pc = fftw_plan_dft_c2r_3d(ng, ng, ng, (fftw_complex *)fkl[c],
                                            fr[c], FFTW_ESTIMATE);
        if (!pc) { rc = PS_ERR_MEMORY; goto done; }
        fftw_execute_dft_c2r(pc, (fftw_complex *)fkl[c], fr[c]);
        fftw_destroy_plan(pc);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (size_t t = 0; t < ntot; t++) fr[c][t] /= ntot;
      }
    }
  }

  /* src/multipole.c:1047-1087 and :1221-1226 */
  const size_t mb = (size_t)r->maxbin;
  for (int c = 0; c < nc; c++) {
    if (!p->isauto[c]) continue;
    double *pl = r->pl + (size_t)c * npole * mb;
    double *tmp = calloc((size_t)npole * nbin, sizeof(double));
    double *lc = calloc((size_t)npole * nbin, sizeof(double));
    if (!tmp || !lc) { free(tmp); free(lc); rc = PS_ERR_MEMORY; goto done; }
    rc = ps_oracle_count_sim(ng, p->box, alias, fk0[c], fk0[c], p->logscale,
                             nbin, r->kedge, p->dk, p->los, npole, p->poles,
                             tmp, lc);
    for (int l = 0; l < npole; l++) {
      for (int i = 0; i < nbin; i++) {
        double v = tmp[(size_t)l * nbin + i];
        if (r->cnt[i]) {
          v /= r->norm[c] * r->cnt[i];
          v -= r->shot[c] * lc[(size_t)l * nbin + i] / r->cnt[i];
        }
        v *= 2 * p->poles[l] + 1;
        pl[l * mb + i] = v;
        r->lcnt[l * mb + i] = lc[(size_t)l * nbin + i];
      }
    }
    free(tmp);
    free(lc);
    if (rc) goto done;
  }
  if (nc == 2 && p->iscross) {
    double *tmp = calloc((size_t)npole * nbin, sizeof(double));
    double *lc = calloc((size_t)npole * nbin, sizeof(double));
    if (!tmp || !lc) { free(tmp); free(lc); rc = PS_ERR_MEMORY; goto done; }
    rc = ps_oracle_count_sim(ng, p->box, alias, fk0[0], fk0[1], p->logscale,
                             nbin, r->kedge, p->dk, p->los, npole, p->poles,
                             tmp, lc);
    for (int l = 0; l < npole; l++) {
      for (int i = 0; i < nbin; i++) {
        double v = tmp[(size_t)l * nbin + i];
        if (r->cnt[i]) v /= sqrt(r->norm[0] * r->norm[1]) * r->cnt[i];
        v *= 2 * p->poles[l] + 1;
        r->xpl[l * mb + i] = v;
        r->lcnt[l * mb + i] = lc[(size_t)l * nbin + i];
      }
    }
    free(tmp);
    free(lc);
    if (rc) goto done;
  }
  /* src/multipole.c:1267-1274, including its reuse of the rescaled k */
  if (p->logscale) {
    for (int i = 0; i < nbin; i++) {
      r->k[i] = pow(10, r->k[i]);
      r->km[i] = pow(10, r->k[i]);
      r->kedge[i] = pow(10, r->k[i]);
    }
    r->kedge[nbin] = pow(10, r->kedge[nbin]);
  }
  r->t_mesh = t1 - t0;
  r->t_pk = wall() - t1;

done:
  for (int c = 0; c < 2; c++) {
    fftw_free(fr[c]);
    fftw_free(frl[c]);
    fftw_free(fk0[c]);
    fftw_free(fkl[c]);
  }
  free(alias);
  return rc;
}

/* ------------------------------------------------------------ survey path */

/* Real spherical harmonics (math/spherical.h:54-262 tabulates one real basis
 * per ell).  Here Y_l0 = K_l0 P_l(cos t), Y_lm = sqrt2 K_lm P_l^m(cos t)
 * cos(m p), Y_l,-m = sqrt2 K_lm P_l^m(cos t) sin(m p), K_lm^2 = (2l+1)/(4 pi)
 * (l-m)!/(l+m)!.  The estimator only uses sums over m of Y_lm(a) Y_lm(b),
 * which by the addition theorem equal (2l+1)/(4 pi) L_l(a . b) for any
 * orthonormal real basis. */
double ps_oracle_ylm(int ell, int m, double ct, double st, double cp, double sp) {
  const int am = m < 0 ? -m : m;
  double f = 1;
  for (int q = ell - am + 1; q <= ell + am; q++) f /= q;
  double kl = sqrt((2 * ell + 1) / (4 * PS_PI) * f);
  if (m) kl *= sqrt(2.0);
  double pmm = 1;
  for (int i = 1; i <= am; i++) pmm *= (2 * i - 1) * st;
  double pl = pmm;
  if (ell > am) {
    double p0 = pmm, p1 = ct * (2 * am + 1) * pmm;
    pl = p1;
    for (int l = am + 2; l <= ell; l++) {
      pl = ((2 * l - 1) * ct * p1 - (l + am - 1) * p0) / (l - am);
      p0 = p1;
      p1 = pl;
    }
  }
  if (!m) return kl * pl;
  double c = 1, s = 0;
  for (int i = 0; i < am; i++) {
    const double c2 = c * cp - s * sp;
    s = s * cp + c * sp;
    c = c2;
  }
  return kl * pl * (m > 0 ? c : s);
}

/* src/multipole.c:579-754: sum over the stored modes with a window factor
 * (the k = 0 mode included) of Re[F1 F2*] x window, twice for the planes
 * 0 < kz < Ng/2, into pl[kbin]. */
static void count_survey(int ng, const double box[3], const double *alias,
                         const double *f1, const double *f2, int logscale,
                         int nbin, const double *kedge, double dk, double *pl) {
  const int ngk = ng / 2 + 1;
  double vec[3];
  for (int d = 0; d < 3; d++) vec[d] = 2 * PS_PI / box[d];
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    double *acc = calloc(nbin, sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int i = 0; i < ng; i++) {
      if (!acc) continue;
      const size_t idx_i = (size_t)i * ng * ngk;
      const double ki = vec[0] * ((i <= (ng >> 1)) ? i : i - ng);
      for (int j = 0; j < ng; j++) {
        const size_t idx_j = idx_i + (size_t)j * ngk;
        const double kj = vec[1] * ((j <= (ng >> 1)) ? j : j - ng);
        const double kmj = ki * ki + kj * kj;
        for (int k = 0; k < ngk; k++) {
          const size_t idx = idx_j + k;
          if (!alias[idx]) continue;
          const double kk = vec[2] * k;
          const double km2 = k ? kmj + kk * kk : kmj;
          const double kmod = logscale ? 0.5 * log10(km2) : sqrt(km2);
          const int b = (int)((kmod - kedge[0]) / dk);
          double v = (f1[2 * idx] * f2[2 * idx] + f1[2 * idx + 1] * f2[2 * idx + 1]) * alias[idx];
          if (k && 2 * k != ng) v *= 2;
          if (b >= 0 && b < nbin) acc[b] += v;
        }
      }
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    if (acc)
      for (int b = 0; b < nbin; b++) pl[b] += acc[b];
    free(acc);
  }
}

/* src/mp_template.c:48-149: fl = sum_m Y_lm(k^) FFT[fr Y_lm(r^)] over the
 * modes with a window factor.  The real-space direction of cell (i, j, k)
 * is ((i, j, k) + origin Ng / L) x L; the row i = j = 0 and the modes with
 * kx = ky = 0 take the harmonic as 1. */
static int harmonic_field(int ng, const double box[3], const double origin[3], int ell,
                          const double *fr, const double *alias, double *frl, double *fa,
                          double *fl) {
  const int ngk = ng / 2 + 1;
  const size_t ncx = (size_t)ng * ng * ngk;
  double smin[3], fac[3];
  for (int d = 0; d < 3; d++) {
    smin[d] = origin[d] * ng / box[d];
    fac[d] = 1 / box[d];
  }
  memset(fl, 0, sizeof(double) * 2 * ncx);
  for (int m = -ell; m <= ell; m++) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < ng; i++) {
      const size_t idx_i = (size_t)i * ng * ng;
      const double ri = (i + smin[0]) * box[0];
      for (int j = 0; j < ng; j++) {
        const size_t idx_j = idx_i + (size_t)j * ng;
        if (idx_j == 0) {
          memcpy(frl, fr, sizeof(double) * ng);
          continue;
        }
        const double rj = (j + smin[1]) * box[1];
        const double r2 = ri * ri + rj * rj, r22 = sqrt(r2);
        for (int k = 0; k < ng; k++) {
          const double rk = (k + smin[2]) * box[2];
          const double r3 = sqrt(r2 + rk * rk);
          frl[idx_j + k] = fr[idx_j + k] * ps_oracle_ylm(ell, m, rk / r3, r22 / r3, ri / r22, rj / r22);
        }
      }
    }
    int rc = ps_oracle_r2c(ng, frl, fa);
    if (rc) return rc;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < ng; i++) {
      const size_t idx_i = (size_t)i * ng * ngk;
      const double ki = fac[0] * ((i <= (ng >> 1)) ? i : i - ng);
      for (int j = 0; j < ng; j++) {
        const size_t idx_j = idx_i + (size_t)j * ngk;
        const double kj = fac[1] * ((j <= (ng >> 1)) ? j : j - ng);
        const double k2 = ki * ki + kj * kj;
        for (int k = 0; k < ngk; k++) {
          const size_t idx = idx_j + k;
          if (!alias[idx]) continue;
          const double kk = fac[2] * k, k3 = sqrt(k2 + kk * kk);
          double y = 1;
          if (k2 != 0 && k3 != 0) {
            const double k22 = sqrt(k2);
            y = ps_oracle_ylm(ell, m, kk / k3, k22 / k3, ki / k22, kj / k22);
          }
          fl[2 * idx] += fa[2 * idx] * y;
          fl[2 * idx + 1] += fa[2 * idx + 1] * y;
        }
      }
    }
  }
  return 0;
}

int ps_oracle_survey(const ps_oracle_params *p, const double origin[3],
                     const double shot[2], const double norm[2],
                     const double *const *xyzw, const size_t *n,
                     ps_oracle_result *r) {
  const int ng = p->ng, nc = p->ncat;
  if (ng < 2 || nc < 1 || nc > 2 || p->npole < 1 || p->npole > 7) return PS_ERR_ARG;
  const int ngk = ng / 2 + 1;
  const size_t ntot = (size_t)ng * ng * ng, ncx = (size_t)ng * ng * ngk;
  const int npole = p->npole;
  const size_t mb = (size_t)r->maxbin;
  int rc = 0;
  double *fr[2] = {0, 0}, *frl[2] = {0, 0}, *fk0[2] = {0, 0}, *fkl[2] = {0, 0};
  double *alias = NULL, *tmp = NULL, *fa = NULL, *wr = NULL;

  double t0 = wall();
  for (int c = 0; c < nc; c++) {
    double w = 0;
    for (size_t i = 0; i < n[c]; i++) w += xyzw[c][4 * i + 3];
    r->wdata[c] = w;
    r->shot[c] = shot[c];
    r->norm[c] = norm[c];
    fr[c] = fftw_malloc(sizeof(double) * ntot);
    fk0[c] = fftw_malloc(sizeof(double) * 2 * ncx);
    fkl[c] = fftw_malloc(sizeof(double) * 2 * ncx);
    if (!fr[c] || !fk0[c] || !fkl[c]) { rc = PS_ERR_MEMORY; goto done; }
    if (p->interlace) {
      frl[c] = fftw_malloc(sizeof(double) * ntot);
      if (!frl[c]) { rc = PS_ERR_MEMORY; goto done; }
    }
    rc = ps_oracle_assign(xyzw[c], n[c], ng, p->box, p->assign, p->interlace, fr[c], frl[c]);
    if (rc) goto done;
  }
  double t1 = wall();

  int nbin = 0;
  rc = ps_oracle_bins(ng, p->box, p->kmin, p->kmax, p->dk, p->logscale, r->maxbin, &nbin,
                      r->kedge, r->k);
  r->nbin = nbin;
  if (rc) goto done;
  alias = malloc(sizeof(double) * ncx);
  tmp = calloc(nbin, sizeof(double));
  fa = fftw_malloc(sizeof(double) * 2 * ncx);
  wr = fftw_malloc(sizeof(double) * ntot);
  if (!alias || !tmp || !fa || !wr) { rc = PS_ERR_MEMORY; goto done; }
  rc = ps_oracle_precomp(ng, p->box, p->assign, p->interlace, p->logscale, nbin, r->kedge,
                         p->dk, alias, r->cnt, r->km);
  if (rc) goto done;

  /* src/multipole.c:435-505: F_0, and with interlacing the combination and
   * its c2r / Ng^3 in place of the plain mesh */
  for (int c = 0; c < nc; c++) {
    if ((rc = ps_oracle_r2c(ng, fr[c], fk0[c]))) goto done;
    if (p->interlace) {
      if ((rc = ps_oracle_r2c(ng, frl[c], fkl[c]))) goto done;
      ps_oracle_combine(ng, fk0[c], fkl[c]);
      memcpy(fkl[c], fk0[c], sizeof(double) * 2 * ncx);
      fftw_plan pc = fftw_plan_dft_c2r_3d(ng, ng, ng, (fftw_complex *)fkl[c], fr[c],
                                          FFTW_ESTIMATE);
      if (!pc) { rc = PS_ERR_MEMORY; goto done; }
      fftw_execute_dft_c2r(pc, (fftw_complex *)fkl[c], fr[c]);
      fftw_destroy_plan(pc);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
      for (size_t t = 0; t < ntot; t++) fr[c][t] /= ntot;
    }
  }

  /* src/multipole.c:1230-1250 with the normalisations of :1090-1160 */
  for (int l = 0; l < npole; l++) {
    const int ell = p->poles[l];
    if (ell > 0)
      for (int c = 0; c < nc; c++)
        if ((rc = harmonic_field(ng, p->box, origin, ell, fr[c], alias, wr, fa, fkl[c])))
          goto done;
    for (int c = 0; c < nc; c++) {
      if (!p->isauto[c]) continue;
      memset(tmp, 0, sizeof(double) * nbin);
      count_survey(ng, p->box, alias, fk0[c], ell ? fkl[c] : fk0[c], p->logscale, nbin, r->kedge,
                   p->dk, tmp);
      double *pl = r->pl + ((size_t)c * npole + l) * mb;
      for (int i = 0; i < nbin; i++) {
        double v = tmp[i];
        if (r->cnt[i]) v = ell ? v * 4 * PS_PI / (norm[c] * r->cnt[i])
                               : (v / r->cnt[i] - shot[c]) / norm[c];
        pl[i] = v;
      }
    }
    if (nc == 2 && p->iscross) {
      memset(tmp, 0, sizeof(double) * nbin);
      if (ell == 0) {
        count_survey(ng, p->box, alias, fk0[0], fk0[1], p->logscale, nbin, r->kedge, p->dk, tmp);
      } else {
        count_survey(ng, p->box, alias, fk0[0], fkl[1], p->logscale, nbin, r->kedge, p->dk, tmp);
        count_survey(ng, p->box, alias, fk0[1], fkl[0], p->logscale, nbin, r->kedge, p->dk, tmp);
      }
      for (int i = 0; i < nbin; i++) {
        double v = tmp[i];
        if (r->cnt[i]) v *= (ell ? 2 * PS_PI : 1.0) / (sqrt(norm[0] * norm[1]) * r->cnt[i]);
        r->xpl[l * mb + i] = v;
      }
    }
  }
  if (p->logscale) {  /* src/multipole.c:1267-1274 */
    for (int i = 0; i < nbin; i++) {
      r->k[i] = pow(10, r->k[i]);
      r->km[i] = pow(10, r->k[i]);
      r->kedge[i] = pow(10, r->k[i]);
    }
    r->kedge[nbin] = pow(10, r->kedge[nbin]);
  }
  r->t_mesh = t1 - t0;
  r->t_pk = wall() - t1;

done:
  for (int c = 0; c < 2; c++) {
    fftw_free(fr[c]);
    fftw_free(frl[c]);
    fftw_free(fk0[c]);
    fftw_free(fkl[c]);
  }
  fftw_free(fa);
  fftw_free(wr);
  free(alias);
  free(tmp);
  return rc;
}
