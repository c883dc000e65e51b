/*
 * ps_oracle.h -- CPU restatement of powspec's periodic-box estimator path.
 *
 * TEST INFRASTRUCTURE (the oracle).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it, as the checker or as the timed CPU
 * baseline; the GPU product never links it.  FP64 throughout, OpenMP like the
 * reference, FFT through the project's FFTW-API shim (fftw_shim/).  Each
 * function cites the reference code it restates; parity of this restatement
 * with the reference itself is pinned by tests/test_oracle_ref.py (reference
 * compiled from source into oracle/_ref) and tests/golden/.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same meaning as the CONF fields the estimator reads (src/load_conf.h:40-117)
 * after load_conf: kmin/kmax are log10 values when logscale is set
 * (src/load_conf.c:1352-1354), kmax <= 0 means unset. */
typedef struct {
  int ng;
  double box[3];
  int assign;     /* 0 NGP, 1 CIC, 2 TSC, 3 PCS */
  int interlace;
  int ncat;       /* 1 or 2 */
  int isauto[2];
  int iscross;
  double los[3];
  double kmin, kmax, dk;
  int logscale;
  int npole;
  int poles[7];   /* sorted, unique, 0..6 */
  int with_c2r;   /* also run the interlace c2r + renormalisation the
                     reference performs (src/multipole.c:489-500) */
} ps_oracle_params;

typedef struct {
  int maxbin;     /* capacity of the arrays below (in bins) */
  int nbin;
  double *k, *kedge, *km; /* [maxbin], [maxbin+1], [maxbin] */
  size_t *cnt;            /* [maxbin] */
  double *lcnt;           /* [npole][maxbin] */
  double *pl;             /* [2][npole][maxbin] */
  double *xpl;            /* [npole][maxbin] */
  double shot[2], norm[2], wdata[2];
  double t_mesh, t_pk;    /* wall seconds of the mesh and estimator phases */
} ps_oracle_result;

void ps_oracle_set_threads(int n);
int ps_oracle_get_threads(void);

/* Particle assignment of N particles (AoS {x,y,z,w} doubles) into mesh0,
 * and, if interlace, into mesh1 on the half-cell shifted grid. */
int ps_oracle_assign(const double *xyzw, size_t n, int ng, const double box[3],
                     int assign, int interlace, double *mesh0, double *mesh1);

/* Bin definition (src/multipole.c:334-394). */
int ps_oracle_bins(int ng, const double box[3], double kmin, double kmax,
                   double dk, int logscale, int maxbin, int *nbin,
                   double *kedge, double *k);

/* Window table + mode counts (src/multipole.c:111-257).  alias: [ng][ng][ng/2+1]. */
int ps_oracle_precomp(int ng, const double box[3], int assign, int interlace,
                      int logscale, int nbin, const double *kedge, double dk,
                      double *alias, size_t *cnt, double *km);

/* r2c of a real mesh into [ng][ng][ng/2+1] complex (interleaved doubles). */
int ps_oracle_r2c(int ng, double *mesh, double *fk);

/* Interlace combine, in place on fk0 (src/multipole.c:462-487). */
int ps_oracle_combine(int ng, double *fk0, const double *fk1);

/* Sim-box binning sums (src/multipole.c:778-1031), unnormalised:
 * pl[npole][nbin] += sum p L_l(mu), lcnt[npole][nbin] = sum w L_l(mu). */
int ps_oracle_count_sim(int ng, const double box[3], const double *alias,
                        const double *f1, const double *f2, int logscale,
                        int nbin, const double *kedge, double dk,
                        const double los[3], int npole, const int *poles,
                        double *pl, double *lcnt);

/* Whole path: assignment, bins, precompute, FFT, combine, binning and
 * normalisation, like genr_mesh + powspec for CUBIC_SIM. */
int ps_oracle_run(const ps_oracle_params *p, const double *const *xyzw,
                  const size_t *n, ps_oracle_result *r);

/* Survey catalogue path (CUBIC_SIM = F), like genr_mesh + powspec for a
 * survey: xyzw[c] holds catalogue c's data (weights w) and randoms
 * (weights -alpha w), positions relative to the box corner `origin`; shot
 * and norm are the catalogue's (src/read_cata.c:165-183).  The k = 0 mode
 * is binned (src/multipole.c:579-754); multipoles l > 0 come from the
 * spherical-harmonic decomposition (src/mp_template.c:48-149), over the
 * c2r / Ng^3 of the combined field with interlacing (src/multipole.c:
 * 489-500).  los and with_c2r of p are not used.  r->shot, r->norm: the
 * given values. */
int ps_oracle_survey(const ps_oracle_params *p, const double origin[3],
                     const double shot[2], const double norm[2],
                     const double *const *xyzw, const size_t *n,
                     ps_oracle_result *r);

/* Real spherical harmonic of degree ell <= 6 and order m of the direction
 * (cos t, sin t, cos p, sin p), an orthonormal real basis. */
double ps_oracle_ylm(int ell, int m, double ct, double st, double cp, double sp);

/* Legendre polynomial P_ell(x), ell <= 6 (math/legpoly.h:47-62). */
double ps_oracle_legpoly(int ell, double x);

/* 1-D window/alias factor (src/multipole.c:46-100). */
double ps_oracle_alias_corr(int interlace, int assign, double pik);

#ifdef __cplusplus
}
#endif

#endif
