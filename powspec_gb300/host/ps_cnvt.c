/*
 * ps_cnvt.c -- (RA, Dec, redshift) -> Cartesian comoving coordinates
 * (src/cnvt_coord.c).
 *
 * The radial comoving distance (Mpc/h) of redshift z is
 *   D(z) = c/(100 km/s) * integral_0^z dz' / E(z'),
 *   E^2 = Omega_m (1+z)^3 + Omega_k (1+z)^2 + Omega_L (1+z)^(3(1+w))
 * (src/cnvt_coord.c:295-306), evaluated either by Gauss-Legendre
 * quadrature of one order for every object, the smallest order at which 128
 * redshifts spread evenly over the catalogues' range converge to CMVDST_ERR
 * between successive orders (src/cnvt_coord.c:153-281, :359-400), or by
 * natural cubic-spline interpolation of a (z, D) table (Z_CMVDST_CNVT,
 * src/cnvt_coord.c:81-151).  Then x = D cos(Dec) cos(RA),
 * y = D cos(Dec) sin(RA), z = D sin(Dec) (src/cnvt_coord.c:122-151).
 *
 * The quadrature nodes and weights are computed here by Newton iteration
 * on the Legendre polynomial P_n (the standard method, e.g. Press et al.,
 * Numerical Recipes, section 4.6); the spline is the usual natural cubic
 * spline from its tridiagonal system.
 */
#define _DEFAULT_SOURCE
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "ps_host.h"

#define CNVT_C_100 2997.92458                   /* speed of light / (100 km/s), Mpc/h */
#define CNVT_DEG 0.017453292519943295769        /* pi / 180 */
#define CNVT_MIN_ORDER 4
#define CNVT_MAX_ORDER 32
#define CNVT_NSAMPLE 128

/* ------------------------------------------------------ Gauss-Legendre */

/* Nodes x_k > 0 (k < n/2, descending) and weights, plus the weight of the
 * node 0 for odd n (at index n/2). */
static void legauss(int n, double *x, double *w) {
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), z1, pp = 0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) <= 1e-16 * fabs(z) + 1e-300) break;
    }
    x[i] = z;
    w[i] = 2 / ((1 - z * z) * pp * pp);
  }
  if (n & 1) x[n / 2] = 0;  /* the middle node: z converges to 0 */
}

static double integrand(const psh_cosmo *c, double z) {
  const double z1 = z + 1, z2 = z1 * z1;
  double d = c->omega_m * z2 * z1;
  if (c->omega_k != 0) d += c->omega_k * z2;
  d += (c->widx != 0) ? c->omega_l * pow(z1, c->widx) : c->omega_l;
  return CNVT_C_100 / sqrt(d);
}

static double quad(const psh_cosmo *c, int n, const double *x, const double *w, double z) {
  const double zp = z * 0.5;
  double s = 0;
  for (int k = 0; k < n / 2; k++)
    s += w[k] * (integrand(c, zp * (1 + x[k])) + integrand(c, zp * (1 - x[k])));
  if (n & 1) s += w[n / 2] * integrand(c, zp);
  return s * zp;
}

/* ----------------------------------------------------------- the spline */

static int spline_setup(psh_cosmo *c) {
  const size_t n = c->ntab;
  if (n < 2) return PSH_ERR_CFG;
  for (size_t i = 1; i < n; i++)
    if (!(c->tz[i] > c->tz[i - 1])) {
      fprintf(stderr, "Error: the redshifts of `Z_CMVDST_CNVT' must increase\n");
      return PSH_ERR_CFG;
    }
  c->typp = calloc(n, sizeof(double));
  double *u = calloc(n, sizeof(double));
  if (!c->typp || !u) {
    free(u);
    return PSH_ERR_MEMORY;
  }
  /* natural spline: y''(ends) = 0; tridiagonal system, forward sweep */
  for (size_t i = 1; i + 1 < n; i++) {
    const double h0 = c->tz[i] - c->tz[i - 1], h1 = c->tz[i + 1] - c->tz[i];
    const double sig = h0 / (h0 + h1), p = sig * c->typp[i - 1] + 2;
    c->typp[i] = (sig - 1) / p;
    const double dy = (c->td[i + 1] - c->td[i]) / h1 - (c->td[i] - c->td[i - 1]) / h0;
    u[i] = (6 * dy / (h0 + h1) - sig * u[i - 1]) / p;
  }
  c->typp[n - 1] = 0;
  for (size_t k = n - 1; k-- > 0;) c->typp[k] = c->typp[k] * c->typp[k + 1] + u[k];
  c->typp[0] = 0;
  free(u);
  return 0;
}

static double spline_eval(const psh_cosmo *c, double z) {
  const size_t n = c->ntab;
  if (!(z >= c->tz[0] && z < c->tz[n - 1])) return HUGE_VAL;
  size_t lo = 0, hi = n - 1;  /* tz[lo] <= z < tz[hi] */
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    if (c->tz[mid] <= z) lo = mid;
    else hi = mid;
  }
  const double h = c->tz[hi] - c->tz[lo], a = (c->tz[hi] - z) / h, b = (z - c->tz[lo]) / h;
  return a * c->td[lo] + b * c->td[hi] +
         ((a * a * a - a) * c->typp[lo] + (b * b * b - b) * c->typp[hi]) * (h * h) / 6;
}

static int read_table(psh_cosmo *c, const char *fname) {
  FILE *fp = fopen(fname, "r");
  if (!fp) {
    fprintf(stderr, "Error: cannot open `Z_CMVDST_CNVT': `%s'\n", fname);
    return PSH_ERR_FILE;
  }
  size_t cap = 1024;
  c->tz = malloc(sizeof(double) * cap);
  c->td = malloc(sizeof(double) * cap);
  char line[4096];
  int rc = (c->tz && c->td) ? 0 : PSH_ERR_MEMORY;
  while (!rc && fgets(line, sizeof line, fp)) {
    const char *s = line;
    while (*s == ' ' || *s == '\t') s++;
    if (*s == '#' || *s == '\n' || *s == '\0' || *s == '\r') continue;
    char *e;
    const double z = psh_strtod(s, &e);
    if (e == s) {
      fprintf(stderr, "Error: cannot read line `%s' of `%s'\n", line, fname);
      rc = PSH_ERR_FILE;
      break;
    }
    s = e;
    const double d = psh_strtod(s + strspn(s, " \t,"), &e);
    if (e == s + strspn(s, " \t,")) {
      fprintf(stderr, "Error: cannot read line `%s' of `%s'\n", line, fname);
      rc = PSH_ERR_FILE;
      break;
    }
    if (c->ntab == cap) {
      cap *= 2;
      double *nz = realloc(c->tz, sizeof(double) * cap), *nd = nz ? realloc(c->td, sizeof(double) * cap) : NULL;
      if (nz) c->tz = nz;
      if (!nz || !nd) {
        rc = PSH_ERR_MEMORY;
        break;
      }
      c->td = nd;
    }
    c->tz[c->ntab] = z;
    c->td[c->ntab] = d;
    c->ntab++;
  }
  fclose(fp);
  if (!rc) rc = spline_setup(c);
  return rc;
}

/* ------------------------------------------------------------- interface */

int psh_cosmo_init(psh_cosmo *c, const char *table, double zmin, double zmax, bool verbose) {
  if (table) {
    const int rc = read_table(c, table);
    if (!rc && verbose)
      printf("  %zu comoving distance samples read from `%s'\n", c->ntab, table);
    return rc;
  }
  c->widx = (c->eos_w == -1) ? 0 : 3 * (1 + c->eos_w);
  if (!(zmin <= zmax)) {
    fprintf(stderr, "Error: invalid redshift value in the catalogs\n");
    return PSH_ERR_CATA;
  }
  int order = 0;
  for (int i = 0; i < CNVT_NSAMPLE; i++) {
    const double z = zmin + i * (zmax - zmin) / (CNVT_NSAMPLE - 1);
    double prev, cur = 0;
    int n = CNVT_MIN_ORDER - 1;
    do {
      if (++n > CNVT_MAX_ORDER) {
        fprintf(stderr, "Error: failed to perform the convergency test for integrations\n");
        return PSH_ERR_CATA;
      }
      prev = cur;
      legauss(n, c->x, c->w);
      cur = quad(c, n, c->x, c->w, z);
    } while (fabs(cur - prev) > cur * c->err);
    if (order < n) order = n;
  }
  c->order = order;
  legauss(order, c->x, c->w);
  if (verbose)
    printf("  Legendre-Gauss order %d chosen for the integration error %g\n", order, c->err);
  return 0;
}

void psh_cosmo_free(psh_cosmo *c) {
  free(c->tz);
  free(c->td);
  free(c->typp);
  c->tz = c->td = c->typp = NULL;
  c->ntab = 0;
}

double psh_cosmo_distance(const psh_cosmo *c, double z) {
  return c->ntab ? spline_eval(c, z) : quad(c, c->order, c->x, c->w, z);
}

typedef struct {
  const psh_cosmo *c;
  double *xyzw;
  size_t beg, end;
} CnvtPart;

static void *cnvt_part(void *arg) {
  CnvtPart *p = arg;
  for (size_t i = p->beg; i < p->end; i++) {
    double *r = p->xyzw + 4 * i;
    const double ra = r[0] * CNVT_DEG, dec = r[1] * CNVT_DEG;
    const double dist = psh_cosmo_distance(p->c, r[2]);
    r[0] = dist * cos(dec) * cos(ra);
    r[1] = dist * cos(dec) * sin(ra);
    r[2] = dist * sin(dec);
  }
  return NULL;
}

void psh_cosmo_convert(const psh_cosmo *c, double *xyzw, size_t n, int nthread) {
  long t = nthread;
  if (t <= 0) {  /* OMP_NUM_THREADS, else the online cores */
    const char *e = getenv("OMP_NUM_THREADS");
    t = (e && *e) ? strtol(e, NULL, 10) : 0;
    if (t <= 0) t = sysconf(_SC_NPROCESSORS_ONLN);
    if (t <= 0) t = 1;
  }
  if (t > 64) t = 64;
  if ((size_t)t > n / 4096 + 1) t = (long)(n / 4096 + 1);
  CnvtPart part[64];
  pthread_t th[64];
  int up[64] = {0};
  for (int i = 0; i < t; i++) {
    part[i].c = c;
    part[i].xyzw = xyzw;
    part[i].beg = n / (size_t)t * (size_t)i;
    part[i].end = i + 1 < t ? n / (size_t)t * (size_t)(i + 1) : n;
  }
  for (int i = 1; i < t; i++) {
    up[i] = pthread_create(&th[i], NULL, cnvt_part, &part[i]) == 0;
    if (!up[i]) cnvt_part(&part[i]);
  }
  cnvt_part(&part[0]);
  for (int i = 1; i < t; i++)
    if (up[i]) pthread_join(th[i], NULL);
}
