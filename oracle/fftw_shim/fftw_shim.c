/*
 * fftw_shim.c -- double-precision FFT behind the FFTW-API subset that the
 * reference powspec uses (src/fftw_define.h:48-61).  Test infrastructure for
 * the oracle only; the GPU product never links it.
 *
 * Engine: Stockham autosort complex FFT (radix 4, 2, then odd prime factors
 * as generic radix-p DFT butterflies), FP64 twiddles from the definition
 * exp(-2 pi i m / n).  Real rows of even length use the half-length complex
 * transform with the standard even/odd split; odd lengths fall back to a
 * full-length complex transform.  Conventions follow FFTW: forward sign -1,
 * unnormalised, output layout [n0][n1][n2/2+1], c2r may clobber its input.
 * Pinned against numpy.fft (pocketfft) by tests/test_oracle_fft.py.
 */
#define _POSIX_C_SOURCE 200112L
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PS_MAXFAC 64
#define PS_COLBLK 16

static const double PS_TWO_PI = 6.283185307179586476925286766559;

typedef struct {
  int n;
  int nfac;
  int fac[PS_MAXFAC];
  double *tw; /* tw[2m], tw[2m+1] = cos(2 pi m/n), sin(2 pi m/n) */
} cplan;

struct ps_shim_plan {
  int n[3];
  int kind; /* 0: r2c, 1: c2r */
  cplan p0, p1, prow; /* axis-0, axis-1, last-axis (half length if even) */
  double *tw_row;     /* exp(2 pi i m / n2), m < n2, for the real-row split */
};

static int g_nthreads = 0;

static void twiddle_table(double *tw, int n) {
  for (int m = 0; m < n; m++) {
    /* Reduce to the nearest of m, n-m so the angle stays in [0, pi]. */
    int mm = (2 * m <= n) ? m : n - m;
    double a = PS_TWO_PI * (double)mm / (double)n;
    double c = cos(a), s = sin(a);
    tw[2 * m] = c;
    tw[2 * m + 1] = (2 * m <= n) ? s : -s;
  }
}

static int cplan_init(cplan *p, int n) {
  p->n = n;
  p->nfac = 0;
  p->tw = NULL;
  int m = n;
  while (m % 4 == 0 && p->nfac < PS_MAXFAC) { p->fac[p->nfac++] = 4; m /= 4; }
  while (m % 2 == 0 && p->nfac < PS_MAXFAC) { p->fac[p->nfac++] = 2; m /= 2; }
  for (int f = 3; (long)f * f <= m; f += 2)
    while (m % f == 0 && p->nfac < PS_MAXFAC) { p->fac[p->nfac++] = f; m /= f; }
  if (m > 1) p->fac[p->nfac++] = m;
  p->tw = malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
  if (!p->tw) return -1;
  twiddle_table(p->tw, n);
  return 0;
}

static void cplan_free(cplan *p) {
  free(p->tw);
  p->tw = NULL;
}

/* One radix-R Stockham pass: src -> dst.  sign = -1 forward, +1 backward. */
static void stockham_pass(const cplan *p, int R, int Ns, int sign,
                          const double *src, double *dst, double *vr,
                          double *vi, double *or_, double *oi) {
  const int n = p->n;
  const int m = n / R;
  const int tws = n / (Ns * R);
  const double *tw = p->tw;
  for (int j = 0; j < m; j++) {
    const int k = j % Ns;
    for (int r = 0; r < R; r++) {
      double xr = src[2 * (j + r * m)], xi = src[2 * (j + r * m) + 1];
      if (r && k) {
        int t = r * k * tws; /* < n */
        double c = tw[2 * t], s = sign * tw[2 * t + 1];
        double yr = xr * c - xi * s;
        double yi = xr * s + xi * c;
        xr = yr;
        xi = yi;
      }
      vr[r] = xr;
      vi[r] = xi;
    }
    if (R == 2) {
      or_[0] = vr[0] + vr[1]; oi[0] = vi[0] + vi[1];
      or_[1] = vr[0] - vr[1]; oi[1] = vi[0] - vi[1];
    } else if (R == 4) {
      double t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
      double t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
      double t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
      double dr = vr[1] - vr[3], di = vi[1] - vi[3];
      /* t3 = (v1 - v3) * (sign * i) */
      double t3r = -sign * di, t3i = sign * dr;
      or_[0] = t0r + t2r; oi[0] = t0i + t2i;
      or_[2] = t0r - t2r; oi[2] = t0i - t2i;
      or_[1] = t1r + t3r; oi[1] = t1i + t3i;
      or_[3] = t1r - t3r; oi[3] = t1i - t3i;
    } else {
      /* Generic radix-R DFT: out[q] = sum_r v[r] exp(sign 2 pi i r q / R). */
      const int step = n / R;
      for (int q = 0; q < R; q++) {
        double sr = 0, si = 0;
        for (int r = 0; r < R; r++) {
          int t = (int)(((long)r * q) % R) * step;
          double c = tw[2 * t], s = sign * tw[2 * t + 1];
          sr += vr[r] * c - vi[r] * s;
          si += vr[r] * s + vi[r] * c;
        }
        or_[q] = sr;
        oi[q] = si;
      }
    }
    const int base = (j / Ns) * Ns * R + k;
    for (int r = 0; r < R; r++) {
      dst[2 * (base + r * Ns)] = or_[r];
      dst[2 * (base + r * Ns) + 1] = oi[r];
    }
  }
}

/* In-place complex FFT of a (n interleaved pairs); work holds 2n + 4*maxR
 * doubles. */
static void cfft_exec(const cplan *p, double *a, double *work, int sign) {
  const int n = p->n;
  if (n <= 1) return;
  int maxr = 1;
  for (int f = 0; f < p->nfac; f++)
    if (p->fac[f] > maxr) maxr = p->fac[f];
  double *b = work;
  double *vr = work + 2 * n, *vi = vr + maxr, *or_ = vi + maxr, *oi = or_ + maxr;
  double *src = a, *dst = b;
  int Ns = 1;
  for (int f = 0; f < p->nfac; f++) {
    int R = p->fac[f];
    stockham_pass(p, R, Ns, sign, src, dst, vr, vi, or_, oi);
    Ns *= R;
    double *t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, sizeof(double) * 2 * n);
}

int ps_shim_cfft1d(int n, int sign, double *data) {
  cplan p;
  if (n < 1 || cplan_init(&p, n)) return -1;
  double *work = malloc(sizeof(double) * (2 * (size_t)n + 4 * (size_t)n + 16));
  if (!work) { cplan_free(&p); return -1; }
  cfft_exec(&p, data, work, sign < 0 ? -1 : 1);
  free(work);
  cplan_free(&p);
  return 0;
}

/* Real row (length n) -> half-complex row (n/2+1). */
static void row_r2c(const struct ps_shim_plan *pl, const double *x, double *X,
                    double *work) {
  const int n = pl->n[2];
  if (n % 2 == 0) {
    const int M = n / 2;
    for (int m = 0; m < M; m++) {
      X[2 * m] = x[2 * m];
      X[2 * m + 1] = x[2 * m + 1];
    }
    cfft_exec(&pl->prow, X, work, -1);
    const double *tw = pl->tw_row;
    double z0r = X[0], z0i = X[1];
    X[0] = z0r + z0i; X[1] = 0;
    X[2 * M] = z0r - z0i; X[2 * M + 1] = 0;
    for (int k = 1; 2 * k <= M; k++) {
      double ar = X[2 * k], ai = X[2 * k + 1];
      double br = X[2 * (M - k)], bi = X[2 * (M - k) + 1];
      /* E = (A + conj B)/2, O = -i/2 (A - conj B) */
      double er = 0.5 * (ar + br), ei = 0.5 * (ai - bi);
      double dr = ar - br, di = ai + bi; /* A - conj B */
      double orr = 0.5 * di, oi = -0.5 * dr;
      /* W^k = exp(-2 pi i k / n) */
      double c = tw[2 * k], s = -tw[2 * k + 1];
      double wor = orr * c - oi * s, woi = orr * s + oi * c;
      X[2 * k] = er + wor; X[2 * k + 1] = ei + woi;
      /* X[M-k] = conj(E) + W^{M-k} conj(O); W^{M-k} = -conj(W^k) */
      double c2 = -c, s2 = s;
      double cor = orr, coi = -oi;
      double wor2 = cor * c2 - coi * s2, woi2 = cor * s2 + coi * c2;
      X[2 * (M - k)] = er + wor2; X[2 * (M - k) + 1] = -ei + woi2;
    }
  } else {
    double *buf = work; /* n complex */
    for (int m = 0; m < n; m++) { buf[2 * m] = x[m]; buf[2 * m + 1] = 0; }
    cfft_exec(&pl->prow, buf, work + 2 * n, -1);
    for (int k = 0; k <= n / 2; k++) { X[2 * k] = buf[2 * k]; X[2 * k + 1] = buf[2 * k + 1]; }
  }
}

/* Half-complex row (n/2+1) -> real row (length n), unnormalised. */
static void row_c2r(const struct ps_shim_plan *pl, double *X, double *x,
                    double *work) {
  const int n = pl->n[2];
  if (n % 2 == 0) {
    const int M = n / 2;
    double *Z = work;
    double *w2 = work + 2 * (M + 1);
    const double *tw = pl->tw_row;
    X[1] = 0;
    X[2 * M + 1] = 0;
    for (int k = 0; k < M; k++) {
      double ar = X[2 * k], ai = X[2 * k + 1];
      double br = X[2 * (M - k)], bi = -X[2 * (M - k) + 1]; /* conj X[M-k] */
      double sr = ar + br, si = ai + bi;
      double dr = ar - br, di = ai - bi;
      /* W^{-k} = exp(+2 pi i k / n) */
      double c = tw[2 * k], s = tw[2 * k + 1];
      double tr = dr * c - di * s, ti = dr * s + di * c;
      /* Z = S + i T */
      Z[2 * k] = sr - ti;
      Z[2 * k + 1] = si + tr;
    }
    cfft_exec(&pl->prow, Z, w2, +1);
    for (int m = 0; m < M; m++) { x[2 * m] = Z[2 * m]; x[2 * m + 1] = Z[2 * m + 1]; }
  } else {
    double *buf = work;
    const int nk = n / 2 + 1;
    for (int k = 0; k < nk; k++) { buf[2 * k] = X[2 * k]; buf[2 * k + 1] = X[2 * k + 1]; }
    buf[1] = 0;
    for (int k = 1; k < nk; k++) {
      buf[2 * (n - k)] = X[2 * k];
      buf[2 * (n - k) + 1] = -X[2 * k + 1];
    }
    cfft_exec(&pl->prow, buf, work + 2 * n, +1);
    for (int m = 0; m < n; m++) x[m] = buf[2 * m];
  }
}

/* Complex FFTs along a strided axis of a half-complex 3-D array: `count`
 * independent lines of length len, element stride `stride` (complex units),
 * lines grouped as (outer, k) with base = o*ostride + k. */
static void axis_fft(const cplan *p, double *a, int len, size_t stride,
                     int nouter, size_t ostride, int nk, int sign) {
  const int nblk = (nk + PS_COLBLK - 1) / PS_COLBLK;
  const long total = (long)nouter * nblk;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_nthreads > 0 ? g_nthreads : omp_get_max_threads())
#endif
  {
    double *col = malloc(sizeof(double) * 2 * (size_t)len * PS_COLBLK);
    double *work = malloc(sizeof(double) * (2 * (size_t)len + 4 * (size_t)len + 16));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long t = 0; t < total; t++) {
      int o = (int)(t / nblk), b = (int)(t % nblk);
      int k0 = b * PS_COLBLK;
      int nb = (nk - k0 < PS_COLBLK) ? nk - k0 : PS_COLBLK;
      double *base = a + 2 * ((size_t)o * ostride + k0);
      for (int j = 0; j < len; j++) {
        const double *row = base + 2 * (size_t)j * stride;
        for (int c = 0; c < nb; c++) {
          col[2 * ((size_t)c * len + j)] = row[2 * c];
          col[2 * ((size_t)c * len + j) + 1] = row[2 * c + 1];
        }
      }
      for (int c = 0; c < nb; c++) cfft_exec(p, col + 2 * (size_t)c * len, work, sign);
      for (int j = 0; j < len; j++) {
        double *row = base + 2 * (size_t)j * stride;
        for (int c = 0; c < nb; c++) {
          row[2 * c] = col[2 * ((size_t)c * len + j)];
          row[2 * c + 1] = col[2 * ((size_t)c * len + j) + 1];
        }
      }
    }
    free(col);
    free(work);
  }
}

void *fftw_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 64)) return NULL;
  return p;
}

void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { g_nthreads = nthreads; }
void fftw_cleanup_threads(void) {}
void fftw_cleanup(void) {}

static fftw_plan plan_3d(int n0, int n1, int n2, int kind) {
  if (n0 < 1 || n1 < 1 || n2 < 1) return NULL;
  struct ps_shim_plan *pl = calloc(1, sizeof *pl);
  if (!pl) return NULL;
  pl->n[0] = n0; pl->n[1] = n1; pl->n[2] = n2;
  pl->kind = kind;
  int rowlen = (n2 % 2 == 0) ? n2 / 2 : n2;
  if (cplan_init(&pl->p0, n0) || cplan_init(&pl->p1, n1) ||
      cplan_init(&pl->prow, rowlen)) {
    fftw_destroy_plan(pl);
    return NULL;
  }
  pl->tw_row = malloc(sizeof(double) * 2 * (size_t)n2);
  if (!pl->tw_row) { fftw_destroy_plan(pl); return NULL; }
  twiddle_table(pl->tw_row, n2);
  return pl;
}

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags) {
  (void)in; (void)out; (void)flags;
  return plan_3d(n0, n1, n2, 0);
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags) {
  (void)in; (void)out; (void)flags;
  return plan_3d(n0, n1, n2, 1);
}

void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  cplan_free(&p->p0);
  cplan_free(&p->p1);
  cplan_free(&p->prow);
  free(p->tw_row);
  free(p);
}

void fftw_execute_dft_r2c(const fftw_plan pl, double *in, fftw_complex *out) {
  const int n0 = pl->n[0], n1 = pl->n[1], n2 = pl->n[2];
  const int nk = n2 / 2 + 1;
  double *o = (double *)out;
  const long rows = (long)n0 * n1;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_nthreads > 0 ? g_nthreads : omp_get_max_threads())
#endif
  {
    double *work = malloc(sizeof(double) * (10 * (size_t)n2 + 32));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long r = 0; r < rows; r++)
      row_r2c(pl, in + (size_t)r * n2, o + 2 * (size_t)r * nk, work);
    free(work);
  }
  /* axis 1: lines over j for each (i, k) */
  axis_fft(&pl->p1, o, n1, (size_t)nk, n0, (size_t)n1 * nk, nk, -1);
  /* axis 0: lines over i for each (j, k) */
  axis_fft(&pl->p0, o, n0, (size_t)n1 * nk, n1, (size_t)nk, nk, -1);
}

void fftw_execute_dft_c2r(const fftw_plan pl, fftw_complex *in, double *out) {
  const int n0 = pl->n[0], n1 = pl->n[1], n2 = pl->n[2];
  const int nk = n2 / 2 + 1;
  double *a = (double *)in;
  axis_fft(&pl->p0, a, n0, (size_t)n1 * nk, n1, (size_t)nk, nk, +1);
  axis_fft(&pl->p1, a, n1, (size_t)nk, n0, (size_t)n1 * nk, nk, +1);
  const long rows = (long)n0 * n1;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_nthreads > 0 ? g_nthreads : omp_get_max_threads())
#endif
  {
    double *work = malloc(sizeof(double) * (10 * (size_t)n2 + 32));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long r = 0; r < rows; r++)
      row_c2r(pl, a + 2 * (size_t)r * nk, out + (size_t)r * n2, work);
    free(work);
  }
}
