/*
 * ps_host.h -- the command-line program of the GB300 periodic-box path.
 *
 * Keeps powspec's interface for the simulation-box case: the configuration
 * file keywords and command-line options (src/load_conf.c:366-417), the ASCII
 * catalogue reader's formatter / column / expression semantics
 * (io/read_ascii.c) -- plus NumPy .npy catalogues -- and the output file
 * format (src/save_res.c:35-229).
 * The estimator itself runs through the C ABI of include/powspec_gpu.h.
 */
#ifndef PS_HOST_H
#define PS_HOST_H

#include <stdbool.h>
#include <stddef.h>

/* Exit codes: the reference's POWSPEC_ERR_* (src/define.h:112-124). */
#define PSH_ERR_MEMORY (-1)
#define PSH_ERR_ARG (-2)
#define PSH_ERR_FILE (-3)
#define PSH_ERR_CFG (-4)
#define PSH_ERR_AST (-5)
#define PSH_ERR_ASCII (-6)
#define PSH_ERR_CONF (-10)
#define PSH_ERR_CATA (-11)

/* ---- configuration: raw string values per keyword, typed on access ---- */
enum { PSH_SRC_NONE = 0, PSH_SRC_FILE = 1, PSH_SRC_CMD = 5 };

typedef struct {
  char sopt;          /* short option, 0 if none */
  const char *lopt;   /* long option */
  const char *key;    /* configuration keyword */
  int array;          /* accepts several values */
  /* value */
  int src;            /* PSH_SRC_*: command line has priority over the file */
  int n;
  char **val;
} psh_opt;

typedef struct {
  psh_opt *opt;
  int nopt;
} psh_cfg;

int psh_cfg_init(psh_cfg *c);
void psh_cfg_free(psh_cfg *c);
/* Command line: -h / --help and -t / --template print and return 1. */
int psh_cfg_cmdline(psh_cfg *c, int argc, char **argv);
int psh_cfg_file(psh_cfg *c, const char *fname);
psh_opt *psh_cfg_get(psh_cfg *c, const char *key);
int psh_size(psh_cfg *c, const char *key);
const char *psh_str(psh_cfg *c, const char *key, int i);
int psh_int(psh_cfg *c, const char *key, int i, long *out);
int psh_dbl(psh_cfg *c, const char *key, int i, double *out);
int psh_bool(psh_cfg *c, const char *key, int i, bool *out);

/* ---- expressions over catalogue columns ($n, ${n}) ---- */
typedef struct psh_expr psh_expr;
/* Compiles src; *maxcol receives the largest column referenced. */
psh_expr *psh_expr_compile(const char *src, int *maxcol, char *err, size_t errlen);
double psh_expr_eval(const psh_expr *e, const double *col);
void psh_expr_free(psh_expr *e);
/* The 0-based column an expression is made of alone ($n), else -1. */
int psh_expr_column(const psh_expr *e);

/* ---- catalogues ---- */
typedef struct {
  const char *fname;
  long skip;          /* ASCII: header lines dropped */
  char comment;       /* ASCII: '\0': no comment lines */
  const char *fmtr;   /* ASCII: scanf-style formatter */
  const char *pos[3];
  const char *wcomp;  /* NULL: unit weights */
  const char *sel;    /* NULL: no selection */
  int nthread;        /* host threads; 0: OMP_NUM_THREADS, else the online cores */
  /* survey catalogues (CUBIC_SIM = F): record weight = completeness x FKP
   * weight; sums as io/read_ascii.c:880-895 */
  int survey;
  const char *wfkp;   /* NULL: 1 */
  const char *nz;     /* NULL: 0 */
  double *sumw2;      /* out: sum of (wc wfkp)^2 (surveys) */
  double *sumw2n;     /* out: sum of wc wfkp^2 nz (surveys) */
} psh_catalog;

/* Reads an ASCII catalogue (DATA_FORMAT = 0) into *xyzw ({x, y, z, w}
 * records in file order), sets *n and *wsum (the sum of the completeness
 * weights, in file order). */
int psh_read_ascii(const psh_catalog *in, double **xyzw, size_t *n, double *wsum, bool verbose);
/* Reads a NumPy .npy array (DATA_FORMAT = 2): 1-D or 2-D, f4 / f8 / i4 / i8
 * of either byte order, C or Fortran order; the columns of a row are $1,
 * $2, ... of the expressions.  skip, comment and fmtr are not used. */
int psh_read_npy(const psh_catalog *in, double **xyzw, size_t *n, double *wsum, bool verbose);
/* Decimal string to double with strtod's syntax and correct rounding. */
double psh_strtod(const char *s, char **end);

/* ---- coordinate conversion: (RA, Dec, z) -> comoving Cartesian ---- */
typedef struct {
  double omega_m, omega_l, omega_k, eos_w;  /* OMEGA_M, OMEGA_LAMBDA, DE_EOS_W */
  double err;                               /* CMVDST_ERR */
  double widx;                              /* 3 (1 + w), 0 for w = -1 */
  int order;                                /* Gauss-Legendre order chosen */
  double x[32], w[32];                      /* its nodes and weights */
  double *tz, *td, *typp;                   /* Z_CMVDST_CNVT table and spline */
  size_t ntab;
} psh_cosmo;

/* Interpolation table `table` (or NULL: quadrature, its order chosen on
 * the redshift range [zmin, zmax]). */
int psh_cosmo_init(psh_cosmo *c, const char *table, double zmin, double zmax, bool verbose);
void psh_cosmo_free(psh_cosmo *c);
double psh_cosmo_distance(const psh_cosmo *c, double z);
/* {RA deg, Dec deg, z, w} records -> {x, y, z, w} in place. */
void psh_cosmo_convert(const psh_cosmo *c, double *xyzw, size_t n, int nthread);

#endif
