/*
 * ps_main.c -- powspec's command-line program for periodic simulation boxes,
 * with the estimator on the GPU through include/powspec_gpu.h.
 *
 * Flow of the reference's main (src/powspec.c:47-103): load and check the
 * configuration (src/load_conf.c:876-1130), read the catalogues, build the
 * meshes and evaluate the power spectrum multipoles, save the results
 * (src/save_res.c:35-229, same header lines, columns and number formats).
 * Survey catalogues (CUBIC_SIM = F): data minus alpha x randoms with FKP
 * weights in a box fitted to the catalogues (src/read_cata.c:95-185,
 * src/genr_mesh.c:427-566, :797-809), from Cartesian or converted (RA, Dec,
 * z) coordinates; multipoles l > 0 by the spherical-harmonic decomposition,
 * with or without interlacing.  FITS catalogues are rejected with an error.  Besides
 * ASCII (DATA_FORMAT = 0), DATA_FORMAT = 2 reads NumPy .npy arrays, whose
 * columns take the same position / weight / selection expressions.
 */
#define _POSIX_C_SOURCE 200809L
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "powspec_gpu.h"
#include "ps_host.h"

#define OFMT_DBL "%.10lg"

typedef struct {
  bool issim, intlace, logscale, oheader, verbose, isauto[2], iscross;
  int ndata, gsize, assign, npole, poles[7];
  int dfmt[2], rfmt[2];  /* DATA_FORMAT, RAND_FORMAT: 0 ASCII, 2 NumPy .npy */
  double bmin[3];        /* lower box corner: 0 for simulation boxes */
  double bpad[3];        /* BOX_PAD (surveys without BOX_SIZE) */
  bool bset;             /* BOX_SIZE given */
  bool cnvt, dcnvt[2], rcnvt[2];  /* coordinate conversion (surveys) */
  const char *ztab;               /* Z_CMVDST_CNVT */
  psh_cosmo cosmo;
  long ovwrite;
  double bsize[3], los[3], kmin, kmax, kbin;
  const char *oauto[2], *ocross;
} Conf;

static const char *kAssignNames[] = {"NGP", "CIC", "TSC", "PCS"};

/* Existing output files: OVERWRITE = 0 refuses, > 0 overwrites, < 0 asks
 * up to |OVERWRITE| times (src/load_conf.c:478-535). */
static int check_output(const char *fname, const char *key, long ovwrite) {
  if (!fname || !*fname) {
    fprintf(stderr, "Error: the output `%s' is not set\n", key);
    return PSH_ERR_CFG;
  }
  if (!access(fname, F_OK)) {
    if (ovwrite == 0) {
      fprintf(stderr, "Error: the output `%s' exists: `%s'\n", key, fname);
      return PSH_ERR_FILE;
    } else if (ovwrite > 0) {
      fprintf(stderr, "Warning: the output `%s' will be overwritten: `%s'\n", key, fname);
    } else {
      fprintf(stderr, "Warning: the output `%s' exists: `%s'\n", key, fname);
      char confirm = 0;
      for (long i = 0; i != ovwrite; i--) {
        fprintf(stderr, "Are you going to overwrite it? (y/n): ");
        if (scanf("%c", &confirm) != 1) continue;
        int ch;
        while ((ch = getchar()) != '\n' && ch != EOF) continue;
        if (confirm == 'n') {
          fprintf(stderr, "Error: cannot write to the file\n");
          return PSH_ERR_FILE;
        } else if (confirm == 'y') {
          break;
        }
      }
      if (confirm != 'y') {
        fprintf(stderr, "Error: too many failed inputs\n");
        return PSH_ERR_FILE;
      }
    }
    if (access(fname, W_OK)) {
      fprintf(stderr, "Error: cannot write to file `%s'\n", fname);
      return PSH_ERR_FILE;
    }
  }
  return 0;
}

/* Reads catalogue i of `which` (DATA or RAND) with its keywords.  Surveys
 * take FKP weights and n(z) too (io/read_ascii.c:880-895). */
static int read_cat(psh_cfg *cfg, const Conf *c, const char *which, int i, int fmt,
                    double **xyzw, size_t *n, double *wsum, double *sumw2, double *sumw2n) {
  char key[32];
  psh_catalog in;
  memset(&in, 0, sizeof in);
#define K(name) (snprintf(key, sizeof key, "%s_" name, which), key)
  in.fname = psh_str(cfg, K("CATALOG"), i);
  long skip = 0;
  if (psh_int(cfg, K("SKIP"), i, &skip) < 0 || skip < 0) return PSH_ERR_CONF;
  in.skip = skip;
  const char *cm = psh_str(cfg, K("COMMENT"), i);
  in.comment = cm ? cm[0] : '\0';
  in.fmtr = psh_str(cfg, K("FORMATTER"), i);
  for (int d = 0; d < 3; d++) in.pos[d] = psh_str(cfg, K("POSITION"), 3 * i + d);
  in.wcomp = psh_str(cfg, K("WT_COMP"), i);
  in.sel = psh_str(cfg, K("SELECTION"), i);
  if (!c->issim) {
    in.survey = 1;
    in.wfkp = psh_str(cfg, K("WT_FKP"), i);
    in.nz = psh_str(cfg, K("NZ"), i);
    in.sumw2 = sumw2;
    in.sumw2n = sumw2n;
  }
#undef K
  if (in.sel && !*in.sel) in.sel = NULL;
  if (in.wcomp && !*in.wcomp) in.wcomp = NULL;
  if (in.wfkp && !*in.wfkp) in.wfkp = NULL;
  if (in.nz && !*in.nz) in.nz = NULL;
  int rc = fmt == 2 ? psh_read_npy(&in, xyzw, n, wsum, c->verbose)
                    : psh_read_ascii(&in, xyzw, n, wsum, c->verbose);
  if (!rc && *n == 0) {
    fprintf(stderr, "Error: no object read from `%s'\n", in.fname);
    rc = PSH_ERR_CATA;
  }
  return rc;
}

/* Cosmology of the coordinate conversion (src/load_conf.c:746-785, :970-987). */
static int check_cosmo(psh_cfg *cfg, Conf *c) {
  psh_cosmo *k = &c->cosmo;
  memset(k, 0, sizeof *k);
  for (int i = 0; i < 2; i++) {
    c->dcnvt[i] = c->rcnvt[i] = false;
    if (psh_size(cfg, "DATA_CONVERT") > i && psh_bool(cfg, "DATA_CONVERT", i, &c->dcnvt[i]))
      return PSH_ERR_CFG;
    if (psh_size(cfg, "RAND_CONVERT") > i && psh_bool(cfg, "RAND_CONVERT", i, &c->rcnvt[i]))
      return PSH_ERR_CFG;
  }
  c->ztab = psh_str(cfg, "Z_CMVDST_CNVT", 0);
  if (c->ztab && *c->ztab) {
    if (access(c->ztab, R_OK)) {
      fprintf(stderr, "Error: cannot access `Z_CMVDST_CNVT': `%s'\n", c->ztab);
      return PSH_ERR_FILE;
    }
    return 0;
  }
  c->ztab = NULL;
  int rc = psh_dbl(cfg, "OMEGA_M", 0, &k->omega_m);
  if (rc) {
    if (rc == 1) fprintf(stderr, "Error: `OMEGA_M' is not set\n");
    return PSH_ERR_CFG;
  }
  if (k->omega_m <= 0 || k->omega_m > 1) {
    fprintf(stderr, "Error: `OMEGA_M' must be > 0 and <= 1\n");
    return PSH_ERR_CFG;
  }
  if ((rc = psh_dbl(cfg, "OMEGA_LAMBDA", 0, &k->omega_l)) < 0) return PSH_ERR_CFG;
  if (rc) {
    k->omega_l = 1 - k->omega_m;
    k->omega_k = 0;
  } else if (k->omega_l < 0) {
    fprintf(stderr, "Error: `OMEGA_LAMBDA' must be >= 0\n");
    return PSH_ERR_CFG;
  } else {
    k->omega_k = 1 - k->omega_m - k->omega_l;
  }
  if ((rc = psh_dbl(cfg, "DE_EOS_W", 0, &k->eos_w)) < 0) return PSH_ERR_CFG;
  if (rc) k->eos_w = -1;
  else if (k->eos_w > -1 / 3.0) {
    fprintf(stderr, "Error: `DE_EOS_W' must be <= -1/3\n");
    return PSH_ERR_CFG;
  }
  const double w3 = k->eos_w * 3, wi = w3 + 1;  /* H^2(z) > 0 */
  if (k->omega_k * pow(k->omega_l * (-wi), wi / w3) <= k->omega_l * w3 * pow(k->omega_m, wi / w3)) {
    fprintf(stderr, "Error: negative H^2 given the cosmological parameters\n");
    return PSH_ERR_CFG;
  }
  if ((rc = psh_dbl(cfg, "CMVDST_ERR", 0, &k->err)) < 0) return PSH_ERR_CFG;
  if (rc) k->err = 1e-8;  /* DEFAULT_CMVDST_ERR */
  else if (k->err < DBL_EPSILON) {
    fprintf(stderr, "Error: `CMVDST_ERR' is smaller than the machine epsilon\n");
    return PSH_ERR_CFG;
  }
  return 0;
}

/* Format, readability and formatter of the DATA or RAND catalogues. */
static int check_files(psh_cfg *cfg, const Conf *c, const char *which, int *fmt) {
  char key[32];
  for (int i = 0; i < c->ndata; i++) {
    long t = 0;
    snprintf(key, sizeof key, "%s_FORMAT", which);
    if (psh_int(cfg, key, i, &t) < 0) return PSH_ERR_CFG;
    if (t == 1) {
      fprintf(stderr, "Error: FITS format is not enabled\n");
      return PSH_ERR_CFG;
    }
    if (t != 0 && t != 2) {
      fprintf(stderr, "Error: invalid `%s': %ld (0: ASCII, 2: NumPy .npy)\n", key, t);
      return PSH_ERR_CFG;
    }
    fmt[i] = (int)t;
    snprintf(key, sizeof key, "%s_CATALOG", which);
    const char *fn = psh_str(cfg, key, i);
    if (access(fn, R_OK)) {
      fprintf(stderr, "Error: cannot access `%s': `%s'\n", key, fn);
      return PSH_ERR_FILE;
    }
    snprintf(key, sizeof key, "%s_FORMATTER", which);
    if (t == 0 && psh_size(cfg, key) <= i) {
      fprintf(stderr, "Error: %s of `%s'\n", psh_size(cfg, key) ? "too few elements" : "not set",
              key);
      return PSH_ERR_CFG;
    }
  }
  snprintf(key, sizeof key, "%s_POSITION", which);
  if (psh_size(cfg, key) < 3 * c->ndata) {
    fprintf(stderr, "Error: %s `%s'\n", psh_size(cfg, key) ? "too few elements of" : "not set:",
            key);
    return PSH_ERR_CFG;
  }
  return 0;
}

static int verify(psh_cfg *cfg, Conf *c) {
  int rc;
  if ((rc = psh_bool(cfg, "CUBIC_SIM", 0, &c->issim))) {
    if (rc == 1) fprintf(stderr, "Error: `CUBIC_SIM' is not set\n");
    return PSH_ERR_CFG;
  }
  /* coordinate conversion: needed when DATA_CONVERT or RAND_CONVERT is set
   * at all (src/load_conf.c:949-968); each catalogue is converted by its
   * own value */
  c->cnvt = !c->issim && (psh_size(cfg, "DATA_CONVERT") || psh_size(cfg, "RAND_CONVERT"));
  if (c->cnvt && (rc = check_cosmo(cfg, c))) return rc;
  c->ovwrite = 0;
  if (psh_int(cfg, "OVERWRITE", 0, &c->ovwrite) < 0) return PSH_ERR_CFG;
  c->iscross = false;
  c->ndata = 0;
  const char *oc = psh_str(cfg, "OUTPUT_CROSS", 0);
  if (oc && *oc) {
    if ((rc = check_output(oc, "OUTPUT_CROSS", c->ovwrite))) return rc;
    c->iscross = true;
    c->ocross = oc;
    c->ndata = 2;
  }
  c->isauto[0] = c->isauto[1] = false;
  int num = psh_size(cfg, "OUTPUT_AUTO");
  if (num) {
    if (!c->iscross) c->ndata = num > 2 ? 2 : num;
    if (num > 2) {
      fprintf(stderr, "Warning: omitting the following `OUTPUT_AUTO':\n");
      for (int i = 2; i < num; i++) fprintf(stderr, "%s\n", psh_str(cfg, "OUTPUT_AUTO", i));
      num = 2;
    }
    for (int i = 0; i < num; i++) {
      const char *o = psh_str(cfg, "OUTPUT_AUTO", i);
      if (o[0]) {
        if ((rc = check_output(o, "OUTPUT_AUTO", c->ovwrite))) return rc;
        c->isauto[i] = true;
        c->oauto[i] = o;
      }
    }
  }
  if (!c->ndata) {
    fprintf(stderr, "Error: no output file specified\n");
    return PSH_ERR_CFG;
  }
  const int nd = psh_size(cfg, "DATA_CATALOG");
  if (!nd) {
    fprintf(stderr, "Error: `DATA_CATALOG' is not set\n");
    return PSH_ERR_CFG;
  }
  if (nd < c->ndata) {
    fprintf(stderr, "Error: too few elements of `DATA_CATALOG' (`OUTPUT_AUTO' or "
                    "`OUTPUT_CROSS' may require more catalogs)\n");
    return PSH_ERR_CFG;
  }
  if ((rc = check_files(cfg, c, "DATA", c->dfmt))) return rc;
  if (!c->issim) {
    if (psh_size(cfg, "RAND_CATALOG") < c->ndata) {
      fprintf(stderr, "Error: %s `RAND_CATALOG'\n",
              psh_size(cfg, "RAND_CATALOG") ? "too few elements of" : "not set:");
      return PSH_ERR_CFG;
    }
    if ((rc = check_files(cfg, c, "RAND", c->rfmt))) return rc;
    if (!psh_size(cfg, "DATA_NZ") && !psh_size(cfg, "RAND_NZ")) {
      fprintf(stderr, "Error: `DATA_NZ' and `RAND_NZ' are both not set\n");
      return PSH_ERR_CFG;
    }
  }
  /* LINE_OF_SIGHT: unit vector, default [0, 0, 1] (simulation boxes) */
  num = c->issim ? psh_size(cfg, "LINE_OF_SIGHT") : 0;
  c->los[0] = c->los[1] = 0;
  c->los[2] = 1;
  if (num) {
    if (num != 3) {
      fprintf(stderr, "Error: `LINE_OF_SIGHT' must be a 3-element array\n");
      return PSH_ERR_CFG;
    }
    for (int d = 0; d < 3; d++)
      if (psh_dbl(cfg, "LINE_OF_SIGHT", d, &c->los[d])) return PSH_ERR_CFG;
    const double t = c->los[0] * c->los[0] + c->los[1] * c->los[1] + c->los[2] * c->los[2];
    if (t < 1 - 1e-8 || t > 1 + 1e-8) {
      fprintf(stderr, "Error: `LINE_OF_SIGHT' must be a unit vector\n");
      return PSH_ERR_CFG;
    }
  }
  /* BOX_SIZE: 1 or 3 positive values; surveys without it fit the box to
   * the catalogues with BOX_PAD (src/load_conf.c:798-850) */
  num = psh_size(cfg, "BOX_SIZE");
  c->bset = num > 0;
  if (!num && c->issim) {
    fprintf(stderr, "Error: `BOX_SIZE' is not set\n");
    return PSH_ERR_CFG;
  }
  if (num && num != 1 && num != 3) {
    fprintf(stderr, "Error: wrong dimension of `BOX_SIZE'");
    return PSH_ERR_CFG;
  }
  for (int d = 0; d < 3 && num; d++) {
    if (psh_dbl(cfg, "BOX_SIZE", num == 1 ? 0 : d, &c->bsize[d])) return PSH_ERR_CFG;
    if (c->bsize[d] <= 0) {
      fprintf(stderr, "Error: `BOX_SIZE' must be > 0\n");
      return PSH_ERR_CFG;
    }
  }
  if (!num) {
    const int np = psh_size(cfg, "BOX_PAD");
    if (np && np != 1 && np != 3) {
      fprintf(stderr, "Error: wrong dimension of `BOX_PAD'");
      return PSH_ERR_CFG;
    }
    for (int d = 0; d < 3; d++) {
      c->bpad[d] = 0.02;  /* DEFAULT_BOX_PAD */
      if (np && psh_dbl(cfg, "BOX_PAD", np == 1 ? 0 : d, &c->bpad[d])) return PSH_ERR_CFG;
      if (c->bpad[d] < 0) {
        fprintf(stderr, "Error: `BOX_PAD' must be >= 0\n");
        return PSH_ERR_CFG;
      }
    }
  }
  long v;
  if ((rc = psh_int(cfg, "GRID_SIZE", 0, &v))) {
    if (rc == 1) fprintf(stderr, "Error: `GRID_SIZE' is not set\n");
    return PSH_ERR_CFG;
  }
  if (v <= 1 || v > 65536) {
    fprintf(stderr, "Error: `GRID_SIZE' must be > 1 and <= 65536\n");
    return PSH_ERR_CFG;
  }
  c->gsize = (int)v;
  c->assign = 2;  /* TSC */
  if ((rc = psh_int(cfg, "PARTICLE_ASSIGN", 0, &v)) < 0) return PSH_ERR_CFG;
  if (!rc) {
    if (v < 0 || v > 3) {
      fprintf(stderr, "Error: invalid `PARTICLE_ASSIGN': %ld\n", v);
      return PSH_ERR_CFG;
    }
    c->assign = (int)v;
  }
  c->intlace = false;
  if (psh_bool(cfg, "GRID_INTERLACE", 0, &c->intlace) < 0) return PSH_ERR_CFG;
  /* MULTIPOLE: sorted, duplicates removed, 0..6 */
  c->npole = psh_size(cfg, "MULTIPOLE");
  if (!c->npole) {
    fprintf(stderr, "Error: `MULTIPOLE' is not set\n");
    return PSH_ERR_CFG;
  }
  int pl[64];
  if (c->npole > 64) c->npole = 64;
  for (int i = 0; i < c->npole; i++) {
    if (psh_int(cfg, "MULTIPOLE", i, &v)) return PSH_ERR_CFG;
    pl[i] = (int)v;
  }
  for (int i = 1; i < c->npole; i++)
    for (int j = i; j > 0 && pl[j - 1] > pl[j]; j--) {
      const int t = pl[j];
      pl[j] = pl[j - 1];
      pl[j - 1] = t;
    }
  int m = 0;
  for (int i = 0; i < c->npole; i++)
    if (i == 0 || pl[i] != pl[m - 1]) pl[m++] = pl[i];
  c->npole = m;
  if (pl[0] < 0 || pl[m - 1] > 6) {
    fprintf(stderr, "Error: `MULTIPOLE' must be between 0 and 6\n");
    return PSH_ERR_CFG;
  }
  for (int i = 0; i < m; i++) c->poles[i] = pl[i];
  c->kmin = 0;
  if ((rc = psh_dbl(cfg, "KMIN", 0, &c->kmin)) < 0) return PSH_ERR_CFG;
  if (c->kmin < 0) {
    fprintf(stderr, "Error: `KMIN' must be >= 0\n");
    return PSH_ERR_CFG;
  }
  c->logscale = false;
  if (psh_bool(cfg, "LOG_SCALE", 0, &c->logscale) < 0) return PSH_ERR_CFG;
  if (c->logscale && c->kmin == 0) {
    fprintf(stderr, "Error: `KMIN' must be > 0 for log scale\n");
    return PSH_ERR_CFG;
  }
  if ((rc = psh_dbl(cfg, "BIN_SIZE", 0, &c->kbin))) {
    if (rc == 1) fprintf(stderr, "Error: `BIN_SIZE' is not set\n");
    return PSH_ERR_CFG;
  }
  if (c->kbin <= 0) {
    fprintf(stderr, "Error: `BIN_SIZE' must be > 0\n");
    return PSH_ERR_CFG;
  }
  c->kmax = -1;  /* unset */
  if ((rc = psh_dbl(cfg, "KMAX", 0, &c->kmax)) < 0) return PSH_ERR_CFG;
  if (!rc) {
    if (c->kmax <= 0) {
      fprintf(stderr, "Error: `KMAX' must be > 0\n");
      return PSH_ERR_CFG;
    }
    if (c->logscale ? (log10(c->kmax) < log10(c->kmin) + c->kbin) : (c->kmax < c->kmin + c->kbin)) {
      fprintf(stderr, "Error: `KMAX' must not be smaller than `KMIN' + `BIN_SIZE'%s\n",
              c->logscale ? " (in log10)" : "");
      return PSH_ERR_CFG;
    }
  }
  c->oheader = true;
  if (psh_bool(cfg, "OUTPUT_HEADER", 0, &c->oheader) < 0) return PSH_ERR_CFG;
  c->verbose = true;
  if (psh_bool(cfg, "VERBOSE", 0, &c->verbose) < 0) return PSH_ERR_CFG;
  /* after the checks, as the reference: log10 limits for log bins */
  if (c->logscale) {
    c->kmin = log10(c->kmin);
    if (c->kmax > 0) c->kmax = log10(c->kmax);
  }
  return 0;
}

static void header_common(FILE *fp, const Conf *c) {
  fprintf(fp, "# Box size: [%lg, %lg, %lg]\n# Box boundaries: [[%lg,%lg], [%lg,%lg], [%lg,%lg]]\n",
          c->bsize[0], c->bsize[1], c->bsize[2], c->bmin[0], c->bmin[0] + c->bsize[0], c->bmin[1],
          c->bmin[1] + c->bsize[1], c->bmin[2], c->bmin[2] + c->bsize[2]);
  fprintf(fp, "# Grid size: %d , assignment scheme: %s , grid interlacing: %s\n", c->gsize,
          kAssignNames[c->assign], c->intlace ? "enabled" : "disabled");
}

static int write_table(FILE *fp, const Conf *c, const ps_gpu_result *r, const double *pl) {
  fprintf(fp, "# kcen(1) kmin(2) kmax(3) kavg(4) nmod(5)");
  for (int l = 0; l < c->npole; l++) fprintf(fp, " P_%d(%d)", c->poles[l], l + 6);
  fprintf(fp, "\n");
  for (int i = 0; i < r->nbin; i++) {
    fprintf(fp, OFMT_DBL " " OFMT_DBL " " OFMT_DBL " " OFMT_DBL " %zu", r->k[i], r->kedge[i],
            r->kedge[i + 1], r->km[i], (size_t)r->cnt[i]);
    for (int l = 0; l < c->npole; l++) fprintf(fp, " " OFMT_DBL, pl[(size_t)l * r->nbin + i]);
    fprintf(fp, "\n");
  }
  return ferror(fp) ? PSH_ERR_FILE : 0;
}

static int save(const Conf *c, const size_t *ndata, const double *wdata, const size_t *nrand,
                const double *wrand, const ps_gpu_result *r) {
  printf("Saving outputs ...%s", c->verbose ? "\n" : "");
  fflush(stdout);
  for (int n = 0; n < c->ndata; n++) {
    if (!c->isauto[n]) continue;
    FILE *fp = fopen(c->oauto[n], "w");
    if (!fp) {
      fprintf(stderr, "Error: cannot write to file `%s'\n", c->oauto[n]);
      return PSH_ERR_FILE;
    }
    if (c->oheader) {
      fprintf(fp, "# Data catalog: %zu objects, total weight: " OFMT_DBL "\n", ndata[n], wdata[n]);
      if (!c->issim)
        fprintf(fp, "# Random catalog: %zu objects, total weight: " OFMT_DBL "\n", nrand[n], wrand[n]);
      header_common(fp, c);
      fprintf(fp, "# Shot noise: " OFMT_DBL " , normalisation: " OFMT_DBL " \n", r->shot[n], r->norm[n]);
    }
    const int rc = write_table(fp, c, r, r->pl + (size_t)n * c->npole * r->nbin);
    if (fclose(fp) || rc) return PSH_ERR_FILE;
    if (c->verbose) {
      if (c->ndata == 2)
        printf("  Auto power spectra for catalog %d saved to file: `%s'\n", n + 1, c->oauto[n]);
      else
        printf("  Auto power spectra saved to file: `%s'\n", c->oauto[n]);
    }
  }
  if (c->iscross) {
    FILE *fp = fopen(c->ocross, "w");
    if (!fp) {
      fprintf(stderr, "Error: cannot write to file `%s'\n", c->ocross);
      return PSH_ERR_FILE;
    }
    if (c->oheader) {
      fprintf(fp,
              "# Data catalog 1: %zu objects, total weight: " OFMT_DBL
              "\n# Data catalog 2: %zu objects, total weight: " OFMT_DBL "\n",
              ndata[0], wdata[0], ndata[1], wdata[1]);
      if (!c->issim)
        fprintf(fp,
                "# Random catalog 1: %zu objects, total weight: " OFMT_DBL
                "\n# Random catalog 2: %zu objects, total weight: " OFMT_DBL "\n",
                nrand[0], wrand[0], nrand[1], wrand[1]);
      header_common(fp, c);
      fprintf(fp, "# Normalisation factor 1: " OFMT_DBL " , Normalisation factor 2: " OFMT_DBL "\n",
              r->norm[0], r->norm[1]);
    }
    const int rc = write_table(fp, c, r, r->xpl);
    if (fclose(fp) || rc) return PSH_ERR_FILE;
    if (c->verbose) printf("  Cross power spectra saved to file: `%s'\n", c->ocross);
  }
  printf("\r\033[70C[\033[32;1mDONE\033[0m]\n");
  return 0;
}

/* Converts the catalogues flagged by DATA_CONVERT / RAND_CONVERT
 * (src/cnvt_coord.c:439-582): the quadrature order is chosen on the range of
 * all their redshifts. */
static int convert(Conf *c, double **data, const size_t *nd, double **rand, const size_t *nr) {
  printf("Converting coordinates ...\n");
  double zmin = DBL_MAX, zmax = -DBL_MAX;
  for (int i = 0; i < c->ndata; i++)
    for (int r = 0; r < 2; r++) {
      if (!(r ? c->rcnvt[i] : c->dcnvt[i])) continue;
      const double *p = r ? rand[i] : data[i];
      const size_t n = r ? nr[i] : nd[i];
      for (size_t k = 0; k < n; k++) {
        const double z = p[4 * k + 2];
        if (z < 0) {
          fprintf(stderr, "Error: invalid negative redshift in the %s catalog:\n(%g, %g, %g)\n",
                  r ? "random" : "data", p[4 * k], p[4 * k + 1], z);
          return PSH_ERR_CATA;
        }
        if (zmax < z) zmax = z;
        if (zmin > z) zmin = z;
      }
    }
  int rc = 0;
  if (zmin <= zmax || c->ztab) rc = psh_cosmo_init(&c->cosmo, c->ztab, zmin, zmax, c->verbose);
  for (int i = 0; i < c->ndata && !rc; i++) {
    if (c->dcnvt[i]) psh_cosmo_convert(&c->cosmo, data[i], nd[i], 0);
    if (c->rcnvt[i]) psh_cosmo_convert(&c->cosmo, rand[i], nr[i], 0);
  }
  psh_cosmo_free(&c->cosmo);
  return rc;
}

int main(int argc, char **argv) {
  psh_cfg cfg = {NULL, 0};
  int rc = psh_cfg_init(&cfg);
  if (rc) return rc;
  rc = psh_cfg_cmdline(&cfg, argc, argv);
  if (rc) {
    psh_cfg_free(&cfg);
    return rc == 1 ? 0 : rc;
  }
  printf("Loading configurations ...\n");
  const char *fconf = psh_str(&cfg, "CONFIG_FILE", 0);
  if (!fconf) fconf = "powspec.conf";
  if (access(fconf, R_OK)) {
    fprintf(stderr, "Warning: cannot access the configuration file: `%s'\n", fconf);
  } else if ((rc = psh_cfg_file(&cfg, fconf))) {
    fprintf(stderr, "Error: failed to read the configuration file `%s'\n", fconf);
    psh_cfg_free(&cfg);
    return rc;
  }
  Conf c;
  memset(&c, 0, sizeof c);
  if ((rc = verify(&cfg, &c))) {
    psh_cfg_free(&cfg);
    return PSH_ERR_CONF;
  }
  if (c.verbose) {
    printf("  Grid size: %d, assignment: %s, interlacing: %s", c.gsize, kAssignNames[c.assign],
           c.intlace ? "T" : "F");
    if (c.issim) printf(", box: [%lg, %lg, %lg]", c.bsize[0], c.bsize[1], c.bsize[2]);
    printf("\n");
  }

  /* catalogues */
  printf("Reading catalogues ...\n");
  double *xyzw[2] = {NULL, NULL}, *rxyzw[2] = {NULL, NULL};
  size_t ndata[2] = {0, 0}, nrand[2] = {0, 0};
  double wsum[2] = {0, 0}, wrand[2] = {0, 0}, shot[2] = {0, 0}, norm[2] = {0, 0};
  double s2[2][2] = {{0, 0}, {0, 0}}, s2n[2][2] = {{0, 0}, {0, 0}};
  for (int i = 0; i < c.ndata && !rc; i++) {
    rc = read_cat(&cfg, &c, "DATA", i, c.dfmt[i], &xyzw[i], &ndata[i], &wsum[i], &s2[i][0],
                  &s2n[i][0]);
    if (!rc && !c.issim)
      rc = read_cat(&cfg, &c, "RAND", i, c.rfmt[i], &rxyzw[i], &nrand[i], &wrand[i], &s2[i][1],
                    &s2n[i][1]);
  }
  if (!rc && c.cnvt) rc = convert(&c, xyzw, ndata, rxyzw, nrand);
  for (int i = 0; i < c.ndata && !rc && !c.issim; i++) {
    /* alpha, shot noise and normalisation (src/read_cata.c:165-183) */
    if (wsum[i] == 0 || s2[i][0] == 0) {
      fprintf(stderr, "Error: invalid completeness or FKP weights in the data catalog\n");
      rc = PSH_ERR_CATA;
    } else if (wrand[i] == 0 || s2[i][1] == 0) {
      fprintf(stderr, "Error: invalid completeness or FKP weights in the random catalog\n");
      rc = PSH_ERR_CATA;
    } else {
      const double alpha = wsum[i] / wrand[i];
      shot[i] = s2[i][0] + alpha * alpha * s2[i][1];
      norm[i] = (s2n[i][0] == 0 || s2n[i][1] != 0) ? alpha * s2n[i][1] : s2n[i][0];
      /* data minus alpha x randoms in one catalogue: weights -alpha w */
      double *all = realloc(xyzw[i], sizeof(double) * 4 * (ndata[i] + nrand[i]));
      if (!all) {
        rc = PSH_ERR_MEMORY;
        continue;
      }
      xyzw[i] = all;
      double *r = all + 4 * ndata[i];
      for (size_t k = 0; k < nrand[i]; k++) {
        r[4 * k] = rxyzw[i][4 * k];
        r[4 * k + 1] = rxyzw[i][4 * k + 1];
        r[4 * k + 2] = rxyzw[i][4 * k + 2];
        r[4 * k + 3] = -alpha * rxyzw[i][4 * k + 3];
      }
      free(rxyzw[i]);
      rxyzw[i] = NULL;
    }
  }
  if (!rc && !c.issim) {
    /* the box (src/genr_mesh.c:427-566): bounds of all data and randoms,
     * centred; BOX_SIZE, or the padded extent rounded up to 10 */
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int i = 0; i < c.ndata; i++)
      for (size_t k = 0; k < ndata[i] + nrand[i]; k++)
        for (int d = 0; d < 3; d++) {
          const double v = xyzw[i][4 * k + d];
          if (mn[d] > v) mn[d] = v;
          if (mx[d] < v) mx[d] = v;
        }
    for (int d = 0; d < 3 && !rc; d++) {
      if (c.bset) {
        if (mx[d] - mn[d] > c.bsize[d]) {
          fprintf(stderr, "Error: BOX_SIZE is too small for the %c coordinates, should be at least "
                          OFMT_DBL "\n", "xyz"[d], mx[d] - mn[d]);
          rc = PSH_ERR_CATA;
        }
      } else {
        c.bsize[d] = ceil((mx[d] - mn[d]) * (1 + c.bpad[d]) / 10) * 10;  /* POWSPEC_BOX_CEIL */
      }
      c.bmin[d] = (mx[d] + mn[d] - c.bsize[d]) * 0.5;
    }
    if (!rc && c.verbose)
      printf("  Box size: [%lg, %lg, %lg]\n  Box boundaries: [[%lg,%lg], [%lg,%lg], [%lg,%lg]]\n",
             c.bsize[0], c.bsize[1], c.bsize[2], c.bmin[0], c.bmin[0] + c.bsize[0], c.bmin[1],
             c.bmin[1] + c.bsize[1], c.bmin[2], c.bmin[2] + c.bsize[2]);
    /* positions relative to the box corner: (x - bmin) as the reference's
     * grid coordinate takes it (src/genr_mesh.c:57-62) */
    for (int i = 0; i < c.ndata && !rc; i++)
      for (size_t k = 0; k < ndata[i] + nrand[i]; k++)
        for (int d = 0; d < 3; d++) xyzw[i][4 * k + d] -= c.bmin[d];
  }

  /* estimator */
  ps_gpu_ctx *ctx = NULL;
  ps_gpu_result res;
  memset(&res, 0, sizeof res);
  double *pl = NULL, *xpl = NULL;
  if (!rc) {
    printf("Evaluating power spectra on the GPU ...\n");
    ps_gpu_params p;
    memset(&p, 0, sizeof p);
    p.ng = c.gsize;
    for (int d = 0; d < 3; d++) {
      p.box[d] = c.bsize[d];
      p.los[d] = c.los[d];
    }
    p.assign = c.assign;
    p.interlace = c.intlace;
    p.ncat = c.ndata;
    p.isauto[0] = c.isauto[0];
    p.isauto[1] = c.isauto[1];
    p.iscross = c.iscross;
    p.kmin = c.kmin;
    p.kmax = c.kmax;
    p.dk = c.kbin;
    p.logscale = c.logscale;
    p.npole = c.npole;
    for (int l = 0; l < c.npole; l++) p.poles[l] = c.poles[l];
    p.device = 0;
    if ((rc = ps_gpu_create(&p, &ctx))) {
      fprintf(stderr, "Error: %s\n", ps_gpu_last_error(ctx));
    } else {
      const int nb = ps_gpu_nbin(ctx);
      res.k = malloc(sizeof(double) * nb);
      res.kedge = malloc(sizeof(double) * (nb + 1));
      res.km = malloc(sizeof(double) * nb);
      res.cnt = malloc(sizeof(uint64_t) * nb);
      res.lcnt = malloc(sizeof(double) * nb * c.npole);
      pl = calloc((size_t)2 * c.npole * nb, sizeof(double));
      xpl = calloc((size_t)c.npole * nb, sizeof(double));
      res.pl = pl;
      res.xpl = xpl;
      if (!res.k || !res.kedge || !res.km || !res.cnt || !res.lcnt || !pl || !xpl) rc = PSH_ERR_MEMORY;
      for (int i = 0; i < c.ndata && !rc; i++) {
        if (!c.issim) rc = ps_gpu_set_survey(ctx, i, shot[i], norm[i], c.bmin);
        if (!rc) rc = ps_gpu_assign_aos(ctx, i, xyzw[i], ndata[i] + nrand[i], 0);
        if (rc) fprintf(stderr, "Error: %s\n", ps_gpu_last_error(ctx));
        free(xyzw[i]);  /* the reference frees the catalogue after assignment */
        xyzw[i] = NULL;
      }
      if (!rc && (rc = ps_gpu_execute(ctx, &res))) fprintf(stderr, "Error: %s\n", ps_gpu_last_error(ctx));
    }
  }
  if (!rc) rc = save(&c, ndata, wsum, nrand, wrand, &res);
  for (int i = 0; i < 2; i++) {
    free(xyzw[i]);
    free(rxyzw[i]);
  }
  free(res.k);
  free(res.kedge);
  free(res.km);
  free(res.cnt);
  free(res.lcnt);
  free(pl);
  free(xpl);
  if (ctx) ps_gpu_destroy(ctx);
  psh_cfg_free(&cfg);
  return rc;
}
