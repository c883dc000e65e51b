/*
 * ref_harness.c -- in-memory driver for the REFERENCE powspec objects.
 *
 * Test infrastructure for the oracle.  It is compiled only by
 * oracle/Makefile, together with the unmodified reference sources read from
 * their read-only location, into oracle/_ref/libpowspec_ref.so (git-ignored).
 * It fills the reference's own CONF and CATA structures (src/load_conf.h:40,
 * src/read_cata.h:48) the way load_conf/read_cata would for a periodic box,
 * then calls the reference entry points genr_mesh (src/genr_mesh.c:874) and
 * powspec (src/multipole.c:1179) and copies the PK/MESH fields that save_res
 * consumes (src/save_res.c:110-124) into caller-owned arrays.
 */
#include "define.h"
#include "load_conf.h"
#include "read_cata.h"
#include "genr_mesh.h"
#include "multipole.h"

#include <stdlib.h>
#include <string.h>
#include <omp.h>

static double now_s(void) { return omp_get_wtime(); }

typedef struct {
  CONF conf;
  CATA cat;
  double bsize[3], bpad[3], los[3];
  int poles[8];
  size_t ndata[2], nrand[2];
  double wdata[2], wrand[2], alpha[2], shot[2], norm[2];
  DATA *dptr[2], *rptr[2];
} ref_setup;

static int setup(ref_setup *s, int ncat, const double *const *data,
                 const size_t *ndata, int ng, const double box[3], int assign,
                 int intlace, const double los[3], const int *poles, int npole,
                 double kmin, double kmax, double dk, int logscale,
                 const int isauto[2], int iscross, int verbose) {
  memset(s, 0, sizeof *s);
  for (int i = 0; i < 3; i++) {
    s->bsize[i] = box[i];
    s->bpad[i] = 0.02;
    s->los[i] = los[i];
  }
  for (int i = 0; i < npole && i < 8; i++) s->poles[i] = poles[i];
  CONF *c = &s->conf;
  c->ndata = ncat;
  c->issim = true;
  c->los = s->los;
  c->bsize = s->bsize;
  c->bpad = s->bpad;
  c->gsize = ng;
  c->assign = assign;
  c->intlace = intlace != 0;
  c->poles = s->poles;
  c->npole = npole;
  c->kmin = kmin;
  c->kmax = kmax;
  c->logscale = logscale != 0;
  c->kbin = dk;
  c->isauto[0] = isauto[0] != 0;
  c->isauto[1] = (ncat > 1) && isauto[1] != 0;
  c->iscross = (ncat > 1) && iscross != 0;
  c->oheader = true;
  c->verbose = verbose != 0;

  CATA *t = &s->cat;
  t->num = ncat;
  t->data = malloc(sizeof(DATA *) * 2);
  t->rand = malloc(sizeof(DATA *) * 2);
  if (!t->data || !t->rand) return -1;
  t->ndata = s->ndata;
  t->nrand = s->nrand;
  t->wdata = s->wdata;
  t->wrand = s->wrand;
  t->alpha = s->alpha;
  t->shot = s->shot;
  t->norm = s->norm;
  for (int i = 0; i < ncat; i++) {
    /* genr_mesh frees the particle arrays (src/genr_mesh.c:917-922): give it
       a private copy. */
    t->data[i] = malloc(sizeof(DATA) * (ndata[i] ? ndata[i] : 1));
    t->rand[i] = NULL;
    if (!t->data[i]) return -1;
    memcpy(t->data[i], data[i], sizeof(DATA) * ndata[i]);
    s->ndata[i] = ndata[i];
    double w = 0;
    for (size_t n = 0; n < ndata[i]; n++) w += t->data[i][n].w;
    s->wdata[i] = w;
  }
  return 0;
}

/* Mesh only: the real-space density fields Fr (and Frl when interlaced) that
 * genr_mesh builds, row-major [ng][ng][ng]. */
int ref_mesh(const double *data, size_t ndata, int ng, const double box[3],
             int assign, int intlace, double *mesh0, double *mesh1) {
  ref_setup s;
  const double *d[1] = {data};
  const int poles[1] = {0};
  const double los[3] = {0, 0, 1};
  const int isauto[2] = {1, 0};
  if (setup(&s, 1, d, &ndata, ng, box, assign, intlace, los, poles, 1, 0,
            POWSPEC_KMAX_UNSET_VAL, 0.01, 0, isauto, 0, 0))
    return POWSPEC_ERR_MEMORY;
  MESH *mesh = genr_mesh(&s.conf, &s.cat);
  if (!mesh) return POWSPEC_ERR_MESH;
  memcpy(mesh0, mesh->Fr[0], sizeof(double) * mesh->Ntot);
  if (intlace && mesh1) memcpy(mesh1, mesh->Frl[0], sizeof(double) * mesh->Ntot);
  mesh_destroy(mesh);
  free(s.cat.data);
  free(s.cat.rand);
  return 0;
}

/* Full periodic-box run: genr_mesh + powspec.  Outputs are caller-owned:
 * k, km: [maxbin]; kedge: [maxbin+1]; cnt: [maxbin]; lcnt: [npole*maxbin];
 * pl: [2][npole][maxbin]; xpl: [npole][maxbin]; shot, norm: [2];
 * times: [2] wall seconds of genr_mesh and powspec. */
int ref_powspec(int ncat, const double *const *data, const size_t *ndata,
                int ng, const double box[3], int assign, int intlace,
                const double los[3], const int *poles, int npole, double kmin,
                double kmax, double dk, int logscale, const int isauto[2],
                int iscross, int maxbin, int *nbin, double *k, double *kedge,
                double *km, size_t *cnt, double *lcnt, double *pl, double *xpl,
                double *shot, double *norm, double *times, int verbose) {
  ref_setup s;
  if (setup(&s, ncat, data, ndata, ng, box, assign, intlace, los, poles, npole,
            kmin, kmax, dk, logscale, isauto, iscross, verbose))
    return POWSPEC_ERR_MEMORY;
  double t0 = now_s();
  MESH *mesh = genr_mesh(&s.conf, &s.cat);
  double t1 = now_s();
  if (!mesh) return POWSPEC_ERR_MESH;
  PK *pk = powspec(&s.conf, &s.cat, mesh);
  double t2 = now_s();
  if (times) { times[0] = t1 - t0; times[1] = t2 - t1; }
  if (!pk) { mesh_destroy(mesh); return POWSPEC_ERR_PK; }
  int rc = 0;
  *nbin = pk->nbin;
  if (pk->nbin > maxbin) {
    rc = POWSPEC_ERR_ARG;
  } else {
    for (int i = 0; i < pk->nbin; i++) {
      k[i] = pk->k[i];
      km[i] = pk->km[i];
      cnt[i] = pk->cnt[i];
      kedge[i] = pk->kedge[i];
      for (int l = 0; l < npole; l++) {
        lcnt[l * maxbin + i] = pk->lcnt[l * pk->nbin + i];
        for (int c = 0; c < 2; c++)
          if (pk->pl[c]) pl[((size_t)c * npole + l) * maxbin + i] = pk->pl[c][l][i];
        if (pk->xpl) xpl[(size_t)l * maxbin + i] = pk->xpl[l][i];
      }
    }
    kedge[pk->nbin] = pk->kedge[pk->nbin];
    for (int c = 0; c < ncat; c++) { shot[c] = s.shot[c]; norm[c] = s.norm[c]; }
  }
  powspec_destroy(pk);
  mesh_destroy(mesh);
  free(s.cat.data);
  free(s.cat.rand);
  return rc;
}
