/*
 * gpu_path.c -- the reference's periodic-box path on the GB300 C ABI.
 *
 * The file a powspec maintainer adds to the reference's own sources in
 * place of src/genr_mesh.c and src/multipole.c.  It keeps their two entry
 * points and destructors with the reference's signatures:
 *
 *   MESH *genr_mesh(const CONF *conf, CATA *cat);   src/genr_mesh.h:86
 *   void  mesh_destroy(MESH *mesh);                 src/genr_mesh.h:95
 *   PK   *powspec(const CONF *conf, const CATA *cat, MESH *mesh);
 *                                                   src/multipole.h:78
 *   void  powspec_destroy(PK *pk);                  src/multipole.h:87
 *
 * and the one global the other reference files read from them,
 * powspec_assign_names (src/genr_mesh.h:45).  main (src/powspec.c),
 * load_conf, read_cata, cnvt_coord and save_res are the reference's,
 * unchanged, and call these as they call the CPU versions
 * (src/powspec.c:47,55).  Only simulation boxes (CUBIC_SIM = T) take this
 * path; a survey configuration is refused with the reference's error code.
 *
 * Ownership is the reference's: genr_mesh frees the particle arrays after
 * assignment and keeps the catalogue metadata (src/genr_mesh.c:917-922);
 * powspec returns a caller-owned PK; the MESH keeps only the metadata
 * save_res reads (bsize, min, Ng, assign, intlace, num).  The GPU context
 * lives between the two calls, one per process (main calls them once).
 *
 * Built with the reference's headers by `make -C oracle binding` (the
 * reference's other objects and this file, linked against
 * libpowspec_gpu.so).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "define.h"
#include "genr_mesh.h"
#include "load_conf.h"
#include "multipole.h"
#include "read_cata.h"

#include "powspec_gpu.h"

const char *powspec_assign_names[] = {"NGP", "CIC", "TSC", "PCS"};

static ps_gpu_ctx *g_ctx;

static void report(const char *what) {
  P_ERR("%s: %s\n", what, g_ctx ? ps_gpu_last_error(g_ctx) : "no GPU context");
}

MESH *genr_mesh(const CONF *conf, CATA *cat) {
  printf("Generating meshes for FFT (GB300) ...");
  fflush(stdout);
  if (!conf) {
    P_ERR("configuration parameters not loaded\n");
    return NULL;
  }
  if (!cat) {
    P_ERR("catalogs not read\n");
    return NULL;
  }
  if (!conf->issim) {
    P_ERR("the GB300 path takes simulation boxes (CUBIC_SIM = T)\n");
    return NULL;
  }
  ps_gpu_params p;
  memset(&p, 0, sizeof p);
  p.ng = conf->gsize;
  p.assign = conf->assign;
  p.interlace = conf->intlace;
  p.ncat = conf->ndata;
  for (int i = 0; i < conf->ndata && i < 2; i++) p.isauto[i] = conf->isauto[i];
  p.iscross = conf->iscross;
  for (int d = 0; d < 3; d++) {
    p.box[d] = conf->bsize[d];
    p.los[d] = conf->los[d];
  }
  p.kmin = conf->kmin;
  p.kmax = conf->kmax;
  p.dk = conf->kbin;
  p.logscale = conf->logscale;
  p.npole = conf->npole;
  for (int l = 0; l < conf->npole && l < 7; l++) p.poles[l] = conf->poles[l];
  p.device = 0;
  if (ps_gpu_create(&p, &g_ctx)) {
    report("GPU context");
    ps_gpu_destroy(g_ctx);
    g_ctx = NULL;
    return NULL;
  }
  MESH *mesh = calloc(1, sizeof(MESH));
  if (!mesh) {
    P_ERR("failed to allocate memory for the mesh metadata\n");
    return NULL;
  }
  mesh->num = cat->num;
  mesh->Ng = conf->gsize;
  mesh->Ngk = conf->gsize / 2 + 1;
  mesh->Ntot = (size_t)mesh->Ng * mesh->Ng * mesh->Ng;
  mesh->Ncmplx = (size_t)mesh->Ng * mesh->Ng * mesh->Ngk;
  mesh->issim = true;
  mesh->intlace = conf->intlace;
  mesh->assign = (powspec_assign_t)conf->assign;
  for (int d = 0; d < 3; d++) {
    /* a simulation box starts at 0 (src/genr_mesh.c:509-540) */
    mesh->bsize[d] = conf->bsize[d];
    mesh->min[d] = 0;
    mesh->max[d] = conf->bsize[d];
    mesh->smin[d] = -0.5 * conf->bsize[d] / conf->gsize;
  }
  for (int i = 0; i < cat->num; i++) {
    /* DATA is {double x[3], w}: the AoS layout of ps_gpu_assign_aos */
    if (ps_gpu_assign_aos(g_ctx, i, (const double *)cat->data[i], cat->ndata[i], 0)) {
      report("particle assignment");
      mesh_destroy(mesh);
      return NULL;
    }
  }
  /* shot noise and normalisation of simulation boxes from the reader's
     total weight (src/genr_mesh.c:904-910) */
  const double vol = mesh->bsize[0] * mesh->bsize[1] * mesh->bsize[2];
  for (int i = 0; i < cat->num; i++) {
    cat->shot[i] = vol / cat->wdata[i];
    cat->norm[i] = cat->wdata[i] * cat->wdata[i] / vol;
  }
  for (int i = 0; i < 3; i++) mesh->smin[i] = mesh->min[i] * mesh->Ng / mesh->bsize[i];
  /* the catalogues are no longer needed (src/genr_mesh.c:917-922) */
  for (int i = 0; i < cat->num; i++) {
    if (cat->data && cat->data[i]) free(cat->data[i]);
    if (cat->rand && cat->rand[i]) free(cat->rand[i]);
  }
  free(cat->data);
  cat->data = NULL;
  free(cat->rand);
  cat->rand = NULL;
  printf(FMT_DONE);
  return mesh;
}

void mesh_destroy(MESH *mesh) {
  if (!mesh) return;
  free(mesh);
  if (g_ctx) {
    ps_gpu_destroy(g_ctx);
    g_ctx = NULL;
  }
}

/* Row pointers [nrow][nbin] over one contiguous block. */
static double **rows(double *block, int nrow, int nbin) {
  double **r = calloc(nrow, sizeof(double *));
  if (!r) return NULL;
  for (int j = 0; j < nrow; j++) {
    r[j] = malloc(sizeof(double) * nbin);
    if (!r[j]) return r; /* partial: freed by powspec_destroy */
    memcpy(r[j], block + (size_t)j * nbin, sizeof(double) * nbin);
  }
  return r;
}

PK *powspec(const CONF *conf, const CATA *cat, MESH *mesh) {
  printf("Evaluating power spectra (GB300) ...");
  fflush(stdout);
  if (!conf || !cat || !mesh || !g_ctx) {
    P_ERR("meshes not generated\n");
    return NULL;
  }
  const int nb = ps_gpu_nbin(g_ctx), nl = conf->npole;
  if (nb <= 0) {
    report("k bins");
    return NULL;
  }
  PK *pk = calloc(1, sizeof(PK));
  if (!pk) return NULL;
  pk->issim = true;
  pk->log = conf->logscale;
  pk->isauto[0] = conf->isauto[0];
  pk->isauto[1] = conf->ndata > 1 ? conf->isauto[1] : false;
  pk->iscross = conf->iscross;
  pk->nl = nl;
  pk->nbin = nb;
  pk->dk = conf->kbin;
  for (int d = 0; d < 3; d++) pk->los[d] = conf->los[d];
  pk->poles = malloc(sizeof(int) * nl);
  pk->kedge = malloc(sizeof(double) * (nb + 1));
  pk->k = malloc(sizeof(double) * nb);
  pk->km = malloc(sizeof(double) * nb);
  pk->cnt = malloc(sizeof(size_t) * nb);
  pk->lcnt = malloc(sizeof(double) * nl * nb);
  uint64_t *cnt = malloc(sizeof(uint64_t) * nb);
  double *pl = calloc((size_t)2 * nl * nb, sizeof(double));
  double *xpl = calloc((size_t)nl * nb, sizeof(double));
  if (!pk->poles || !pk->kedge || !pk->k || !pk->km || !pk->cnt || !pk->lcnt || !cnt || !pl ||
      !xpl) {
    P_ERR("failed to allocate memory for the power spectra\n");
    free(cnt); free(pl); free(xpl);
    powspec_destroy(pk);
    return NULL;
  }
  memcpy(pk->poles, conf->poles, sizeof(int) * nl);
  ps_gpu_result r;
  memset(&r, 0, sizeof r);
  r.k = pk->k;
  r.kedge = pk->kedge;
  r.km = pk->km;
  r.cnt = cnt;
  r.lcnt = pk->lcnt;
  r.pl = pl;
  r.xpl = xpl;
  int rc = ps_gpu_execute(g_ctx, &r);
  if (rc) {
    report("power spectra");
    free(cnt); free(pl); free(xpl);
    powspec_destroy(pk);
    return NULL;
  }
  for (int b = 0; b < nb; b++) pk->cnt[b] = (size_t)cnt[b];
  /* pl[c][l][b] and xpl[l][b] as the reference's row arrays */
  for (int c = 0; c < 2; c++)
    if (pk->isauto[c] && !(pk->pl[c] = rows(pl + (size_t)c * nl * nb, nl, nb))) rc = 1;
  if (pk->iscross && !(pk->xpl = rows(xpl, nl, nb))) rc = 1;
  free(cnt); free(pl); free(xpl);
  if (rc) {
    P_ERR("failed to allocate memory for the power spectra\n");
    powspec_destroy(pk);
    return NULL;
  }
  printf(FMT_DONE);
  return pk;
}

void powspec_destroy(PK *pk) {
  if (!pk) return;
  free(pk->poles);
  free(pk->kedge);
  free(pk->k);
  free(pk->km);
  free(pk->cnt);
  free(pk->lcnt);
  for (int c = 0; c < 2; c++) {
    if (!pk->pl[c]) continue;
    for (int j = 0; j < pk->nl; j++) free(pk->pl[c][j]);
    free(pk->pl[c]);
  }
  if (pk->xpl) {
    for (int j = 0; j < pk->nl; j++) free(pk->xpl[j]);
    free(pk->xpl);
  }
  free(pk);
}
