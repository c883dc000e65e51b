/*
 * ps_read.c -- ASCII catalogues for the simulation-box path.
 *
 * Semantics of the reference's reader (io/read_ascii.c): the first `skip`
 * lines are dropped, lines whose first non-blank character is the comment
 * character are ignored (blank lines too), each line is parsed with the
 * scanf-style formatter, and the unsuppressed fields (%*... is skipped and
 * not counted) are the columns $1, $2, ... of the position, weight and
 * selection expressions.  Selected objects keep x, y, z and the completeness
 * weight; the total weight is their sum (io/read_ascii.c:903).
 */
#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ps_host.h"

enum { F_WS, F_LIT, F_NUM, F_STR, F_CHAR };

typedef struct {
  int kind;
  int skip;   /* suppressed with '*' */
  int width;  /* 0: none */
  char lit;
} Field;

/* Parses the formatter into fields; returns the count or < 0 on error. */
static int parse_fmt(const char *f, Field *out, int cap, int *ncol) {
  int n = 0;
  *ncol = 0;
  while (*f) {
    if (n == cap) return -1;
    Field fd = {F_LIT, 0, 0, 0};
    if (isspace((unsigned char)*f)) {
      while (isspace((unsigned char)*f)) f++;
      fd.kind = F_WS;
    } else if (*f != '%') {
      fd.lit = *f++;
    } else if (f[1] == '%') {
      fd.lit = '%';
      f += 2;
    } else {
      f++;
      if (*f == '*') {
        fd.skip = 1;
        f++;
      }
      while (isdigit((unsigned char)*f)) fd.width = fd.width * 10 + (*f++ - '0');
      while (*f == 'h' || *f == 'l' || *f == 'L' || *f == 'j' || *f == 'z' || *f == 't') f++;
      switch (*f) {
        case 'd': case 'i': case 'u': case 'o': case 'x': case 'X':
        case 'f': case 'F': case 'e': case 'E': case 'g': case 'G': case 'a': case 'A':
          fd.kind = F_NUM;
          break;
        case 's':
          fd.kind = F_STR;
          break;
        case 'c':
          fd.kind = F_CHAR;
          break;
        default:
          return -2;
      }
      f++;
      if (!fd.skip) (*ncol)++;
    }
    out[n++] = fd;
  }
  return n;
}

/* Parses one line; returns 0, or the 1-based index of the failing field. */
static int scan_line(const char *s, const Field *fd, int nf, double *col) {
  int c = 0;
  for (int k = 0; k < nf; k++) {
    const Field *f = &fd[k];
    if (f->kind == F_WS) {
      while (isspace((unsigned char)*s)) s++;
      continue;
    }
    if (f->kind == F_LIT) {
      if (*s != f->lit) return k + 1;
      s++;
      continue;
    }
    if (f->kind != F_CHAR)
      while (isspace((unsigned char)*s)) s++;
    if (!*s) return k + 1;
    char buf[128];
    const char *src = s;
    if (f->width) {  /* a field width limits the characters consumed */
      size_t w = (size_t)f->width < sizeof buf - 1 ? (size_t)f->width : sizeof buf - 1;
      size_t l = strlen(s);
      if (l < w) w = l;
      memcpy(buf, s, w);
      buf[w] = '\0';
      src = buf;
    }
    double v = 0;
    size_t used;
    if (f->kind == F_NUM) {
      char *e;
      errno = 0;
      v = strtod(src, &e);
      if (e == src) return k + 1;
      used = (size_t)(e - src);
    } else if (f->kind == F_STR) {
      used = 0;
      while (src[used] && !isspace((unsigned char)src[used])) used++;
    } else {
      used = f->width ? strlen(src) : 1;
    }
    s += used;
    if (!f->skip) col[c++] = v;
  }
  return 0;
}

int psh_read_ascii(const psh_ascii *in, double **xyzw, size_t *n, double *wsum, bool verbose) {
  Field fd[256];
  int ncol = 0;
  const int nf = parse_fmt(in->fmtr, fd, 256, &ncol);
  if (nf < 0) {
    fprintf(stderr, "Error: unsupported DATA_FORMATTER: `%s'\n", in->fmtr);
    return PSH_ERR_ASCII;
  }
  char err[256];
  psh_expr *ex[5] = {NULL, NULL, NULL, NULL, NULL};
  const char *src[5] = {in->pos[0], in->pos[1], in->pos[2], in->wcomp, in->sel};
  int rc = 0;
  for (int k = 0; k < 5 && !rc; k++) {
    if (!src[k]) continue;
    int maxcol = 0;
    ex[k] = psh_expr_compile(src[k], &maxcol, err, sizeof err);
    if (!ex[k]) {
      fprintf(stderr, "Error: invalid expression `%s': %s\n", src[k], err);
      rc = PSH_ERR_AST;
    } else if (maxcol > ncol) {
      fprintf(stderr, "Error: `%s' refers to column %d; the formatter has %d\n", src[k], maxcol, ncol);
      rc = PSH_ERR_AST;
    }
  }
  FILE *fp = rc ? NULL : fopen(in->fname, "r");
  if (!rc && !fp) {
    fprintf(stderr, "Error: cannot open catalogue `%s'\n", in->fname);
    rc = PSH_ERR_FILE;
  }
  size_t cap = 0, cnt = 0;
  double *buf = NULL, wtot = 0;
  double col[256];
  size_t lsize = 1 << 16;
  char *line = rc ? NULL : malloc(lsize);
  if (!rc && !line) rc = PSH_ERR_MEMORY;
  long lineno = 0;
  while (!rc) {
    /* one full line, however long */
    size_t len = 0;
    int got = 0;
    while (fgets(line + len, (int)(lsize - len), fp)) {
      got = 1;
      len += strlen(line + len);
      if (len && line[len - 1] == '\n') break;
      if (len + 1 < lsize) break;  /* last line without a newline */
      char *nl = realloc(line, lsize * 2);
      if (!nl) {
        rc = PSH_ERR_MEMORY;
        break;
      }
      line = nl;
      lsize *= 2;
    }
    if (!got || rc) break;
    lineno++;
    if (lineno <= in->skip) continue;
    const char *s = line;
    while (isspace((unsigned char)*s)) s++;
    if (!*s) continue;
    if (in->comment && *s == in->comment) continue;
    const int bad = scan_line(line, fd, nf, col);
    if (bad) {
      fprintf(stderr, "Error: failed to read line %ld of `%s' (field %d of the formatter)\n",
              lineno, in->fname, bad);
      rc = PSH_ERR_ASCII;
      break;
    }
    if (ex[4] && psh_expr_eval(ex[4], col) == 0) continue;
    if (cnt == cap) {
      cap = cap ? 2 * cap : 4096;
      double *nb = realloc(buf, sizeof(double) * 4 * cap);
      if (!nb) {
        rc = PSH_ERR_MEMORY;
        break;
      }
      buf = nb;
    }
    double *r = buf + 4 * cnt;
    for (int d = 0; d < 3; d++) r[d] = psh_expr_eval(ex[d], col);
    r[3] = ex[3] ? psh_expr_eval(ex[3], col) : 1.0;
    wtot += r[3];
    cnt++;
  }
  free(line);
  if (fp) fclose(fp);
  for (int k = 0; k < 5; k++) psh_expr_free(ex[k]);
  if (rc) {
    free(buf);
    return rc;
  }
  if (verbose) printf("  %zu objects read from `%s'\n", cnt, in->fname);
  *xyzw = buf;
  *n = cnt;
  *wsum = wtot;
  return 0;
}
