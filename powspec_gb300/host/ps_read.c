/*
 * ps_read.c -- catalogues for the simulation-box path: ASCII files
 * (DATA_FORMAT = 0) and NumPy .npy arrays (DATA_FORMAT = 2).
 *
 * ASCII semantics of the reference's reader (io/read_ascii.c:533-1142): the
 * first `skip` lines are dropped, lines whose first non-blank character is
 * the comment character are ignored (blank lines too), each line is parsed
 * with the scanf-style formatter after its leading blanks, and the
 * unsuppressed fields (%*... is skipped and not counted) are the columns
 * $1, $2, ... of the position, weight and selection expressions.  Selected
 * objects keep x, y, z and the completeness weight; the total weight is
 * their sum in file order (io/read_ascii.c:903).
 *
 * The file is mapped and cut at line boundaries (rows, for .npy) into one
 * range per host thread.  Each thread parses its range into its own
 * records; the records are then joined in file order, so the catalogue and
 * its total weight do not depend on the number of threads.  (The
 * reference's OpenMP build flushes per-thread pools in whatever order the
 * threads reach a critical section, io/read_ascii.c:1037-1058.)
 *
 * Numbers: a decimal string with at most 19 significant digits whose value
 * is m * 10^e with m <= 2^53 and |e| <= 22 is converted by one IEEE
 * multiply or divide of two exact doubles, which rounds correctly (Clinger's
 * fast path: W. D. Clinger, "How to read floating point numbers
 * accurately", PLDI 1990).  Every other string goes to strtod.  Both round
 * correctly, so the values are strtod's.
 */
#define _DEFAULT_SOURCE
#include <ctype.h>
#include <errno.h>
#include <fcntl.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "ps_host.h"

/* ---------------------------------------------------------------- numbers */

static const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,
                                  1e8,  1e9,  1e10, 1e11, 1e12, 1e13, 1e14, 1e15,
                                  1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

static int is_digit(char c) { return (unsigned)(c - '0') < 10u; }

double psh_strtod(const char *s, char **end) {
  const char *p = s;
  int neg = 0;
  if (*p == '+' || *p == '-') neg = (*p++ == '-');
  if (p[0] == '0' && (p[1] == 'x' || p[1] == 'X')) return strtod(s, end);
  uint64_t m = 0;
  int nd = 0, e10 = 0, any = 0, many = 0;
  for (; is_digit(*p); p++) {
    any = 1;
    if (m == 0 && *p == '0') continue;
    if (nd < 19) {
      m = m * 10 + (uint64_t)(*p - '0');
      nd++;
    } else {
      many = 1;
    }
  }
  if (*p == '.') {
    for (p++; is_digit(*p); p++) {
      any = 1;
      if (m == 0 && *p == '0') {
        e10--;
        continue;
      }
      if (nd < 19) {
        m = m * 10 + (uint64_t)(*p - '0');
        nd++;
        e10--;
      } else {
        many = 1;
      }
    }
  }
  if (!any) return strtod(s, end);  /* inf, nan, or not a number */
  if (*p == 'e' || *p == 'E') {
    const char *q = p + 1;
    int eneg = 0;
    if (*q == '+' || *q == '-') eneg = (*q++ == '-');
    if (is_digit(*q)) {  /* else the exponent is not part of the number */
      long ev = 0;
      for (; is_digit(*q); q++)
        if (ev < 100000) ev = ev * 10 + (*q - '0');
      e10 += (int)(eneg ? -ev : ev);
      p = q;
    }
  }
  if (many || m > ((uint64_t)1 << 53) || e10 < -22 || e10 > 22) return strtod(s, end);
  double v = (double)m;
  if (m) v = e10 >= 0 ? v * kPow10[e10] : v / kPow10[-e10];
  if (end) *end = (char *)p;
  return neg ? -v : v;
}

/* -------------------------------------------------------------- formatter */

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

/* Parses one NUL-terminated line; returns 0, or the 1-based index of the
 * failing field with *stop at the character where it failed. */
static int scan_line(const char *s, const Field *fd, int nf, double *col, const char **stop) {
  int c = 0;
  for (int k = 0; k < nf; k++) {
    const Field *f = &fd[k];
    *stop = s;
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
    *stop = s;
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
      v = psh_strtod(src, &e);
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

/* ------------------------------------------------------------ file access */

typedef struct {
  const char *p;
  size_t size;
  void *map;
  char *heap;
} Mapped;

static int map_file(const char *fname, Mapped *m) {
  memset(m, 0, sizeof *m);
  m->p = "";
  const int fd = open(fname, O_RDONLY);
  if (fd < 0) return PSH_ERR_FILE;
  struct stat st;
  if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode)) {
    m->size = (size_t)st.st_size;
    if (!m->size) {
      close(fd);
      return 0;
    }
    void *a = mmap(NULL, m->size, PROT_READ, MAP_PRIVATE, fd, 0);
    if (a != MAP_FAILED) {
      madvise(a, m->size, MADV_SEQUENTIAL);
      m->map = a;
      m->p = a;
      close(fd);
      return 0;
    }
  }
  /* not a mappable file (a pipe, say): read it whole */
  size_t cap = (size_t)1 << 20, len = 0;
  char *b = malloc(cap);
  int rc = b ? 0 : PSH_ERR_MEMORY;
  while (!rc) {
    if (len == cap) {
      char *nb = realloc(b, cap * 2);
      if (!nb) {
        rc = PSH_ERR_MEMORY;
        break;
      }
      b = nb;
      cap *= 2;
    }
    const ssize_t r = read(fd, b + len, cap - len);
    if (r < 0 && errno == EINTR) continue;
    if (r < 0) rc = PSH_ERR_FILE;
    if (r <= 0) break;
    len += (size_t)r;
  }
  close(fd);
  if (rc) {
    free(b);
    return rc;
  }
  m->heap = b;
  m->p = b;
  m->size = len;
  return 0;
}

static void unmap_file(Mapped *m) {
  if (m->map) munmap(m->map, m->size);
  free(m->heap);
}

/* Host threads: OMP_NUM_THREADS as the reference's OpenMP build reads it,
 * else the online cores; with at least `grain` units for each. */
static int host_threads(int want, size_t units, size_t grain) {
  long t = want;
  if (t <= 0) {
    const char *e = getenv("OMP_NUM_THREADS");
    if (e && *e) t = strtol(e, NULL, 10);
    if (t <= 0) t = sysconf(_SC_NPROCESSORS_ONLN);
    const size_t most = units / grain + 1;
    if (t > 0 && (size_t)t > most) t = (long)most;
  }
  if (t <= 0) t = 1;
  if (t > 256) t = 256;
  return (int)t;
}

/* ---------------------------------------------------- per-thread records */

typedef struct {
  Field fd[256];
  int nf, ncol;
  char comment;
  psh_expr *ex[7];  /* x, y, z, completeness weight, selection, FKP weight, n(z) */
  int colof[7];     /* an expression that is one column: its index, else -1 */
  int survey;
  const char *buf;  /* ASCII text, or .npy data */
  size_t size;
  /* .npy */
  size_t nrow;
  int ncolumn, esize, kind, swap, fortran, need;
} Reader;

typedef struct {
  const Reader *rd;
  size_t beg, end;  /* ASCII: byte range of whole lines; .npy: rows */
  double *rec;      /* {x, y, z, w} */
  double *ext;      /* surveys: {wc, wfkp, nz} per record */
  size_t cnt, cap;
  int err;
  size_t bad;       /* ASCII: offset of the line that failed; SIZE_MAX: none */
  size_t bad_stop;  /* and of the character where it failed */
  int bad_field;
  double *dst;      /* join: where this range's records go */
} Part;

static double value(const Reader *rd, int k, const double *col, double unset) {
  if (!rd->ex[k]) return unset;
  return rd->colof[k] >= 0 ? col[rd->colof[k]] : psh_expr_eval(rd->ex[k], col);
}

static int push(Part *pt, const double *col) {
  const Reader *rd = pt->rd;
  if (rd->ex[4] && psh_expr_eval(rd->ex[4], col) == 0) return 0;
  if (pt->cnt == pt->cap) {
    const size_t cap = pt->cap ? 2 * pt->cap : 4096;
    double *nb = realloc(pt->rec, sizeof(double) * 4 * cap);
    if (!nb) return PSH_ERR_MEMORY;
    pt->rec = nb;
    if (rd->survey) {
      double *ne = realloc(pt->ext, sizeof(double) * 3 * cap);
      if (!ne) return PSH_ERR_MEMORY;
      pt->ext = ne;
    }
    pt->cap = cap;
  }
  double *r = pt->rec + 4 * pt->cnt;
  for (int d = 0; d < 3; d++) r[d] = value(rd, d, col, 0.0);
  r[3] = value(rd, 3, col, 1.0);
  if (rd->survey) {  /* io/read_ascii.c:880-895 */
    double *x = pt->ext + 3 * pt->cnt;
    x[0] = r[3];
    x[1] = value(rd, 5, col, 1.0);
    x[2] = value(rd, 6, col, 0.0);
    r[3] = x[0] * x[1];
  }
  pt->cnt++;
  return 0;
}

static void *ascii_part(void *arg) {
  Part *pt = arg;
  const Reader *rd = pt->rd;
  size_t lcap = 512;
  char *line = malloc(lcap);
  double col[256];
  if (!line) {
    pt->err = PSH_ERR_MEMORY;
    return NULL;
  }
  const char *p = rd->buf + pt->beg, *const end = rd->buf + pt->end;
  while (p < end) {
    const char *nl = memchr(p, '\n', (size_t)(end - p));
    const char *le = nl ? nl : end, *next = nl ? nl + 1 : end;
    const char *s = p;
    while (s < le && isspace((unsigned char)*s)) s++;
    if (s == le || !*s || (rd->comment && *s == rd->comment)) {
      p = next;
      continue;
    }
    const size_t len = (size_t)(le - s);
    if (len + 1 > lcap) {
      while (len + 1 > lcap) lcap *= 2;
      char *nb = realloc(line, lcap);
      if (!nb) {
        pt->err = PSH_ERR_MEMORY;
        break;
      }
      line = nb;
    }
    memcpy(line, s, len);
    line[len] = '\0';
    const char *stop = line;
    const int bad = scan_line(line, rd->fd, rd->nf, col, &stop);
    if (bad) {
      pt->bad = (size_t)(p - rd->buf);
      pt->bad_stop = (size_t)(s - rd->buf) + (size_t)(stop - line);
      pt->bad_field = bad;
      break;
    }
    if ((pt->err = push(pt, col))) break;
    p = next;
  }
  free(line);
  return NULL;
}

enum { K_F4, K_F8, K_I4, K_I8 };

static double npy_value(const Reader *rd, size_t i, int j) {
  const size_t k = rd->fortran ? (size_t)j * rd->nrow + i : i * (size_t)rd->ncolumn + (size_t)j;
  unsigned char b[8];
  memcpy(b, rd->buf + k * (size_t)rd->esize, (size_t)rd->esize);
  if (rd->swap)
    for (int a = 0, z = rd->esize - 1; a < z; a++, z--) {
      const unsigned char t = b[a];
      b[a] = b[z];
      b[z] = t;
    }
  switch (rd->kind) {
    case K_F4: {
      float v;
      memcpy(&v, b, 4);
      return v;
    }
    case K_F8: {
      double v;
      memcpy(&v, b, 8);
      return v;
    }
    case K_I4: {
      int32_t v;
      memcpy(&v, b, 4);
      return (double)v;
    }
    default: {
      int64_t v;
      memcpy(&v, b, 8);
      return (double)v;
    }
  }
}

static void *npy_part(void *arg) {
  Part *pt = arg;
  const Reader *rd = pt->rd;
  double col[256];
  for (size_t i = pt->beg; i < pt->end; i++) {
    for (int j = 0; j < rd->need; j++) col[j] = npy_value(rd, i, j);
    if ((pt->err = push(pt, col))) break;
  }
  return NULL;
}

static void *copy_part(void *arg) {
  Part *pt = arg;
  if (pt->cnt) memcpy(pt->dst, pt->rec, sizeof(double) * 4 * pt->cnt);
  free(pt->rec);
  pt->rec = NULL;
  return NULL;
}

/* Survey sums in file order: completeness weights, (wc wfkp)^2, wc wfkp^2 nz. */
static void survey_sums(const Part *pt, int np, const psh_catalog *in, double *wsum) {
  double w = 0, w2 = 0, w2n = 0;
  for (int i = 0; i < np; i++)
    for (size_t k = 0; k < pt[i].cnt; k++) {
      const double *x = pt[i].ext + 3 * k;
      const double wt = x[0] * x[1];
      w += x[0];
      w2 += wt * wt;
      w2n += x[0] * x[1] * x[1] * x[2];
    }
  *wsum = w;
  if (in->sumw2) *in->sumw2 = w2;
  if (in->sumw2n) *in->sumw2n = w2n;
}

/* Runs fn on every part, part 0 on the calling thread. */
static void run_parts(Part *pt, int np, void *(*fn)(void *)) {
  pthread_t th[256];
  int up[256];
  for (int i = 1; i < np; i++) {
    up[i] = pthread_create(&th[i], NULL, fn, &pt[i]) == 0;
    if (!up[i]) fn(&pt[i]);
  }
  fn(&pt[0]);
  for (int i = 1; i < np; i++)
    if (up[i]) pthread_join(th[i], NULL);
}

/* Joins the parts' records in order and sums the weights in that order. */
static int join_parts(Part *pt, int np, double **xyzw, size_t *n, double *wsum) {
  size_t tot = 0;
  for (int i = 0; i < np; i++) tot += pt[i].cnt;
  double *out = NULL;
  if (tot && !(out = malloc(sizeof(double) * 4 * tot))) return PSH_ERR_MEMORY;
  size_t off = 0;
  for (int i = 0; i < np; i++) {
    pt[i].dst = out + 4 * off;
    off += pt[i].cnt;
  }
  const int survey = np > 0 && pt[0].rd->survey;
  run_parts(pt, np, copy_part);
  double w = 0;
  if (!survey)  /* surveys: the completeness weights (survey_sums) */
    for (size_t i = 0; i < tot; i++) w += out[4 * i + 3];
  *xyzw = out;
  *n = tot;
  if (!survey) *wsum = w;
  return 0;
}

static void free_parts(Part *pt, int np) {
  for (int i = 0; i < np; i++) {
    free(pt[i].rec);
    free(pt[i].ext);
  }
}

/* Compiles the expressions; maxcol: the columns there are. */
static int compile_exprs(const psh_catalog *in, Reader *rd, int ncol, const char *what) {
  const char *src[7] = {in->pos[0], in->pos[1], in->pos[2], in->wcomp, in->sel,
                        in->survey ? in->wfkp : NULL, in->survey ? in->nz : NULL};
  char err[256];
  rd->need = 0;
  rd->survey = in->survey;
  for (int k = 0; k < 7; k++) {
    rd->ex[k] = NULL;
    rd->colof[k] = -1;
    if (!src[k]) continue;
    int maxcol = 0;
    rd->ex[k] = psh_expr_compile(src[k], &maxcol, err, sizeof err);
    if (!rd->ex[k]) {
      fprintf(stderr, "Error: invalid expression `%s': %s\n", src[k], err);
      return PSH_ERR_AST;
    }
    if (maxcol > ncol) {
      fprintf(stderr, "Error: `%s' refers to column %d; the %s has %d\n", src[k], maxcol, what,
              ncol);
      return PSH_ERR_AST;
    }
    if (maxcol > rd->need) rd->need = maxcol;
    rd->colof[k] = psh_expr_column(rd->ex[k]);
  }
  return 0;
}

static void free_exprs(Reader *rd) {
  for (int k = 0; k < 7; k++) psh_expr_free(rd->ex[k]);
}

/* First line start at or after byte off. */
static size_t line_start(const char *b, size_t size, size_t off) {
  if (off == 0 || off >= size) return off >= size ? size : 0;
  if (b[off - 1] == '\n') return off;
  const char *nl = memchr(b + off, '\n', size - off);
  return nl ? (size_t)(nl - b) + 1 : size;
}

static size_t count_lines(const char *b, size_t len) {
  size_t c = 0;
  for (const char *p = b, *e = b + len; (p = memchr(p, '\n', (size_t)(e - p))); p++) c++;
  return c;
}

int psh_read_ascii(const psh_catalog *in, double **xyzw, size_t *n, double *wsum, bool verbose) {
  Reader *rd = calloc(1, sizeof *rd);
  if (!rd) return PSH_ERR_MEMORY;
  rd->nf = parse_fmt(in->fmtr, rd->fd, 256, &rd->ncol);
  int rc = 0;
  if (rd->nf < 0) {
    fprintf(stderr, "Error: unsupported DATA_FORMATTER: `%s'\n", in->fmtr);
    rc = PSH_ERR_ASCII;
  }
  if (!rc) rc = compile_exprs(in, rd, rd->ncol, "formatter");
  Mapped m;
  memset(&m, 0, sizeof m);
  if (!rc && (rc = map_file(in->fname, &m)))
    fprintf(stderr, "Error: cannot %s catalogue `%s'\n",
            rc == PSH_ERR_MEMORY ? "allocate memory for the" : "open", in->fname);
  Part pt[256];
  int np = 0;
  if (!rc) {
    rd->buf = m.p;
    rd->size = m.size;
    rd->comment = in->comment;
    size_t start = 0;
    for (long l = 0; l < in->skip && start < m.size; l++) {
      const char *nl = memchr(m.p + start, '\n', m.size - start);
      start = nl ? (size_t)(nl - m.p) + 1 : m.size;
    }
    np = host_threads(in->nthread, m.size - start, (size_t)1 << 20);
    memset(pt, 0, sizeof(Part) * (size_t)np);
    for (int i = 0; i < np; i++) {
      pt[i].rd = rd;
      pt[i].bad = SIZE_MAX;
      pt[i].beg = i ? line_start(m.p, m.size, start + (m.size - start) / (size_t)np * (size_t)i)
                    : start;
    }
    for (int i = 0; i < np; i++) {
      pt[i].end = i + 1 < np ? pt[i + 1].beg : m.size;
      if (pt[i].end < pt[i].beg) pt[i].end = pt[i].beg;
    }
    run_parts(pt, np, ascii_part);
    for (int i = 0; i < np && !rc; i++) {
      if (pt[i].err) {
        fprintf(stderr, "Error: failed to allocate memory for the catalogue `%s'\n", in->fname);
        rc = pt[i].err;
      } else if (pt[i].bad != SIZE_MAX) {
        const char *l = m.p + pt[i].bad;
        const char *nl = memchr(l, '\n', m.size - pt[i].bad);
        int len = (int)((nl ? (size_t)(nl - l) : m.size - pt[i].bad));
        fprintf(stderr, "Error: failed to read line %zu of `%s' with format `%s' (field %d):\n",
                count_lines(m.p, pt[i].bad) + 1, in->fname, in->fmtr, pt[i].bad_field);
        fprintf(stderr, "%.*s\n%*s^\n", len, l, (int)(pt[i].bad_stop - pt[i].bad), "");
        rc = PSH_ERR_ASCII;
      }
    }
  }
  if (!rc && in->survey) survey_sums(pt, np, in, wsum);
  if (!rc) rc = join_parts(pt, np, xyzw, n, wsum);
  free_parts(pt, np);
  unmap_file(&m);
  free_exprs(rd);
  free(rd);
  if (rc) return rc;
  if (verbose) printf("  %zu objects read from `%s'\n", *n, in->fname);
  return 0;
}

/* ------------------------------------------------------------------ .npy */

/* The value text of key in the header dict, or NULL. */
static const char *npy_key(const char *h, const char *key) {
  const char *k = strstr(h, key);
  if (!k) return NULL;
  k += strlen(key);
  while (*k == ' ' || *k == '\'' || *k == '"') k++;
  if (*k != ':') return NULL;
  for (k++; *k == ' '; k++) {}
  return k;
}

static int npy_header(const Mapped *m, Reader *rd, char *err, size_t errlen) {
  const unsigned char *u = (const unsigned char *)m->p;
  if (m->size < 10 || memcmp(u, "\x93NUMPY", 6)) {
    snprintf(err, errlen, "not a .npy file");
    return PSH_ERR_FILE;
  }
  size_t hl, off;
  if (u[6] == 1) {
    hl = (size_t)u[8] | (size_t)u[9] << 8;
    off = 10;
  } else if ((u[6] == 2 || u[6] == 3) && m->size >= 12) {
    hl = (size_t)u[8] | (size_t)u[9] << 8 | (size_t)u[10] << 16 | (size_t)u[11] << 24;
    off = 12;
  } else {
    snprintf(err, errlen, "unsupported .npy version %d", u[6]);
    return PSH_ERR_FILE;
  }
  if (off + hl > m->size || hl > 65536) {
    snprintf(err, errlen, "truncated .npy header");
    return PSH_ERR_FILE;
  }
  char h[65537];
  memcpy(h, m->p + off, hl);
  h[hl] = '\0';
  const char *d = npy_key(h, "'descr'"), *f = npy_key(h, "'fortran_order'");
  const char *s = npy_key(h, "'shape'");
  if (!d || !f || !s || (*d != '\'' && *d != '"') || *s != '(') {
    snprintf(err, errlen, "unrecognised .npy header `%.200s'", h);
    return PSH_ERR_FILE;
  }
  /* descr: byte order [<>|=], kind [fi], size */
  const char order = d[1], kind = d[2];
  const int size = atoi(d + 3);
  const uint16_t one = 1;
  const int little = *(const unsigned char *)&one == 1;
  if (kind == 'f' && size == 4) rd->kind = K_F4;
  else if (kind == 'f' && size == 8) rd->kind = K_F8;
  else if (kind == 'i' && size == 4) rd->kind = K_I4;
  else if (kind == 'i' && size == 8) rd->kind = K_I8;
  else {
    snprintf(err, errlen, "unsupported .npy dtype (f4, f8, i4 or i8 only)");
    return PSH_ERR_FILE;
  }
  rd->esize = size;
  rd->swap = (order == '>' && little) || (order == '<' && !little);
  rd->fortran = !strncmp(f, "True", 4);
  /* shape: (n,) or (n, k) */
  size_t dim[3];
  int nd = 0;
  for (const char *p = s + 1; *p && *p != ')';) {
    while (*p == ' ' || *p == ',') p++;
    if (*p == ')') break;
    if (!is_digit(*p) || nd == 3) {
      snprintf(err, errlen, "bad .npy shape");
      return PSH_ERR_FILE;
    }
    char *e;
    dim[nd++] = (size_t)strtoull(p, &e, 10);
    p = e;
  }
  if (nd < 1 || nd > 2 || (nd == 2 && (dim[1] < 1 || dim[1] > 256))) {
    snprintf(err, errlen, "a .npy catalogue is a 1-D array or a 2-D array of 1 to 256 columns");
    return PSH_ERR_FILE;
  }
  rd->nrow = dim[0];
  rd->ncolumn = nd == 2 ? (int)dim[1] : 1;
  const size_t data = off + hl;
  if (rd->nrow > (m->size - data) / (size_t)rd->ncolumn / (size_t)size) {
    snprintf(err, errlen, "the file is shorter than its %zu x %d array", rd->nrow, rd->ncolumn);
    return PSH_ERR_FILE;
  }
  rd->buf = m->p + data;
  rd->size = m->size - data;
  return 0;
}

int psh_read_npy(const psh_catalog *in, double **xyzw, size_t *n, double *wsum, bool verbose) {
  Reader *rd = calloc(1, sizeof *rd);
  if (!rd) return PSH_ERR_MEMORY;
  Mapped m;
  int rc = map_file(in->fname, &m);
  if (rc) fprintf(stderr, "Error: cannot open catalogue `%s'\n", in->fname);
  char err[256];
  if (!rc && (rc = npy_header(&m, rd, err, sizeof err)))
    fprintf(stderr, "Error: `%s': %s\n", in->fname, err);
  if (!rc) rc = compile_exprs(in, rd, rd->ncolumn, "array");
  Part pt[256];
  int np = 0;
  if (!rc) {
    np = host_threads(in->nthread, rd->nrow, (size_t)1 << 16);
    memset(pt, 0, sizeof(Part) * (size_t)np);
    for (int i = 0; i < np; i++) {
      pt[i].rd = rd;
      pt[i].beg = rd->nrow / (size_t)np * (size_t)i;
      pt[i].end = i + 1 < np ? rd->nrow / (size_t)np * (size_t)(i + 1) : rd->nrow;
    }
    run_parts(pt, np, npy_part);
    for (int i = 0; i < np && !rc; i++)
      if (pt[i].err) {
        fprintf(stderr, "Error: failed to allocate memory for the catalogue `%s'\n", in->fname);
        rc = pt[i].err;
      }
  }
  if (!rc && in->survey) survey_sums(pt, np, in, wsum);
  if (!rc) rc = join_parts(pt, np, xyzw, n, wsum);
  free_parts(pt, np);
  unmap_file(&m);
  free_exprs(rd);
  free(rd);
  if (rc) return rc;
  if (verbose) printf("  %zu objects read from `%s'\n", *n, in->fname);
  return 0;
}
