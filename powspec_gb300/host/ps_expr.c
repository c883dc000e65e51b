/*
 * ps_expr.c -- expressions over catalogue columns, for DATA_POSITION,
 * DATA_WT_COMP and DATA_SELECTION (the reference evaluates these with its
 * expression library; the syntax kept here: numbers, $n and ${n} column
 * references (1-based, counting the unsuppressed formatter fields),
 * + - * / % ^ (or **), comparisons, && || !, parentheses, and the functions
 * sqrt exp log log10 sin cos tan asin acos atan abs fabs floor ceil pow).
 *
 * Compiled by recursive descent into a postfix program evaluated on a
 * small stack; logical values are 1 / 0.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ps_host.h"

enum {
  OP_NUM, OP_COL, OP_NEG, OP_NOT, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_POW,
  OP_LT, OP_LE, OP_GT, OP_GE, OP_EQ, OP_NE, OP_AND, OP_OR, OP_F1
};

typedef struct {
  int op;
  int col;
  double num;
  double (*f1)(double);
} Ins;

struct psh_expr {
  Ins *ins;
  int n, cap, depth;
};

typedef struct {
  const char *s;
  psh_expr *e;
  int maxcol;
  char *err;
  size_t errlen;
  int fail;
} Parser;

static void emit(Parser *p, Ins in) {
  if (p->fail) return;
  psh_expr *e = p->e;
  if (e->n == e->cap) {
    const int cap = e->cap ? 2 * e->cap : 32;
    Ins *ni = realloc(e->ins, sizeof(Ins) * (size_t)cap);
    if (!ni) {
      p->fail = 1;
      return;
    }
    e->ins = ni;
    e->cap = cap;
  }
  e->ins[e->n++] = in;
}

static void fail(Parser *p, const char *msg) {
  if (!p->fail) snprintf(p->err, p->errlen, "%s near `%s'", msg, p->s);
  p->fail = 1;
}

static void skip_ws(Parser *p) {
  while (isspace((unsigned char)*p->s)) p->s++;
}

static int accept(Parser *p, const char *tok) {
  skip_ws(p);
  const size_t l = strlen(tok);
  if (!strncmp(p->s, tok, l)) {
    p->s += l;
    return 1;
  }
  return 0;
}

static void parse_or(Parser *p);

static double f_abs(double x) { return fabs(x); }

static void parse_primary(Parser *p) {
  skip_ws(p);
  if (p->fail) return;
  const char *s = p->s;
  if (*s == '(') {
    p->s++;
    parse_or(p);
    if (!accept(p, ")")) fail(p, "missing `)'");
    return;
  }
  if (*s == '$') {
    p->s++;
    const int brace = (*p->s == '{');
    if (brace) p->s++;
    char *end;
    const long c = strtol(p->s, &end, 10);
    if (end == p->s || c < 1) {
      fail(p, "column numbers start at 1");
      return;
    }
    p->s = end;
    if (brace && !accept(p, "}")) {
      fail(p, "missing `}'");
      return;
    }
    Ins in = {OP_COL, (int)c - 1, 0, NULL};
    emit(p, in);
    if (c > p->maxcol) p->maxcol = (int)c;
    return;
  }
  if (isdigit((unsigned char)*s) || *s == '.') {
    char *end;
    const double v = strtod(s, &end);
    if (end == s) {
      fail(p, "bad number");
      return;
    }
    p->s = end;
    Ins in = {OP_NUM, 0, v, NULL};
    emit(p, in);
    return;
  }
  if (isalpha((unsigned char)*s)) {
    const char *t = s;
    while (isalnum((unsigned char)*t) || *t == '_') t++;
    const size_t l = (size_t)(t - s);
    static const struct {
      const char *name;
      double (*f)(double);
    } fn[] = {{"sqrt", sqrt},   {"exp", exp},   {"log", log},     {"log10", log10},
              {"sin", sin},     {"cos", cos},   {"tan", tan},     {"asin", asin},
              {"acos", acos},   {"atan", atan}, {"abs", f_abs},   {"fabs", f_abs},
              {"floor", floor}, {"ceil", ceil}};
    p->s = t;
    if (l == 3 && !strncmp(s, "pow", 3)) {
      if (!accept(p, "(")) { fail(p, "expected `('"); return; }
      parse_or(p);
      if (!accept(p, ",")) { fail(p, "pow needs two arguments"); return; }
      parse_or(p);
      if (!accept(p, ")")) { fail(p, "missing `)'"); return; }
      Ins in = {OP_POW, 0, 0, NULL};
      emit(p, in);
      return;
    }
    for (size_t k = 0; k < sizeof fn / sizeof fn[0]; k++)
      if (strlen(fn[k].name) == l && !strncmp(s, fn[k].name, l)) {
        if (!accept(p, "(")) { fail(p, "expected `('"); return; }
        parse_or(p);
        if (!accept(p, ")")) { fail(p, "missing `)'"); return; }
        Ins in = {OP_F1, 0, 0, fn[k].f};
        emit(p, in);
        return;
      }
    p->s = s;
    fail(p, "unknown function");
    return;
  }
  fail(p, "unexpected character");
}

static void parse_unary(Parser *p);

static void parse_power(Parser *p) {
  parse_primary(p);
  if (accept(p, "**") || accept(p, "^")) {
    parse_unary(p);  /* right associative */
    Ins in = {OP_POW, 0, 0, NULL};
    emit(p, in);
  }
}

static void parse_unary(Parser *p) {
  if (accept(p, "-")) {
    parse_unary(p);
    Ins in = {OP_NEG, 0, 0, NULL};
    emit(p, in);
  } else if (accept(p, "+")) {
    parse_unary(p);
  } else if (accept(p, "!")) {
    skip_ws(p);
    if (*p->s == '=') { fail(p, "unexpected `='"); return; }
    parse_unary(p);
    Ins in = {OP_NOT, 0, 0, NULL};
    emit(p, in);
  } else {
    parse_power(p);
  }
}

static void parse_mul(Parser *p) {
  parse_unary(p);
  for (;;) {
    int op;
    skip_ws(p);
    if (p->s[0] == '*' && p->s[1] != '*') op = OP_MUL;
    else if (*p->s == '/') op = OP_DIV;
    else if (*p->s == '%') op = OP_MOD;
    else break;
    p->s++;
    parse_unary(p);
    Ins in = {op, 0, 0, NULL};
    emit(p, in);
  }
}

static void parse_add(Parser *p) {
  parse_mul(p);
  for (;;) {
    int op;
    if (accept(p, "+")) op = OP_ADD;
    else if (accept(p, "-")) op = OP_SUB;
    else break;
    parse_mul(p);
    Ins in = {op, 0, 0, NULL};
    emit(p, in);
  }
}

static void parse_cmp(Parser *p) {
  parse_add(p);
  int op = -1;
  if (accept(p, "<=")) op = OP_LE;
  else if (accept(p, ">=")) op = OP_GE;
  else if (accept(p, "==")) op = OP_EQ;
  else if (accept(p, "!=")) op = OP_NE;
  else if (accept(p, "<")) op = OP_LT;
  else if (accept(p, ">")) op = OP_GT;
  if (op >= 0) {
    parse_add(p);
    Ins in = {op, 0, 0, NULL};
    emit(p, in);
  }
}

static void parse_and(Parser *p) {
  parse_cmp(p);
  while (accept(p, "&&")) {
    parse_cmp(p);
    Ins in = {OP_AND, 0, 0, NULL};
    emit(p, in);
  }
}

static void parse_or(Parser *p) {
  parse_and(p);
  while (accept(p, "||")) {
    parse_and(p);
    Ins in = {OP_OR, 0, 0, NULL};
    emit(p, in);
  }
}

psh_expr *psh_expr_compile(const char *src, int *maxcol, char *err, size_t errlen) {
  psh_expr *e = calloc(1, sizeof *e);
  if (!e) return NULL;
  Parser p = {src, e, 0, err, errlen, 0};
  parse_or(&p);
  skip_ws(&p);
  if (!p.fail && *p.s) fail(&p, "trailing characters");
  if (!p.fail && e->n == 0) fail(&p, "empty expression");
  if (p.fail) {
    psh_expr_free(e);
    return NULL;
  }
  /* stack depth */
  int d = 0, dmax = 0;
  for (int i = 0; i < e->n; i++) {
    const int op = e->ins[i].op;
    if (op == OP_NUM || op == OP_COL) d++;
    else if (op != OP_NEG && op != OP_NOT && op != OP_F1) d--;
    if (d > dmax) dmax = d;
  }
  e->depth = dmax;
  if (maxcol) *maxcol = p.maxcol;
  return e;
}

double psh_expr_eval(const psh_expr *e, const double *col) {
  double st[64];
  double *heap = NULL, *s = st;
  if (e->depth > 64) {
    heap = malloc(sizeof(double) * (size_t)e->depth);
    if (!heap) return NAN;
    s = heap;
  }
  int t = -1;
  for (int i = 0; i < e->n; i++) {
    const Ins *in = &e->ins[i];
    switch (in->op) {
      case OP_NUM: s[++t] = in->num; break;
      case OP_COL: s[++t] = col[in->col]; break;
      case OP_NEG: s[t] = -s[t]; break;
      case OP_NOT: s[t] = (s[t] == 0) ? 1 : 0; break;
      case OP_F1: s[t] = in->f1(s[t]); break;
      default: {
        const double b = s[t--], a = s[t];
        double r;
        switch (in->op) {
          case OP_ADD: r = a + b; break;
          case OP_SUB: r = a - b; break;
          case OP_MUL: r = a * b; break;
          case OP_DIV: r = a / b; break;
          case OP_MOD: r = fmod(a, b); break;
          case OP_POW: r = pow(a, b); break;
          case OP_LT: r = a < b; break;
          case OP_LE: r = a <= b; break;
          case OP_GT: r = a > b; break;
          case OP_GE: r = a >= b; break;
          case OP_EQ: r = a == b; break;
          case OP_NE: r = a != b; break;
          case OP_AND: r = (a != 0) && (b != 0); break;
          default: r = (a != 0) || (b != 0); break;
        }
        s[t] = r;
      }
    }
  }
  const double r = s[0];
  free(heap);
  return r;
}

int psh_expr_column(const psh_expr *e) {
  return (e && e->n == 1 && e->ins[0].op == OP_COL) ? e->ins[0].col : -1;
}

void psh_expr_free(psh_expr *e) {
  if (!e) return;
  free(e->ins);
  free(e);
}
