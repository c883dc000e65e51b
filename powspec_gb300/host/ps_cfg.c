/*
 * ps_cfg.c -- configuration file and command-line options.
 *
 * Keywords, short and long option names are powspec's
 * (src/load_conf.c:366-417); command-line values take priority over the
 * file (POWSPEC_PRIOR_CMD > POWSPEC_PRIOR_FILE, src/define.h:71-72).
 * File syntax: `KEYWORD = value  # comment`, arrays as `[a, b, c]` (may
 * span lines), strings optionally quoted with "" or ''.
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ps_host.h"

static const psh_opt kOpts[] = {
    {'c', "conf", "CONFIG_FILE", 0},         {'d', "data", "DATA_CATALOG", 1},
    {'r', "rand", "RAND_CATALOG", 1},        {'f', "data-format", "DATA_FORMAT", 1},
    {'F', "rand-format", "RAND_FORMAT", 1},  {0, "data-skip", "DATA_SKIP", 1},
    {0, "rand-skip", "RAND_SKIP", 1},        {0, "data-comment", "DATA_COMMENT", 1},
    {0, "rand-comment", "RAND_COMMENT", 1},  {0, "data-formatter", "DATA_FORMATTER", 1},
    {0, "rand-formatter", "RAND_FORMATTER", 1}, {'p', "data-pos", "DATA_POSITION", 1},
    {'P', "rand-pos", "RAND_POSITION", 1},   {0, "data-wt-comp", "DATA_WT_COMP", 1},
    {0, "rand-wt-comp", "RAND_WT_COMP", 1},  {0, "data-wt-fkp", "DATA_WT_FKP", 1},
    {0, "rand-wt-fkp", "RAND_WT_FKP", 1},    {0, "data-nz", "DATA_NZ", 1},
    {0, "rand-nz", "RAND_NZ", 1},            {0, "data-select", "DATA_SELECTION", 1},
    {0, "rand-select", "RAND_SELECTION", 1}, {0, "data-convert", "DATA_CONVERT", 1},
    {0, "rand-convert", "RAND_CONVERT", 1},  {'m', "omega-m", "OMEGA_M", 0},
    {0, "omega-l", "OMEGA_LAMBDA", 0},       {0, "eos-w", "DE_EOS_W", 0},
    {0, "cmvdst-err", "CMVDST_ERR", 0},      {0, "cmvdst-file", "Z_CMVDST_CNVT", 0},
    {'s', "sim", "CUBIC_SIM", 0},            {0, "line-of-sight", "LINE_OF_SIGHT", 1},
    {'B', "box-size", "BOX_SIZE", 1},        {0, "box-pad", "BOX_PAD", 1},
    {'G', "grid-size", "GRID_SIZE", 0},      {'n', "part-assign", "PARTICLE_ASSIGN", 0},
    {'i', "interlace", "GRID_INTERLACE", 0}, {'l', "pole", "MULTIPOLE", 1},
    {0, "log-scale", "LOG_SCALE", 0},        {'k', "kmin", "KMIN", 0},
    {'K', "kmax", "KMAX", 0},                {'b', "bin-size", "BIN_SIZE", 0},
    {'a', "auto", "OUTPUT_AUTO", 1},         {'x', "cross", "OUTPUT_CROSS", 0},
    {0, "output-header", "OUTPUT_HEADER", 0}, {'w', "overwrite", "OVERWRITE", 0},
    {'v', "verbose", "VERBOSE", 0},
};

int psh_cfg_init(psh_cfg *c) {
  c->nopt = (int)(sizeof kOpts / sizeof kOpts[0]);
  c->opt = calloc((size_t)c->nopt, sizeof(psh_opt));
  if (!c->opt) return PSH_ERR_MEMORY;
  memcpy(c->opt, kOpts, sizeof kOpts);
  return 0;
}

static void clear_val(psh_opt *o) {
  for (int i = 0; i < o->n; i++) free(o->val[i]);
  free(o->val);
  o->val = NULL;
  o->n = 0;
}

void psh_cfg_free(psh_cfg *c) {
  if (!c->opt) return;
  for (int i = 0; i < c->nopt; i++) clear_val(&c->opt[i]);
  free(c->opt);
  c->opt = NULL;
}

psh_opt *psh_cfg_get(psh_cfg *c, const char *key) {
  for (int i = 0; i < c->nopt; i++)
    if (!strcmp(c->opt[i].key, key)) return &c->opt[i];
  return NULL;
}

static char *dup_range(const char *s, const char *e) {
  while (s < e && isspace((unsigned char)*s)) s++;
  while (e > s && isspace((unsigned char)e[-1])) e--;
  if (e - s >= 2 && (*s == '"' || *s == '\'') && e[-1] == *s) {
    s++;
    e--;
  }
  char *r = malloc((size_t)(e - s) + 1);
  if (!r) return NULL;
  memcpy(r, s, (size_t)(e - s));
  r[e - s] = '\0';
  return r;
}

/* Splits a value into elements: "[a, b]" (commas outside quotes) or a scalar;
 * on the command line a bare "a,b" is an array too. */
static int set_value(psh_opt *o, const char *v, int src, int cmd) {
  if (o->src > src) return 0;  /* a higher-priority source already set it */
  clear_val(o);
  while (isspace((unsigned char)*v)) v++;
  size_t len = strlen(v);
  while (len && isspace((unsigned char)v[len - 1])) len--;
  if (!len) {
    o->src = src;
    return 0;  /* empty: unset */
  }
  const char *s = v, *e = v + len;
  int bracket = (*s == '[');
  if (bracket) {
    if (e[-1] != ']') {
      fprintf(stderr, "Error: unclosed array for `%s'\n", o->key);
      return PSH_ERR_CFG;
    }
    s++;
    e--;
  }
  const int split = bracket || (cmd && o->array);
  const char *p = s;
  char q = 0;
  for (const char *t = s;; t++) {
    const int end = (t == e);
    if (!end && q) {
      if (*t == q) q = 0;
      continue;
    }
    if (!end && (*t == '"' || *t == '\'')) {
      q = *t;
      continue;
    }
    if (end || (split && *t == ',')) {
      char *el = dup_range(p, t);
      if (!el) return PSH_ERR_MEMORY;
      char **nv = realloc(o->val, sizeof(char *) * (size_t)(o->n + 1));
      if (!nv) {
        free(el);
        return PSH_ERR_MEMORY;
      }
      o->val = nv;
      o->val[o->n++] = el;
      p = t + 1;
      if (end) break;
    }
  }
  if (!o->array && o->n > 1) {
    fprintf(stderr, "Error: `%s' takes a single value\n", o->key);
    return PSH_ERR_CFG;
  }
  o->src = src;
  return 0;
}

int psh_cfg_file(psh_cfg *c, const char *fname) {
  FILE *fp = fopen(fname, "r");
  if (!fp) return PSH_ERR_FILE;
  char line[65536];
  char *acc = NULL;  /* an array continued over several lines */
  size_t acclen = 0;
  int rc = 0;
  while (fgets(line, sizeof line, fp)) {
    /* strip the comment (outside quotes) */
    char q = 0;
    for (char *t = line; *t; t++) {
      if (q) {
        if (*t == q) q = 0;
      } else if (*t == '"' || *t == '\'') {
        q = *t;
      } else if (*t == '#') {
        *t = '\0';
        break;
      }
    }
    const size_t l = strlen(line);
    char *nacc = realloc(acc, acclen + l + 2);
    if (!nacc) {
      rc = PSH_ERR_MEMORY;
      break;
    }
    acc = nacc;
    memcpy(acc + acclen, line, l + 1);
    acclen += l;
    /* an opened '[' without ']' continues on the next line */
    char *eq = strchr(acc, '=');
    if (eq) {
      const char *v = eq + 1;
      while (isspace((unsigned char)*v)) v++;
      if (*v == '[' && !strchr(v, ']')) continue;
    }
    char *s = acc;
    while (isspace((unsigned char)*s)) s++;
    if (*s) {
      if (!eq) {
        fprintf(stderr, "Warning: ignoring line without `=' in `%s': %s\n", fname, s);
      } else {
        char *k = s, *ke = eq;
        while (ke > k && isspace((unsigned char)ke[-1])) ke--;
        *ke = '\0';
        psh_opt *o = psh_cfg_get(c, k);
        if (!o || !strcmp(k, "CONFIG_FILE")) {
          fprintf(stderr, "Warning: unknown keyword `%s' in `%s'\n", k, fname);
        } else {
          /* flatten the newlines of a multi-line array */
          for (char *t = eq + 1; *t; t++)
            if (*t == '\n' || *t == '\r') *t = ' ';
          if ((rc = set_value(o, eq + 1, PSH_SRC_FILE, 0))) break;
        }
      }
    }
    acclen = 0;
    acc[0] = '\0';
  }
  free(acc);
  fclose(fp);
  return rc;
}

static void usage(const char *prog) {
  printf("Usage: %s [OPTION]\n"
         "Power spectrum multipoles of periodic simulation boxes on the GPU.\n"
         "  -h, --help          print this message and exit\n"
         "  -t, --template      print a template configuration file and exit\n",
         prog);
  for (size_t i = 0; i < sizeof kOpts / sizeof kOpts[0]; i++) {
    if (kOpts[i].sopt)
      printf("  -%c, --%-16s %s\n", kOpts[i].sopt, kOpts[i].lopt, kOpts[i].key);
    else
      printf("      --%-16s %s\n", kOpts[i].lopt, kOpts[i].key);
  }
  printf("Keywords take the same values in the configuration file "
         "(default: powspec.conf);\ncommand-line values have priority.\n");
}

static void template_conf(void) {
  printf("# Configuration file for the GPU periodic-box estimator.\n"
         "# Format: KEYWORD = value # comment, arrays as [a, b].\n\n");
  for (size_t i = 0; i < sizeof kOpts / sizeof kOpts[0]; i++)
    if (strcmp(kOpts[i].key, "CONFIG_FILE")) printf("%-16s=\n", kOpts[i].key);
}

int psh_cfg_cmdline(psh_cfg *c, int argc, char **argv) {
  for (int i = 1; i < argc; i++) {
    const char *a = argv[i];
    psh_opt *o = NULL;
    const char *val = NULL;
    if (a[0] == '-' && a[1] == '-') {
      const char *name = a + 2;
      const char *eq = strchr(name, '=');
      const size_t nl = eq ? (size_t)(eq - name) : strlen(name);
      if ((nl == 4 && !strncmp(name, "help", 4))) {
        usage(argv[0]);
        return 1;
      }
      if (nl == 8 && !strncmp(name, "template", 8)) {
        template_conf();
        return 1;
      }
      for (int k = 0; k < c->nopt; k++)
        if (strlen(c->opt[k].lopt) == nl && !strncmp(c->opt[k].lopt, name, nl)) o = &c->opt[k];
      if (!o) {
        fprintf(stderr, "Error: unrecognised option `%s'\n", a);
        return PSH_ERR_ARG;
      }
      if (eq) val = eq + 1;
    } else if (a[0] == '-' && a[1]) {
      if (a[1] == 'h') {
        usage(argv[0]);
        return 1;
      }
      if (a[1] == 't') {
        template_conf();
        return 1;
      }
      for (int k = 0; k < c->nopt; k++)
        if (c->opt[k].sopt == a[1]) o = &c->opt[k];
      if (!o) {
        fprintf(stderr, "Error: unrecognised option `%s'\n", a);
        return PSH_ERR_ARG;
      }
      if (a[2]) val = a + 2;
    } else {
      fprintf(stderr, "Error: unrecognised argument `%s'\n", a);
      return PSH_ERR_ARG;
    }
    if (!val) {
      if (i + 1 >= argc) {
        fprintf(stderr, "Error: option `%s' needs a value\n", a);
        return PSH_ERR_ARG;
      }
      val = argv[++i];
    }
    const int rc = set_value(o, val, PSH_SRC_CMD, 1);
    if (rc) return rc;
  }
  return 0;
}

int psh_size(psh_cfg *c, const char *key) {
  psh_opt *o = psh_cfg_get(c, key);
  return o ? o->n : 0;
}

const char *psh_str(psh_cfg *c, const char *key, int i) {
  psh_opt *o = psh_cfg_get(c, key);
  return (o && i < o->n) ? o->val[i] : NULL;
}

int psh_int(psh_cfg *c, const char *key, int i, long *out) {
  const char *s = psh_str(c, key, i);
  if (!s) return 1;
  char *e;
  const long v = strtol(s, &e, 10);
  while (isspace((unsigned char)*e)) e++;
  if (e == s || *e) {
    fprintf(stderr, "Error: `%s' is not an integer: %s\n", key, s);
    return PSH_ERR_CFG;
  }
  *out = v;
  return 0;
}

int psh_dbl(psh_cfg *c, const char *key, int i, double *out) {
  const char *s = psh_str(c, key, i);
  if (!s) return 1;
  char *e;
  const double v = strtod(s, &e);
  while (isspace((unsigned char)*e)) e++;
  if (e == s || *e) {
    fprintf(stderr, "Error: `%s' is not a number: %s\n", key, s);
    return PSH_ERR_CFG;
  }
  *out = v;
  return 0;
}

int psh_bool(psh_cfg *c, const char *key, int i, bool *out) {
  const char *s = psh_str(c, key, i);
  if (!s) return 1;
  char b[16];
  size_t k = 0;
  for (; s[k] && k < sizeof b - 1; k++) b[k] = (char)toupper((unsigned char)s[k]);
  b[k] = '\0';
  if (!strcmp(b, "T") || !strcmp(b, "TRUE") || !strcmp(b, ".TRUE.") || !strcmp(b, "1")) {
    *out = true;
    return 0;
  }
  if (!strcmp(b, "F") || !strcmp(b, "FALSE") || !strcmp(b, ".FALSE.") || !strcmp(b, "0")) {
    *out = false;
    return 0;
  }
  fprintf(stderr, "Error: `%s' is not a boolean: %s\n", key, s);
  return PSH_ERR_CFG;
}
