/*
 * SW2 case reader: m4 subset, expression evaluation and the tag sequence of
 * the reference's initialize() (init.c:48-237). See swcase.h.
 */
#include "swcase.h"

#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ buffers */
typedef struct {
  char *s;
  size_t n, cap;
} sbuf;

static int sb_put(sbuf *b, const char *p, size_t n) {
  if (b->n + n + 1 > b->cap) {
    size_t cap = b->cap ? b->cap : 256;
    while (cap < b->n + n + 1) cap *= 2;
    char *t = (char *)realloc(b->s, cap);
    if (!t) return -1;
    b->s = t;
    b->cap = cap;
  }
  memcpy(b->s + b->n, p, n);
  b->n += n;
  b->s[b->n] = '\0';
  return 0;
}

static void set_err(char *err, size_t errlen, const char *fmt, ...) {
  if (!err || !errlen) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, errlen, fmt, ap);
  va_end(ap);
}

static char *read_file(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  sbuf b = {0};
  char chunk[4096];
  size_t k;
  while ((k = fread(chunk, 1, sizeof chunk, f)) > 0)
    if (sb_put(&b, chunk, k)) {
      free(b.s);
      fclose(f);
      return NULL;
    }
  fclose(f);
  if (!b.s) {
    b.s = (char *)calloc(1, 1);
  }
  return b.s;
}

/* ------------------------------------------------------------ m4 subset */
typedef struct {
  char **name, **value;
  int n, cap;
} macros;

static const char *mac_get(const macros *m, const char *name, size_t len) {
  for (int k = m->n - 1; k >= 0; k--)
    if (strlen(m->name[k]) == len && !strncmp(m->name[k], name, len)) return m->value[k];
  return NULL;
}

static int mac_set(macros *m, const char *name, const char *value) {
  for (int k = 0; k < m->n; k++)
    if (!strcmp(m->name[k], name)) {
      char *v = strdup(value);
      if (!v) return -1;
      free(m->value[k]);
      m->value[k] = v;
      return 0;
    }
  if (m->n == m->cap) {
    int cap = m->cap ? 2 * m->cap : 16;
    char **a = (char **)realloc(m->name, cap * sizeof(char *));
    if (!a) return -1;
    m->name = a;
    a = (char **)realloc(m->value, cap * sizeof(char *));
    if (!a) return -1;
    m->value = a;
    m->cap = cap;
  }
  m->name[m->n] = strdup(name);
  m->value[m->n] = strdup(value);
  if (!m->name[m->n] || !m->value[m->n]) return -1;
  m->n++;
  return 0;
}

static void mac_free(macros *m) {
  for (int k = 0; k < m->n; k++) {
    free(m->name[k]);
    free(m->value[k]);
  }
  free(m->name);
  free(m->value);
}

static int is_word0(char c) { return isalpha((unsigned char)c) || c == '_'; }
static int is_word(char c) { return isalnum((unsigned char)c) || c == '_'; }

/* Arguments of a parenthesised list starting at text[*pos] == '(' (nested
 * parentheses kept, commas at depth 1 separate, leading blanks dropped). */
static int m4_args(const char *text, size_t *pos, char ***out, int *nout) {
  int depth = 0, cap = 4, n = 0;
  char **a = (char **)calloc(cap, sizeof(char *));
  sbuf cur = {0};
  size_t i = *pos;
  if (!a) return -1;
  for (; text[i]; i++) {
    const char c = text[i];
    if (c == '(') {
      depth++;
      if (depth > 1) sb_put(&cur, &c, 1);
    } else if (c == ')') {
      depth--;
      if (depth == 0) break;
      sb_put(&cur, &c, 1);
    } else if (c == ',' && depth == 1) {
      if (n + 1 >= cap) a = (char **)realloc(a, (cap *= 2) * sizeof(char *));
      a[n++] = cur.s ? cur.s : strdup("");
      cur = (sbuf){0};
    } else {
      sb_put(&cur, &c, 1);
    }
  }
  if (!text[i]) {
    free(cur.s);
    for (int k = 0; k < n; k++) free(a[k]);
    free(a);
    return -1;
  }
  if (n + 1 >= cap) a = (char **)realloc(a, (cap *= 2) * sizeof(char *));
  a[n++] = cur.s ? cur.s : strdup("");
  for (int k = 0; k < n; k++) {  /* drop leading blanks and newlines */
    char *p = a[k];
    while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++;
    memmove(a[k], p, strlen(p) + 1);
  }
  *pos = i + 1;
  *out = a;
  *nout = n;
  return 0;
}

static void trim(char *s) {
  char *p = s;
  while (*p == ' ' || *p == '\t' || *p == '\n') p++;
  memmove(s, p, strlen(p) + 1);
  size_t n = strlen(s);
  while (n && (s[n - 1] == ' ' || s[n - 1] == '\t' || s[n - 1] == '\n' || s[n - 1] == '\r')) s[--n] = '\0';
}

static int m4_expand(const char *text, macros *m, const char *dir, int depth, sbuf *out, char *err, size_t errlen) {
  if (depth > 50) {
    set_err(err, errlen, "m4: macro or include recursion too deep");
    return -1;
  }
  size_t i = 0;
  while (text[i]) {
    const char c = text[i];
    if (c == '#') {  /* comment: copied, not expanded */
      size_t j = i;
      while (text[j] && text[j] != '\n') j++;
      sb_put(out, text + i, j - i);
      i = j;
      continue;
    }
    if (is_word0(c) && (i == 0 || !is_word(text[i - 1]))) {
      size_t j = i;
      while (is_word(text[j])) j++;
      const size_t len = j - i;
      const int is_def = (len == 6 && !strncmp(text + i, "define", 6));
      const int is_inc = (len == 7 && !strncmp(text + i, "include", 7));
      if ((is_def || is_inc) && text[j] == '(') {
        char **a = NULL;
        int na = 0;
        if (m4_args(text, &j, &a, &na)) {
          set_err(err, errlen, "m4: unterminated argument list");
          return -1;
        }
        int rc = 0;
        if (is_def) {
          trim(a[0]);
          rc = mac_set(m, a[0], na > 1 ? a[1] : "");
        } else {
          trim(a[0]);
          char path[4096];
          if (a[0][0] == '/' || !dir || !dir[0]) snprintf(path, sizeof path, "%s", a[0]);
          else snprintf(path, sizeof path, "%s/%s", dir, a[0]);
          char *body = read_file(path);
          if (!body) {
            set_err(err, errlen, "m4: cannot include '%s'", path);
            rc = -1;
          } else {
            char sub[4096];
            snprintf(sub, sizeof sub, "%s", path);
            char *slash = strrchr(sub, '/');
            if (slash) *slash = '\0';
            else strcpy(sub, ".");
            rc = m4_expand(body, m, sub, depth + 1, out, err, errlen);
            free(body);
          }
        }
        for (int k = 0; k < na; k++) free(a[k]);
        free(a);
        if (rc) return -1;
        i = j;
        continue;
      }
      const char *v = mac_get(m, text + i, len);
      if (v) {
        char *copy = strdup(v);
        if (!copy) return -1;
        const int rc = m4_expand(copy, m, dir, depth + 1, out, err, errlen);
        free(copy);
        if (rc) return -1;
      } else {
        sb_put(out, text + i, len);
      }
      i = j;
      continue;
    }
    sb_put(out, &c, 1);
    i++;
  }
  return 0;
}

char *swcase_m4(const char *path, char *err, size_t errlen) {
  char *text = read_file(path);
  if (!text) {
    set_err(err, errlen, "cannot read '%s'", path);
    return NULL;
  }
  char dir[4096];
  snprintf(dir, sizeof dir, "%s", path);
  char *slash = strrchr(dir, '/');
  if (slash) *slash = '\0';
  else strcpy(dir, ".");
  macros m = {0};
  sbuf out = {0};
  const int rc = m4_expand(text, &m, dir, 0, &out, err, errlen);
  free(text);
  mac_free(&m);
  if (rc) {
    free(out.s);
    return NULL;
  }
  if (!out.s) out.s = (char *)calloc(1, 1);
  return out.s;
}

/* ------------------------------------------------------------ expressions */
typedef struct {
  const char *p;
  int err;
} ex;

static void ex_skip(ex *e) {
  while (*e->p == ' ' || *e->p == '\t' || *e->p == '\n' || *e->p == '\r') e->p++;
}

static double ex_list(ex *e);
static double ex_power(ex *e);

/* Integer part of a non-negative double not above 2^32-1, as a C cast to
 * unsigned int gives it; NaN gives 0 (what that cast yields on x86-64 and
 * aarch64 alike). */
static unsigned long long to_u32(double a) { return (a == a) ? (unsigned long long)(unsigned)a : 0ULL; }

/* fac and ncr give the values of the reference's expression library
 * (sppde/sppde_tinyexpr.c:122-149): exact products in 64-bit unsigned
 * integers, rounded to double once, and infinite as soon as a product leaves
 * 64 bits (fac(21) already does), not when a double would overflow. */
static double fac(double a) {
  if (a < 0.0) return NAN;
  if (a > 4294967295.0) return INFINITY;
  const unsigned long long n = to_u32(a);
  unsigned long long p = 1;
  for (unsigned long long k = 2; k <= n; k++)
    if (__builtin_mul_overflow(p, k, &p)) return INFINITY;
  return (double)p;
}
/* C(n, k) by the multiplicative formula over the shorter of k and n-k; after
 * step m the running value is C(n-k+m, m), an integer, so the division is exact. */
static double ncr(double n, double r) {
  if (n < 0.0 || r < 0.0 || n < r) return NAN;
  if (n > 4294967295.0 || r > 4294967295.0) return INFINITY;
  const unsigned long long top = to_u32(n);
  unsigned long long k = to_u32(r);
  if (k > top / 2) k = top - k;
  unsigned long long c = 1;
  for (unsigned long long m = 1; m <= k; m++) {
    if (__builtin_mul_overflow(c, top - k + m, &c)) return INFINITY;
    c /= m;
  }
  return (double)c;
}
static double npr(double n, double r) { return ncr(n, r) * fac(r); }

static int name_is(const char *s, size_t n, const char *w) { return strlen(w) == n && !strncmp(s, w, n); }

static double ex_base(ex *e) {
  ex_skip(e);
  const char c = *e->p;
  if (isdigit((unsigned char)c) || c == '.') {
    char *end;
    const double v = strtod(e->p, &end);
    if (end == e->p) {
      e->err = 1;
      return NAN;
    }
    e->p = end;
    return v;
  }
  if (c == '(') {
    e->p++;
    const double v = ex_list(e);
    ex_skip(e);
    if (*e->p != ')') {
      e->err = 1;
      return NAN;
    }
    e->p++;
    return v;
  }
  if (isalpha((unsigned char)c)) {
    const char *s = e->p;
    while (isalnum((unsigned char)*e->p) || *e->p == '_') e->p++;
    const size_t n = (size_t)(e->p - s);
    if (name_is(s, n, "pi") || name_is(s, n, "e")) {  /* constants; "()" optional */
      ex_skip(e);
      if (*e->p == '(') {
        e->p++;
        ex_skip(e);
        if (*e->p != ')') {
          e->err = 1;
          return NAN;
        }
        e->p++;
      }
      return name_is(s, n, "pi") ? 3.14159265358979323846 : 2.71828182845904523536;
    }
    double (*f1)(double) = NULL;
    if (name_is(s, n, "abs")) f1 = fabs;
    else if (name_is(s, n, "acos")) f1 = acos;
    else if (name_is(s, n, "asin")) f1 = asin;
    else if (name_is(s, n, "atan")) f1 = atan;
    else if (name_is(s, n, "ceil")) f1 = ceil;
    else if (name_is(s, n, "cos")) f1 = cos;
    else if (name_is(s, n, "cosh")) f1 = cosh;
    else if (name_is(s, n, "exp")) f1 = exp;
    else if (name_is(s, n, "fac")) f1 = fac;
    else if (name_is(s, n, "floor")) f1 = floor;
    else if (name_is(s, n, "ln")) f1 = log;
    else if (name_is(s, n, "log")) f1 = log10;
    else if (name_is(s, n, "log10")) f1 = log10;
    else if (name_is(s, n, "sin")) f1 = sin;
    else if (name_is(s, n, "sinh")) f1 = sinh;
    else if (name_is(s, n, "sqrt")) f1 = sqrt;
    else if (name_is(s, n, "tan")) f1 = tan;
    else if (name_is(s, n, "tanh")) f1 = tanh;
    if (f1) return f1(ex_power(e));
  }
  e->err = 1;
  return NAN;
}

static double ex_expr(ex *e);

/* a two-argument call body after '(' : expr ',' expr ')' */
static double ex_call2(ex *e, double (*f2)(double, double)) {
  const double a = ex_expr(e);
  ex_skip(e);
  if (*e->p != ',') {
    e->err = 1;
    return NAN;
  }
  e->p++;
  const double b = ex_expr(e);
  ex_skip(e);
  if (*e->p != ')') {
    e->err = 1;
    return NAN;
  }
  e->p++;
  return f2(a, b);
}

static double ex_primary(ex *e) {
  ex_skip(e);
  const char *s = e->p;
  if (isalpha((unsigned char)*s)) {
    const char *q = s;
    while (isalnum((unsigned char)*q) || *q == '_') q++;
    const size_t n = (size_t)(q - s);
    double (*f2)(double, double) = NULL;
    if (name_is(s, n, "atan2")) f2 = atan2;
    else if (name_is(s, n, "pow")) f2 = pow;
    else if (name_is(s, n, "ncr")) f2 = ncr;
    else if (name_is(s, n, "npr")) f2 = npr;
    if (f2) {
      e->p = q;
      ex_skip(e);
      if (*e->p != '(') {
        e->err = 1;
        return NAN;
      }
      e->p++;
      return ex_call2(e, f2);
    }
  }
  return ex_base(e);
}

/* <power> = {("-" | "+")} <base> */
static double ex_power(ex *e) {
  int sign = 1;
  ex_skip(e);
  while (*e->p == '-' || *e->p == '+') {
    if (*e->p == '-') sign = -sign;
    e->p++;
    ex_skip(e);
  }
  const double v = ex_primary(e);
  return sign < 0 ? -v : v;
}

/* <factor> = <power> {"^" <power>}  (left-associative) */
static double ex_factor(ex *e) {
  double v = ex_power(e);
  for (;;) {
    ex_skip(e);
    if (*e->p != '^') return v;
    e->p++;
    v = pow(v, ex_power(e));
  }
}

/* <term> = <factor> {("*" | "/" | "%") <factor>} */
static double ex_term(ex *e) {
  double v = ex_factor(e);
  for (;;) {
    ex_skip(e);
    const char c = *e->p;
    if (c != '*' && c != '/' && c != '%') return v;
    e->p++;
    const double w = ex_factor(e);
    v = (c == '*') ? v * w : (c == '/') ? v / w : fmod(v, w);
  }
}

/* <expr> = <term> {("+" | "-") <term>} */
static double ex_expr(ex *e) {
  double v = ex_term(e);
  for (;;) {
    ex_skip(e);
    const char c = *e->p;
    if (c != '+' && c != '-') return v;
    e->p++;
    const double w = ex_term(e);
    v = (c == '+') ? v + w : v - w;
  }
}

/* <list> = <expr> {"," <expr>}: the value of the last */
static double ex_list(ex *e) {
  double v = ex_expr(e);
  for (;;) {
    ex_skip(e);
    if (*e->p != ',') return v;
    e->p++;
    v = ex_expr(e);
  }
}

int swcase_eval(const char *expr, double *value) {
  ex e = {expr, 0};
  const double v = ex_list(&e);
  ex_skip(&e);
  if (e.err || *e.p != '\0') return -1;
  *value = v;
  return 0;
}

/* ------------------------------------------------------------ lines */
#define MAXL 1000  /* line buffer of the reference's reader */

typedef struct {
  char *text;   /* m4 output */
  size_t pos;
  char line[2 * MAXL + 64];
  char *err;
  size_t errlen;
  int failed;
} reader;

/* Cuts the line at '#' or newline; 1 if anything but blanks remains. */
static int clean_line(char *q) {
  int text = 0;
  for (; *q; q++) {
    if (*q == '\n' || *q == '#') {
      *q = '\0';
      break;
    }
    if (*q != ' ' && *q != '\t') text = 1;
  }
  return text;
}

/* Replaces each <expr> by its value printed with "%.15e"; "\<" and "\>"
 * stand for themselves (the backslash is dropped). */
static int eval_line(reader *r, char *input) {
  char result[2 * MAXL + 64], expr[MAXL + 1];
  size_t pr = 0, p = 0;
  int copy = 0, backs = 0, skip = 0;
  for (const char *q = input; *q; q++) {
    if (backs && (*q == '<' || *q == '>')) {
      skip = 1;
      backs = 0;
    }
    if (*q == '\\') {
      backs = 1;
      continue;
    }
    if (*q == '>' && !skip && copy) {
      copy = 0;
      expr[p] = '\0';
      double v;
      if (swcase_eval(expr, &v)) {
        set_err(r->err, r->errlen, "expression '%s' cannot be evaluated", expr);
        return -1;
      }
      char num[64];
      const int nch = snprintf(num, sizeof num, "%.15e", v);
      if (pr + nch >= sizeof result) return -1;
      memcpy(result + pr, num, nch);
      pr += nch;
      continue;
    }
    if (*q == '<' && !skip && !copy) {
      copy = 1;
      p = 0;
      continue;
    }
    if (copy) {
      if (p >= MAXL) return -1;
      expr[p++] = *q;
    } else {
      if (backs) {
        result[pr++] = '\\';
        backs = 0;
      }
      if (pr + 1 >= sizeof result) return -1;
      result[pr++] = *q;
    }
  }
  if (copy) {
    set_err(r->err, r->errlen, "missing '>' in '%s'", input);
    return -1;
  }
  result[pr] = '\0';
  strcpy(input, result);
  return 0;
}

static char *next_line(reader *r) {
  while (r->text[r->pos]) {
    size_t e = r->pos, n = 0;
    while (r->text[e] && r->text[e] != '\n' && n < MAXL - 2) {
      e++;
      n++;
    }
    memcpy(r->line, r->text + r->pos, n);
    r->line[n] = '\0';
    r->pos = (r->text[e] == '\n') ? e + 1 : e;
    if (clean_line(r->line)) {
      if (eval_line(r, r->line)) {
        r->failed = 1;
        return NULL;
      }
      return r->line;
    }
  }
  set_err(r->err, r->errlen, "unexpected end of file");
  r->failed = 1;
  return NULL;
}

/* Next line; with a tag, checks that its first token is the tag and returns the rest. */
static char *tagged(reader *r, const char *tag) {
  char *l = next_line(r);
  if (!l) return NULL;
  if (!tag[0]) return l;
  while (*l == ' ' || *l == '\t') l++;
  char *s = l;
  while (*l && *l != ' ' && *l != '\t') l++;
  const size_t n = (size_t)(l - s);
  if (n != strlen(tag) || strncmp(s, tag, n)) {
    set_err(r->err, r->errlen, "expecting '%s', found '%.*s'", tag, (int)n, s);
    r->failed = 1;
    return NULL;
  }
  while (*l == ' ' || *l == '\t') l++;
  return l;
}

static int get_int(reader *r, const char *tag, int *out) {
  char *l = tagged(r, tag);
  double aux, ip;
  if (!l) return -1;
  if (sscanf(l, "%le", &aux) != 1 || modf(aux, &ip) != 0) {
    set_err(r->err, r->errlen, "tag '%s': expecting an integer, found '%s'", tag, l);
    return -1;
  }
  *out = (int)aux;
  return 0;
}

static int get_double(reader *r, const char *tag, double *out) {
  char *l = tagged(r, tag);
  if (!l) return -1;
  if (sscanf(l, "%le", out) != 1) {
    set_err(r->err, r->errlen, "tag '%s': expecting a number, found '%s'", tag, l);
    return -1;
  }
  return 0;
}

static int get_doubles(reader *r, const char *tag, int nd, double *d) {
  char *l = tagged(r, tag);
  if (!l) return -1;
  char *save = NULL;
  for (int i = 0; i < nd; i++) {
    char *tok = strtok_r(i == 0 ? l : NULL, " \t", &save);
    if (!tok || sscanf(tok, "%lf", d + i) != 1) {
      set_err(r->err, r->errlen, "tag '%s': expecting %d numbers", tag, nd);
      return -1;
    }
  }
  return 0;
}

/* A table: rows, columns, then the rows (sppde_parser.c:290-318). */
static int get_table(reader *r, int transpose, int *nr, int *nc, double **out) {
  if (get_int(r, "", nr) || get_int(r, "", nc)) return -1;
  if (*nr < 0 || *nc < 1 || *nc > 100) {
    set_err(r->err, r->errlen, "table with %d rows and %d columns", *nr, *nc);
    return -1;
  }
  double *t = (double *)calloc((size_t)(*nr) * (*nc) + 1, sizeof(double));
  double row[100];
  if (!t) return -1;
  for (int i = 0; i < *nr; i++) {
    if (get_doubles(r, "", *nc, row)) {
      free(t);
      return -1;
    }
    for (int c = 0; c < *nc; c++) {
      if (!transpose) t[i * (*nc) + c] = row[c];
      else t[i + c * (*nr)] = row[c];
    }
  }
  *out = t;
  return 0;
}

static double deg2rad(double a) { return a * ((4.0 * atan(1.0)) / 180.0); }  /* sw.h:16, 108 */

#define RD(call)                 \
  do {                           \
    if (call) goto fail;         \
  } while (0)

int swcase_read(const char *path, swcase *c, char *err, size_t errlen) {
  memset(c, 0, sizeof *c);
  reader r = {0};
  r.err = err;
  r.errlen = errlen;
  r.text = swcase_m4(path, err, errlen);
  if (!r.text) return -1;
  double v, nu[3];
  RD(get_int(&r, "sch", &c->sch));
  RD(get_int(&r, "polar", &c->polar));
  if (c->polar == 0) {
    RD(get_double(&r, "lon0", &v)); c->lon0 = deg2rad(v);
    RD(get_double(&r, "lon1", &v)); c->lon1 = deg2rad(v);
    RD(get_double(&r, "lat0", &v)); c->lat0 = deg2rad(v);
    RD(get_double(&r, "lat1", &v)); c->lat1 = deg2rad(v);
    RD(get_int(&r, "nx", &c->nx));
    RD(get_int(&r, "ny", &c->ny));
  } else if (c->polar == 1 || c->polar == -1) {
    RD(get_double(&r, "angleSim", &v));
    c->lon0 = c->lat0 = -deg2rad(v);
    c->lon1 = c->lat1 = deg2rad(v);
    RD(get_int(&r, "n", &c->nx));
    c->ny = c->nx;
  } else {
    set_err(err, errlen, "polar=%d and should be 0, 1 or -1", c->polar);
    goto fail;
  }
  RD(get_double(&r, "t0", &c->t0));
  RD(get_double(&r, "t1", &c->t1));
  RD(get_double(&r, "Dt", &c->Dt));
  RD(get_double(&r, "CFL", &c->CFL));
  c->N = (int)((c->t1 - c->t0) / c->Dt);  /* init.c:107 */
  RD(get_double(&r, "Tau", &c->tau));
  c->sigma_dis = (c->tau > 1e10) ? 0 : 1.0 / c->tau;
  RD(get_doubles(&r, "Hypernu", 3, nu));
  c->nu2 = nu[0];
  c->nu4 = nu[1];
  c->nu6 = nu[2];
  if (c->nu2 < 0 || c->nu4 < 0 || c->nu6 < 0) {
    set_err(err, errlen, "hyperviscosity coefficients must be entered as >= 0");
    goto fail;
  }
  RD(get_int(&r, "IteInfo", &c->IteInfo));
  RD(get_int(&r, "SaveEvery", &c->saveEvery));
  RD(get_int(&r, "LoadFrom", &c->loadFrom));
  RD(get_int(&r, "reftype", &c->reftype));
  if (c->reftype == 1) {
    int nr, nc;
    double *t = NULL;
    RD(!tagged(&r, "refname"));
    RD(get_table(&r, 0, &nr, &nc, &t));
    free(t);
  } else if (c->reftype != 0) {
    set_err(err, errlen, "wrong reftype=%d", c->reftype);
    goto fail;
  }
  RD(get_double(&r, "Omega", &c->Omega));
  RD(get_double(&r, "rE", &c->rE));
  RD(get_double(&r, "rP", &c->rP));
  c->epsilon2 = (c->rE / c->rP) * (c->rE / c->rP);
  RD(get_double(&r, "gE", &c->gE));
  RD(get_double(&r, "depth", &c->depth));
  if (c->polar != 0) {
    RD(get_double(&r, "BetaSp", &c->beta_sponge));
    RD(get_double(&r, "SigSp", &c->sigma_sponge));
  }
  RD(get_int(&r, "geoeq", &c->geoeq));
  if (c->geoeq != 0 && c->geoeq != 1) {
    set_err(err, errlen, "geoeq=%d and should be 0 or 1", c->geoeq);
    goto fail;
  }
  {
    int nr, nc;
    RD(get_table(&r, 0, &nr, &nc, &c->vortices));
    if (nc != SWC_VORTEX_COLS) {
      set_err(err, errlen, "vortex table has %d columns, not %d", nc, SWC_VORTEX_COLS);
      goto fail;
    }
    c->num_vortices = nr;
    RD(get_table(&r, 0, &nr, &nc, &c->gaussians));
    if (nc != SWC_GAUSS_COLS) {
      set_err(err, errlen, "Gaussian table has %d columns, not %d", nc, SWC_GAUSS_COLS);
      goto fail;
    }
    c->num_gaussians = nr;
  }
  RD(get_double(&r, "TracerDis", &c->tracer_dis));
  {
    int nr, nc;
    RD(get_table(&r, 1, &nr, &nc, &c->wind));
    if (nc < 2) {
      set_err(err, errlen, "wind table needs 2 columns");
      goto fail;
    }
    c->wind_rows = nr;
  }
  free(r.text);
  return 0;
fail:
  if (err && errlen && !err[0]) set_err(err, errlen, "malformed case file");
  free(r.text);
  swcase_free(c);
  return -1;
}

void swcase_free(swcase *c) {
  free(c->vortices);
  free(c->gaussians);
  free(c->wind);
  c->vortices = c->gaussians = c->wind = NULL;
}
