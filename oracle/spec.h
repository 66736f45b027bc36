/*
 * TEST INFRASTRUCTURE (oracle).  Not part of the product; only the tests,
 * the smoke check and the benchmark's CPU-baseline leg use it.
 *
 * Parser for the decomposition spec strings that tests use to describe one
 * Decomp to several independent builders (the oracle restatement, the
 * reference driver, the product's Python mirror).
 *
 *   decomp   := "packed:" dim ("|" dim)*
 *             | "axes:" dim "@" stride "," rank_stride ("|" dim "@" stride "," rank_stride)*
 *   dim      := "block(" len "," procs ")"
 *             | "blockf(" len "," factor "," procs ")"
 *             | "local(" len ")"
 *             | "single(" len "," rank "," procs ")"
 *             | "rotate(" r "," dim ")"
 *             | "interleave(" dim "," B ")"
 *             | "frev(" A "," B "," dim ")"
 *
 * Header-only; every function is static.
 */
#ifndef ORACLE_SPEC_H
#define ORACLE_SPEC_H
#include <ctype.h>
#include <stdlib.h>
#include <string.h>

enum spec_kind { SK_BLOCK = 1, SK_BLOCKF, SK_LOCAL, SK_SINGLE, SK_ROTATE, SK_INTERLEAVE, SK_FREV };

typedef struct spec_dim {
  int kind;
  int v[3];
  struct spec_dim *nested;
} spec_dim;

#define SPEC_MAXD 8
typedef struct {
  int packed;
  int ndim;
  spec_dim *dims[SPEC_MAXD];
  int stride[SPEC_MAXD];
  int rank_stride[SPEC_MAXD];
} spec_decomp;

static const char *spec_ws(const char *s) {
  while (*s && isspace((unsigned char)*s)) ++s;
  return s;
}
static const char *spec_int(const char *s, int *out, int *ok) {
  s = spec_ws(s);
  char *e;
  long v = strtol(s, &e, 10);
  if (e == s) *ok = 0;
  *out = (int)v;
  return spec_ws(e);
}
static const char *spec_lit(const char *s, const char *lit, int *ok) {
  s = spec_ws(s);
  size_t n = strlen(lit);
  if (strncmp(s, lit, n) != 0) {
    *ok = 0;
    return s;
  }
  return spec_ws(s + n);
}
static void spec_free_dim(spec_dim *d) {
  if (!d) return;
  spec_free_dim(d->nested);
  free(d);
}
static const char *spec_parse_dim(const char *s, spec_dim **out, int *ok) {
  spec_dim *d = (spec_dim *)calloc(1, sizeof(spec_dim));
  *out = d;
  s = spec_ws(s);
  if (!strncmp(s, "blockf(", 7)) {
    d->kind = SK_BLOCKF;
    s = spec_int(s + 7, &d->v[0], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[1], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[2], ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "block(", 6)) {
    d->kind = SK_BLOCK;
    s = spec_int(s + 6, &d->v[0], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[1], ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "local(", 6)) {
    d->kind = SK_LOCAL;
    s = spec_int(s + 6, &d->v[0], ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "single(", 7)) {
    d->kind = SK_SINGLE;
    s = spec_int(s + 7, &d->v[0], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[1], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[2], ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "rotate(", 7)) {
    d->kind = SK_ROTATE;
    s = spec_int(s + 7, &d->v[0], ok);
    s = spec_lit(s, ",", ok);
    s = spec_parse_dim(s, &d->nested, ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "interleave(", 11)) {
    d->kind = SK_INTERLEAVE;
    s = spec_parse_dim(s + 11, &d->nested, ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[0], ok);
    s = spec_lit(s, ")", ok);
  } else if (!strncmp(s, "frev(", 5)) {
    d->kind = SK_FREV;
    s = spec_int(s + 5, &d->v[0], ok);
    s = spec_lit(s, ",", ok);
    s = spec_int(s, &d->v[1], ok);
    s = spec_lit(s, ",", ok);
    s = spec_parse_dim(s, &d->nested, ok);
    s = spec_lit(s, ")", ok);
  } else {
    *ok = 0;
  }
  return s;
}
/* Returns 0 on success. */
static int spec_parse(const char *s, spec_decomp *out) {
  memset(out, 0, sizeof(*out));
  int ok = 1;
  s = spec_ws(s);
  if (!strncmp(s, "packed:", 7)) {
    out->packed = 1;
    s += 7;
  } else if (!strncmp(s, "axes:", 5)) {
    out->packed = 0;
    s += 5;
  } else {
    return -1;
  }
  for (;;) {
    if (out->ndim >= SPEC_MAXD) return -1;
    int i = out->ndim++;
    s = spec_parse_dim(s, &out->dims[i], &ok);
    if (!out->packed) {
      s = spec_lit(s, "@", &ok);
      s = spec_int(s, &out->stride[i], &ok);
      s = spec_lit(s, ",", &ok);
      s = spec_int(s, &out->rank_stride[i], &ok);
    }
    if (!ok) return -1;
    s = spec_ws(s);
    if (*s == '|') {
      ++s;
      continue;
    }
    break;
  }
  return (*spec_ws(s) == 0 && ok) ? 0 : -1;
}
static void spec_free(spec_decomp *d) {
  for (int i = 0; i < d->ndim; ++i) spec_free_dim(d->dims[i]);
  memset(d, 0, sizeof(*d));
}
#endif
