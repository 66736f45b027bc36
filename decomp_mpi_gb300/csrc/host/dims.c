/*
 * The six per-axis decomposition plugins and the generic DimDecomp calls.
 *
 * Each map is a pure integer function of the global coordinate; the
 * formulas are the reference's (block_decomp.c:6-13, interleave_decomp.c:6-20,
 * rotate_decomp.c:28-33, factor_reverse_decomp.c:27-34, single_decomp.c:6-12,
 * local_decomp.c:6-11).  Decorators own a clone of the decomp they wrap and
 * free it when they are freed.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "block_decomp.h"
#include "interleave_decomp.h"
#include "rotate_decomp.h"
#include "factor_reverse_decomp.h"
#include "single_decomp.h"
#include "local_decomp.h"

/* ---- generic ---- */

void freeDimDecomp(DimDecomp d) {
  if (!d) return;
  if (d->destroy) d->destroy(d);
  free(d);
}

DimDecomp cloneDimDecomp(DimDecomp d) {
  if (!d || !d->cloner) return NULL;
  return d->cloner(d);
}

int sizeDimDecomp(DimDecomp d) { return d->coord_size; }

void describeDimDecomp(FILE *out, DimDecomp d) {
  fprintf(out, "DimDecomp(%s) coords=%d procs=%d", d->type ? d->type : "?", d->coord_size,
          d->proc_size);
  if (d->printer) d->printer(out, d);
}

/* ---- block ---- */

int block_rank_offset(DimDecomp d, int global) { return global / ((BlockDecomp)d)->blocksize; }
int block_type_offset(DimDecomp d, int global) { return global % ((BlockDecomp)d)->blocksize; }

static void block_print(FILE *out, DimDecomp d) {
  fprintf(out, " blocksize=%d", ((BlockDecomp)d)->blocksize);
}
static DimDecomp block_clone(DimDecomp d) {
  BlockDecomp c = (BlockDecomp)calloc(1, sizeof(struct block_decomp));
  if (c) *c = *(BlockDecomp)d;
  return (DimDecomp)c;
}

DimDecomp makeBlockDecomp(int len, int procs) { return makeBlockDecompWithFactor(len, 1, procs); }

DimDecomp makeBlockDecompWithFactor(int len, int factor, int procs) {
  if (factor < 1 || procs < 1 || len < 1 || len % factor != 0) return NULL;
  BlockDecomp b = (BlockDecomp)calloc(1, sizeof(struct block_decomp));
  if (!b) return NULL;
  b->parent.coord_size = len;
  b->parent.proc_size = procs;
  b->parent.rank_offset = block_rank_offset;
  b->parent.type_offset = block_type_offset;
  b->parent.printer = block_print;
  b->parent.cloner = block_clone;
  b->parent.destroy = NULL;
  b->parent.type = "block";
  /* blocks of a whole number of factors, ceil((len/factor)/procs) of them */
  int units = len / factor;
  b->blocksize = factor * ((units + procs - 1) / procs);
  return (DimDecomp)b;
}

/* ---- interleave ---- */

int interleave_rank_offset(DimDecomp d, int global) {
  InterleaveDecomp s = (InterleaveDecomp)d;
  return s->nested->rank_offset(s->nested, global % s->A);
}
int interleave_type_offset(DimDecomp d, int global) {
  InterleaveDecomp s = (InterleaveDecomp)d;
  int y = global % s->A, z = global / s->A;
  return z + s->B * s->nested->type_offset(s->nested, y);
}
static void interleave_destroy(DimDecomp d) { freeDimDecomp(((InterleaveDecomp)d)->nested); }
void print_interleave(FILE *out, DimDecomp d) {
  InterleaveDecomp s = (InterleaveDecomp)d;
  fprintf(out, " A=%d B=%d nested:", s->A, s->B);
  describeDimDecomp(out, s->nested);
}
DimDecomp clone_interleave(DimDecomp d) {
  InterleaveDecomp c = (InterleaveDecomp)calloc(1, sizeof(struct interleave_decomp));
  if (!c) return NULL;
  *c = *(InterleaveDecomp)d;
  c->nested = cloneDimDecomp(((InterleaveDecomp)d)->nested);
  return (DimDecomp)c;
}
DimDecomp makeInterleaveDecomp(DimDecomp nested, int B) {
  if (!nested || B < 1) return NULL;
  InterleaveDecomp s = (InterleaveDecomp)calloc(1, sizeof(struct interleave_decomp));
  if (!s) return NULL;
  s->A = nested->coord_size;
  s->B = B;
  s->parent.coord_size = s->A * B;
  s->parent.proc_size = nested->proc_size;
  s->parent.rank_offset = interleave_rank_offset;
  s->parent.type_offset = interleave_type_offset;
  s->parent.destroy = interleave_destroy;
  s->parent.printer = print_interleave;
  s->parent.cloner = clone_interleave;
  s->parent.type = "interleave";
  s->nested = cloneDimDecomp(nested);
  return (DimDecomp)s;
}

/* ---- rotate ---- */

static int rotate_coord(RotateDecomp r, int global) {
  int len = r->parent.coord_size;
  return (global + len + r->rotate) % len;
}
int rotate_rank_offset(DimDecomp d, int global) {
  RotateDecomp r = (RotateDecomp)d;
  return r->nested->rank_offset(r->nested, rotate_coord(r, global));
}
int rotate_type_offset(DimDecomp d, int global) {
  RotateDecomp r = (RotateDecomp)d;
  return r->nested->type_offset(r->nested, rotate_coord(r, global));
}
static void rotate_destroy(DimDecomp d) { freeDimDecomp(((RotateDecomp)d)->nested); }
static void rotate_print(FILE *out, DimDecomp d) {
  RotateDecomp r = (RotateDecomp)d;
  fprintf(out, " rotate=%d nested:", r->rotate);
  describeDimDecomp(out, r->nested);
}
DimDecomp clone_rotate(DimDecomp d) {
  RotateDecomp c = (RotateDecomp)calloc(1, sizeof(struct rotate_decomp));
  if (!c) return NULL;
  *c = *(RotateDecomp)d;
  c->nested = cloneDimDecomp(((RotateDecomp)d)->nested);
  return (DimDecomp)c;
}
DimDecomp makeRotatedDecomp(int rotate, DimDecomp nested) {
  if (!nested) return NULL;
  RotateDecomp r = (RotateDecomp)calloc(1, sizeof(struct rotate_decomp));
  if (!r) return NULL;
  r->parent.coord_size = nested->coord_size;
  r->parent.proc_size = nested->proc_size;
  r->parent.rank_offset = rotate_rank_offset;
  r->parent.type_offset = rotate_type_offset;
  r->parent.destroy = rotate_destroy;
  r->parent.printer = rotate_print;
  r->parent.cloner = clone_rotate;
  r->parent.type = "rotate";
  r->rotate = rotate;
  r->nested = cloneDimDecomp(nested);
  return (DimDecomp)r;
}

/* ---- factor_reverse ---- */

static int factor_reverse_coord(FactorReverseDecomp f, int global) {
  int y = global % f->A, z = global / f->A;
  return z + f->B * y;
}
int factor_reverse_rank_offset(DimDecomp d, int global) {
  FactorReverseDecomp f = (FactorReverseDecomp)d;
  return f->nested->rank_offset(f->nested, factor_reverse_coord(f, global));
}
int factor_reverse_type_offset(DimDecomp d, int global) {
  FactorReverseDecomp f = (FactorReverseDecomp)d;
  return f->nested->type_offset(f->nested, factor_reverse_coord(f, global));
}
static void factor_reverse_destroy(DimDecomp d) { freeDimDecomp(((FactorReverseDecomp)d)->nested); }
static void factor_reverse_print(FILE *out, DimDecomp d) {
  FactorReverseDecomp f = (FactorReverseDecomp)d;
  fprintf(out, " A=%d B=%d nested:", f->A, f->B);
  describeDimDecomp(out, f->nested);
}
DimDecomp clone_factor_reverse(DimDecomp d) {
  FactorReverseDecomp c = (FactorReverseDecomp)calloc(1, sizeof(struct factor_reverse_decomp));
  if (!c) return NULL;
  *c = *(FactorReverseDecomp)d;
  c->nested = cloneDimDecomp(((FactorReverseDecomp)d)->nested);
  return (DimDecomp)c;
}
DimDecomp makeFactorReverseDecomp(int A, int B, DimDecomp nested) {
  if (!nested) return NULL;
  if (A < 1 || B < 1 || A * B != nested->coord_size) {
    fprintf(stderr, "FactorReverse: factors do not equal size\n");
    return NULL;
  }
  FactorReverseDecomp f = (FactorReverseDecomp)calloc(1, sizeof(struct factor_reverse_decomp));
  if (!f) return NULL;
  f->parent.coord_size = nested->coord_size;
  f->parent.proc_size = nested->proc_size;
  f->parent.rank_offset = factor_reverse_rank_offset;
  f->parent.type_offset = factor_reverse_type_offset;
  f->parent.destroy = factor_reverse_destroy;
  f->parent.printer = factor_reverse_print;
  f->parent.cloner = clone_factor_reverse;
  f->parent.type = "factor_reverse";
  f->A = A;
  f->B = B;
  f->nested = cloneDimDecomp(nested);
  return (DimDecomp)f;
}

/* ---- single ---- */

int single_rank_offset(DimDecomp d, int global) {
  (void)global;
  return ((SingleDecomp)d)->rank;
}
int single_type_offset(DimDecomp d, int global) {
  (void)d;
  return global;
}
static void single_print(FILE *out, DimDecomp d) { fprintf(out, " rank=%d", ((SingleDecomp)d)->rank); }
DimDecomp single_clone(DimDecomp d) {
  SingleDecomp c = (SingleDecomp)calloc(1, sizeof(struct single_decomp));
  if (c) *c = *(SingleDecomp)d;
  return (DimDecomp)c;
}
DimDecomp makeSingleDecomp(int coord_size, int rank, int size) {
  if (coord_size < 1 || size < 1) return NULL;
  SingleDecomp s = (SingleDecomp)calloc(1, sizeof(struct single_decomp));
  if (!s) return NULL;
  s->parent.coord_size = coord_size;
  s->parent.proc_size = size;
  s->parent.rank_offset = single_rank_offset;
  s->parent.type_offset = single_type_offset;
  s->parent.destroy = NULL;
  s->parent.printer = single_print;
  s->parent.cloner = single_clone;
  s->parent.type = "single";
  s->rank = rank;
  return (DimDecomp)s;
}

/* ---- local ---- */

int local_rank_offset(DimDecomp d, int global) {
  (void)d;
  (void)global;
  return 0;
}
int local_type_offset(DimDecomp d, int global) {
  (void)d;
  return global;
}
DimDecomp local_clone(DimDecomp d) {
  LocalDecomp c = (LocalDecomp)calloc(1, sizeof(struct local_decomp));
  if (c) *c = *(LocalDecomp)d;
  return (DimDecomp)c;
}
DimDecomp makeLocalDecomp(int len) {
  if (len < 1) return NULL;
  LocalDecomp l = (LocalDecomp)calloc(1, sizeof(struct local_decomp));
  if (!l) return NULL;
  l->parent.coord_size = len;
  l->parent.proc_size = 1;
  l->parent.rank_offset = local_rank_offset;
  l->parent.type_offset = local_type_offset;
  l->parent.destroy = NULL;
  l->parent.printer = NULL;
  l->parent.cloner = local_clone;
  l->parent.type = "local";
  return (DimDecomp)l;
}
