/*
 * A caller-defined DimDecomp plugin, as an application would write one
 * against the reference's plugin API (reshape.h:21-54): block-cyclic
 * distribution of `len` coordinates in blocks of `block` over `procs`
 * positions.  Coordinate g lies in block q = g / block, which goes to
 * position q % procs at local block q / procs:
 *   rank_offset(g) = (g / block) % procs
 *   type_offset(g) = (g / (block * procs)) * block + g % block
 * It uses only the plugin struct, calloc and memcpy, so the same source
 * compiles against this library's reshape.h and against the reference's.
 */
#include <stdlib.h>
#include <string.h>
#include "reshape.h"

struct block_cyclic {
  struct dim_decomp parent; /* first, so that a DimDecomp is a block_cyclic */
  int block;
};

static int bc_rank(DimDecomp d, int g) {
  const struct block_cyclic *b = (const struct block_cyclic *)d;
  return (g / b->block) % d->proc_size;
}

static int bc_offset(DimDecomp d, int g) {
  const struct block_cyclic *b = (const struct block_cyclic *)d;
  return (g / (b->block * d->proc_size)) * b->block + g % b->block;
}

static DimDecomp bc_clone(DimDecomp d) {
  struct block_cyclic *c = (struct block_cyclic *)calloc(1, sizeof(struct block_cyclic));
  if (c) memcpy(c, d, sizeof(struct block_cyclic));
  return (DimDecomp)c;
}

/* NULL unless len is a whole number of rounds of procs blocks */
DimDecomp make_block_cyclic(int len, int block, int procs) {
  if (block < 1 || procs < 1 || len % (block * procs) != 0) return NULL;
  struct block_cyclic *b = (struct block_cyclic *)calloc(1, sizeof(struct block_cyclic));
  if (!b) return NULL;
  b->parent.rank_offset = bc_rank;
  b->parent.type_offset = bc_offset;
  b->parent.destroy = NULL;
  b->parent.printer = NULL;
  b->parent.cloner = bc_clone;
  b->parent.type = "block_cyclic";
  b->parent.coord_size = len;
  b->parent.proc_size = procs;
  b->block = block;
  return (DimDecomp)b;
}
