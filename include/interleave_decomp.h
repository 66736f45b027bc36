#ifndef DMG_INTERLEAVE_DECOMP_H
#define DMG_INTERLEAVE_DECOMP_H
/** @file interleave_decomp.h
 * Interleaved sub-sequences (reference interleave_decomp.h:5-29):
 * x = y + A*z with y in [0,A), z in [0,B).  The position comes from
 * nested(y); the offset is z + B * nested_offset(y), so each stride-A
 * sub-sequence is local and contiguous.
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct interleave_decomp {
  struct dim_decomp parent; /**< super-type */
  DimDecomp nested;         /**< decomposition of the y sub-coordinate (owned) */
  int A;                    /**< number of sequences (nested coord_size) */
  int B;                    /**< length of each sequence */
};
typedef struct interleave_decomp *InterleaveDecomp;

/** The plugin's hooks (reference interleave_decomp.h:20-23): rank and local offset of a
 * global coordinate, clone, print. */
int interleave_rank_offset(DimDecomp d, int global);
int interleave_type_offset(DimDecomp d, int global);
void print_interleave(FILE *out, DimDecomp d);
DimDecomp clone_interleave(DimDecomp d);
/** Interleave `B`-long sequences over the positions of `nested`; clones
 * `nested` (reference interleave_decomp.h:29). */
DimDecomp makeInterleaveDecomp(DimDecomp nested, int B);
#ifdef __cplusplus
}
#endif
#endif
