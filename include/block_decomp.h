#ifndef DMG_BLOCK_DECOMP_H
#define DMG_BLOCK_DECOMP_H
/** @file block_decomp.h
 * Block distribution (reference block_decomp.h:5-27): position = g / blocksize,
 * offset = g % blocksize, blocksize = factor * ceil((len / factor) / procs).
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct block_decomp {
  struct dim_decomp parent; /**< super-type */
  int blocksize;            /**< largest block */
};
typedef struct block_decomp *BlockDecomp;

/** The plugin's hooks (reference block_decomp.h:13-14): rank and local offset of a
 * global coordinate. */
int block_rank_offset(DimDecomp d, int global);
int block_type_offset(DimDecomp d, int global);
/** Block decomposition of `len` coordinates over `proc` positions
 * (reference block_decomp.h:20). */
DimDecomp makeBlockDecomp(int len, int proc);
/** Block decomposition whose block size is a multiple of `factor`; NULL
 * when factor does not divide len (reference block_decomp.h:27). */
DimDecomp makeBlockDecompWithFactor(int len, int factor, int procs);
#ifdef __cplusplus
}
#endif
#endif
