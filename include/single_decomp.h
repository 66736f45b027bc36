#ifndef DMG_SINGLE_DECOMP_H
#define DMG_SINGLE_DECOMP_H
/** @file single_decomp.h
 * Every coordinate at one position (reference single_decomp.h:5-23);
 * offset = g.
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct single_decomp {
  struct dim_decomp parent; /**< super-type */
  int rank;                 /**< position holding the data */
};
typedef struct single_decomp *SingleDecomp;

/** The plugin's hooks (reference single_decomp.h:14-16): rank and local offset of a
 * global coordinate, clone. */
int single_rank_offset(DimDecomp d, int global);
int single_type_offset(DimDecomp d, int global);
DimDecomp single_clone(DimDecomp d);
/** All `coord_size` coordinates at position `rank` of `size` positions
 * (reference single_decomp.h:23). */
DimDecomp makeSingleDecomp(int coord_size, int rank, int size);
#ifdef __cplusplus
}
#endif
#endif
