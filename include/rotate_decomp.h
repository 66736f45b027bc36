#ifndef DMG_ROTATE_DECOMP_H
#define DMG_ROTATE_DECOMP_H
/** @file rotate_decomp.h
 * Cyclic shift decorator (reference rotate_decomp.h:3-14):
 * maps g to nested((g + len + rotate) % len).
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct rotate_decomp {
  struct dim_decomp parent;
  int rotate;
  DimDecomp nested; /**< owned */
};
typedef struct rotate_decomp *RotateDecomp;

/** The plugin's hooks (reference rotate_decomp.h:10-12): rank and local offset of a
 * global coordinate, clone. */
int rotate_rank_offset(DimDecomp d, int global);
int rotate_type_offset(DimDecomp d, int global);
DimDecomp clone_rotate(DimDecomp d);
/** Rotate `nested` by `rotate`; clones `nested` (reference rotate_decomp.h:14). */
DimDecomp makeRotatedDecomp(int rotate, DimDecomp nested);
#ifdef __cplusplus
}
#endif
#endif
