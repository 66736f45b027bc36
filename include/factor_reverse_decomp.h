#ifndef DMG_FACTOR_REVERSE_DECOMP_H
#define DMG_FACTOR_REVERSE_DECOMP_H
/** @file factor_reverse_decomp.h
 * Factor-reversal decorator (reference factor_reverse_decomp.h:5-23):
 * maps g = y + A*z to nested(z + B*y), swapping the significance of the two
 * factors of the coordinate.  A*B must equal the nested size.
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct factor_reverse_decomp {
  struct dim_decomp parent;
  int A;
  int B;
  DimDecomp nested; /**< owned */
};
typedef struct factor_reverse_decomp *FactorReverseDecomp;

/** The plugin's hooks (reference factor_reverse_decomp.h:18-20): rank and local offset of a
 * global coordinate, clone. */
int factor_reverse_rank_offset(DimDecomp d, int global);
int factor_reverse_type_offset(DimDecomp d, int global);
DimDecomp clone_factor_reverse(DimDecomp d);
/** Factor-reverse `nested`; NULL when A*B != nested size; clones `nested`
 * (reference factor_reverse_decomp.h:21). */
DimDecomp makeFactorReverseDecomp(int A, int B, DimDecomp nested);
/** AxisDecomp over factor_reverse(A,B, orig's decomp) with orig's strides
 * (reference factor_reverse_decomp.h:23). */
AxisDecomp makeFactorReverseAxisDecomp(int A, int B, AxisDecomp orig);
#ifdef __cplusplus
}
#endif
#endif
