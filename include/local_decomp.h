#ifndef DMG_LOCAL_DECOMP_H
#define DMG_LOCAL_DECOMP_H
/** @file local_decomp.h
 * A non-distributed axis (reference local_decomp.h:4-17): one position,
 * offset = g.
 */
#include "reshape.h"
#ifdef __cplusplus
extern "C" {
#endif
struct local_decomp {
  struct dim_decomp parent;
};
typedef struct local_decomp *LocalDecomp;

/** The plugin's hooks (reference local_decomp.h:11-13): rank and local offset of a
 * global coordinate, clone. */
int local_rank_offset(DimDecomp d, int global);
int local_type_offset(DimDecomp d, int global);
DimDecomp local_clone(DimDecomp d);
/** Local axis of `len` coordinates (reference local_decomp.h:17). */
DimDecomp makeLocalDecomp(int len);
#ifdef __cplusplus
}
#endif
#endif
