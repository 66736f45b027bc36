#ifndef DMG_VISIT_H
#define DMG_VISIT_H
/**
 * Device visitors over every slot of a distributed array.
 *
 * The reference visits one rank's local slots on the host: visitData
 * (split_fft.c:862-889) calls a function per slot, and decomp_scale
 * (dimscale.c:7-67) multiplies every slot by the product of per-dimension
 * factors (the split FFT's twiddle).  On the virtual grid these run on the
 * device over all ranks at once.  Factors are indexed by global coordinate
 * (the reference indexes them by a rank's local position, which on one
 * process would need a table per rank).
 */
#include "reshape.h"

#ifdef __cplusplus
extern "C" {
#endif

/** data[x] *= f_0[x_0] * f_1[x_1] * ... for every global coordinate x the
 * decomposition holds (at most 3 dimensions), with the product formed in
 * dimension order as decomp_scale does (dimscale.c:7-67) and conjugated when
 * sign == 1; a slot whose product is 0 is left unchanged (the reference's
 * "unused index").  factors[d]: host array of L_d complex values
 * (interleaved re, im; double for complex128 data, float for complex64), or
 * NULL for all ones.  complex64: 0 for complex128 data, 1 for complex64.
 * Waits for the stream. */
int dmg_decomp_scale(Decomp d, int complex64, void *data, const void *const *factors, int sign, void *stream);

/** Set every slot the decomposition holds to its global C-order linear
 * index (4- or 8-byte integers): the value pattern of the reference's
 * test.c:27.  Waits for the stream. */
int dmg_visit_fill_index(Decomp d, int type_size, void *data, void *stream);

#ifdef __cplusplus
}
#endif
#endif
