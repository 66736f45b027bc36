#ifndef DMG_INTERNAL_H
#define DMG_INTERNAL_H
/* Internal helpers shared by the host-side C sources. */
#include <stdint.h>
#include "reshape.h"
#include "dmg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Record an error with a code; returns the code. */
int dmg_error(int code, const char *fmt, ...);

/* Sentinel added to an address table entry for a coordinate that a side does
 * not hold.  Eight of them still sum to a negative int64, and no real address
 * comes near 2^58 elements. */
#define DMG_ABSENT (-(((int64_t)1) << 58))

/* Position of virtual rank r along axis a: (r / rank_stride) % proc_size
 * (reference reshape.c:72). */
static inline int dmg_axis_pos(AxisDecomp a, int r) {
  return (r / a->rank_stride) % a->decomp->proc_size;
}

/* Is the virtual comm valid. */
int dmg_comm_ok(MPI_Comm comm);

/* Per-virtual-rank memory stride of axis a. */
static inline long long dmg_axis_stride(AxisDecomp a, int r) {
  return a->rank_memory_stride ? a->rank_memory_stride[r] : (long long)a->memory_stride;
}

/* Does virtual rank r hold data in d (every axis has local points at r's position). */
int dmg_rank_holds(Decomp d, int r);

/* Order of dimensions, fastest first, computed from the src strides seen by
 * rank r (reference reshape.c:330-350). */
void dmg_sort_order(int ndim, int *order, Decomp src, int r);

/* Proper processor grid: rank = sum rank_stride_i * pos_i inverts the
 * positions for every data-holding rank and no rank holds a copy of
 * another's data.  DMG_OK or an error code (recorded). */
int dmg_check_proper_grid(Decomp D, const char *side);

/* Split-plan autotuner: times candidate factorisations on the GPU. */
struct split_fft_plan;
struct split_fft_plan *dmg_autotune_split(Decomp start, void *dat, long long length, void *workspace, int dtype,
                                          int full_grid_search);

/* Device-side helpers implemented in the CUDA sources. */
int dmg_dev_alloc(void **ptr, size_t bytes);
void dmg_dev_free(void *ptr);
int dmg_dev_upload(void *dst, const void *src, size_t bytes);
void *dmg_current_stream(void);
int dmg_copy_sync(void *dst, const void *src, size_t bytes, int to_host, void *stream);
int dmg_stream_sync(void *stream);
int dmg_rt_stream_create(void **s);
void dmg_rt_stream_destroy(void *s);
int dmg_rt_event_create(void **ev);
void dmg_rt_event_destroy(void *ev);
int dmg_rt_event_record(void *ev, void *s);
int dmg_rt_event_done(void *ev);
int dmg_rt_copy_async(void *dst, const void *src, size_t bytes, int kind, void *s);
int dmg_rt_copy2d_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                        int kind, void *s);
int dmg_rt_get_device(int *dev);
int dmg_rt_set_device(int dev);

#ifdef __cplusplus
}
#endif
#endif
