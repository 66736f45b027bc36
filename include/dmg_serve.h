#ifndef DMG_SERVE_H
#define DMG_SERVE_H
/**
 * Served form of the split FFT: a request loop that runs reshape + split-FFT
 * jobs of mixed sizes as they arrive, with continuous batching.
 *
 * A job is one cube of side L (L^3 complex128 or complex64 values) on a
 * g x g virtual grid, given in the block decomposition
 * (block(L,g) | block(L,g) | local(L)).  Its work is the benchmark chain of
 * the reference's drivers (split_plan_test.c:276-326): reshape block ->
 * rotate (rotate(L/3, block) | rotate(1, block) | local), split 3D FFT
 * forward (spectrum in the plan's B decomposition, as runSplitPlan leaves it
 * in the workspace), then the inverse (N times the rotated input).
 *
 * The server owns one device arena.  A submitted job waits until a stream
 * slot is free and the arena has room for its buffers (admission by free
 * HBM); jobs of the same side and type that are waiting at that moment join
 * it, up to DMG_FFT_MAXBATCH, and their FFT passes run as shared persistent
 * launches.  Jobs in different slots overlap on the device.  Plans, with
 * their device address tables, are cached per (side, type).  A scheduler
 * thread does all of this; submit and poll only touch its queues.
 *
 * No counterpart in the reference, which runs one transform per call.
 */
#include "split_fft.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dmg_server *DmgServer;

/** One request.  Host arrays should be pinned (cudaHostAlloc) so that the
 * copies run asynchronously; they must stay valid until the job completes. */
typedef struct {
  int side;          /**< cube side L */
  int dtype;         /**< DMG_C128 or DMG_C64 */
  const void *input; /**< P * pitch_in values: the cube in the block decomposition */
  void *spectrum;    /**< P * extent_B values (rank r's B-layout result at r * extent_B), or NULL */
  void *output;      /**< P * pitch_rot values: the inverse result in the rotate decomposition, or NULL */
} dmg_job;

/** A completed job, with host times (seconds, CLOCK_MONOTONIC). */
typedef struct {
  long long id;
  double t_submit, t_start, t_done;
  int batch;  /**< jobs that shared its launches */
  int status; /**< DMG_OK or an error code */
} dmg_job_done;

/** A server on a g x g virtual grid with an arena of arena_bytes of device
 * memory and `slots` streams; max_batch jobs at most share launches (1: no
 * batching).  NULL on failure. */
DmgServer dmg_server_create(int grid, long long arena_bytes, int slots, int max_batch);
/** Arithmetic of the server's plans of one element type: DMG_ARITH_DF (the
 * default) or DMG_ARITH_FP64 for DMG_C128, DMG_ARITH_FP32 (the default) or
 * DMG_ARITH_TC16 for DMG_C64.  Applies to cached plans too; refused while
 * jobs are queued or running. */
int dmg_server_set_arith(DmgServer s, int dtype, int arith);
/** Mixing: jobs of sides up to max_side (and one element type) may share
 * launches with jobs of other such sides, the reshapes and every split-FFT
 * pass of a mixed batch in one launch each; the plans of those sides run the
 * runtime radix schedule DMG_RADIX_PLAN8.  0 (the default) batches only jobs
 * of one side.  Applies to cached plans too; refused while jobs are queued
 * or running. */
int dmg_server_set_mixing(DmgServer s, int max_side);
/** Element counts of a job's host arrays (input, spectrum, output). */
int dmg_server_job_sizes(DmgServer s, int side, int dtype, long long *input, long long *spectrum, long long *output);
/** Queue a job; returns its id (>= 0) or a negative error code.  A job that
 * could never fit the arena is refused here. */
long long dmg_server_submit(DmgServer s, const dmg_job *job);
/** Copy out up to max completed jobs (each reported once); returns the count. */
int dmg_server_poll(DmgServer s, dmg_job_done *done, int max);
/** Wait until every submitted job has completed. */
int dmg_server_drain(DmgServer s);
/** Jobs queued, running, and arena bytes in use. */
int dmg_server_status(DmgServer s, int *queued, int *running, long long *arena_used);
/** Finish the queued and running jobs, stop the scheduler thread and free
 * the arena, the streams and the cached plans. */
void dmg_server_destroy(DmgServer s);

#ifdef __cplusplus
}
#endif
#endif
