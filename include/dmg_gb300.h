#ifndef DMG_GB300_H
#define DMG_GB300_H
/**
 * @file dmg_gb300.h
 * GB300 additions to the reference API: streams, error status, array
 * pitches, status-returning run calls and plan introspection.
 *
 * Streams are passed as `void *` (a cudaStream_t) so that this header does
 * not need the CUDA headers.  NULL means the legacy default stream.
 */
#include "reshape.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error status (replaces the reference's MPI_Abort paths) ---- */
#define DMG_OK 0
#define DMG_ERR_ARG 1         /**< invalid argument or descriptor */
#define DMG_ERR_UNSUPPORTED 2 /**< valid in the reference model but not supported here */
#define DMG_ERR_CUDA 3        /**< a CUDA call failed */
#define DMG_ERR_NOMEM 4       /**< host or device allocation failed */
#define DMG_ERR_BOUNDS 5      /**< an access would leave its buffer */
#define DMG_ERR_WORKSPACE 6   /**< workspace too small */

/** Message of the last error recorded on this thread ("" when none). */
const char *dmg_last_error(void);
/** Code of the last error recorded on this thread (DMG_OK when none). */
int dmg_last_error_code(void);
/** Clear this thread's error. */
void dmg_clear_error(void);
/** Print this thread's errors to stderr when they are recorded (default
 * on); returns the previous setting. */
int dmg_set_error_printing(int on);

/* ---- streams ---- */
/** Set the stream that run calls without an explicit stream use (this thread). */
void dmg_set_stream(void *stream);
/** The stream set by dmg_set_stream on this thread (NULL: the default stream). */
void *dmg_get_stream(void);
/** cudaDeviceSynchronize; returns DMG_OK or DMG_ERR_CUDA. */
int dmg_device_synchronize(void);

/* ---- reshape plans ---- */
/** Override the per-rank pitch (elements) of the src and dest virtual-grid
 * arrays; each must be at least the matching extent64().  Pass 0 to keep
 * the current value. */
int dmg_reshape_set_pitch(ReshapePlan plan, long long src_pitch, long long dest_pitch);
/** Status-returning run on an explicit stream.  src and dest must not
 * overlap. */
int dmg_reshape_run(ReshapePlan plan, const void *src, void *dest, void *stream);
/** Several reshapes, each with its own plan (any sizes and decompositions)
 * and buffers, enqueued on one stream: those whose data moves along one
 * contiguous axis on both sides (every packed layout) and that move units of
 * the same size share one persistent kernel launch, up to 16 per launch;
 * the others launch alone.  Each result is bit-identical to dmg_reshape_run
 * with the same plan and buffers.  No counterpart in the reference, where
 * every rank runs its own reshape. */
int dmg_reshape_run_group(int count, const ReshapePlan *plans, const void *const *srcs, void *const *dests,
                          void *stream);
/** Bytes one run reads plus writes (2 * elements moved * element size). */
long long dmg_reshape_bytes(ReshapePlan plan);
/** Number of elements one run moves. */
long long dmg_reshape_elements(ReshapePlan plan);
/** Per-rank pitch (elements) of the src (which=0) or dest (which=1) array. */
long long dmg_reshape_pitch(ReshapePlan plan, int which);
/** Short description of how the plan runs on the device (address mode,
 * tile axes, vector width); the string lives as long as the plan. */
const char *dmg_reshape_describe(ReshapePlan plan);
/** Kernel launches one run makes. */
int dmg_reshape_launches(ReshapePlan plan);

#ifdef __cplusplus
}
#endif
#endif
