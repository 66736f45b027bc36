#ifndef SPLIT_FFT
#define SPLIT_FFT
/**
 * @file split_fft.h
 * Two-stage (split) parallel 3D FFT on the single-GPU virtual grid.
 *
 * Same plan-create / execute API as the reference's split_fft.h:10-63.
 * Each length L_i = A_i * B_i: stage 1 transforms the B_i-long stride-A_i
 * sub-sequences (x = y + A*z, over z), multiplies by exp(-2 pi i y k1 / L),
 * and stage 2 transforms the A_i-long ones, so that the B decomposition's
 * global slot s = k2 + A*k1 holds frequency k = k1 + B*k2.
 *
 * Buffers are device pointers to virtual-grid arrays: `dat` holds the input
 * in the `start` decomposition (rank r at element r * extent(start), or the
 * pitch set by dmg_split_set_dat_pitch); `workspace` holds every rank's
 * workspace of `length` elements (rank r at element r * length).  After a
 * forward run rank r's result is at workspace[r*length + 0 ..) in the B
 * decomposition, as in the reference.  The rest of each rank's workspace is
 * scratch.  runSplitPlan(FFTW_BACKWARD) runs the inverse of the forward
 * transform (unnormalised, FFTW convention): it reads the B-layout data in
 * the workspace and writes N times the original into `dat`.
 *
 * Data is complex128 unless the plan was made for complex64
 * (dmg_makeSplitPlanTyped); see DMG_ARITH_* for the arithmetic.  No FFTW,
 * cuFFT or CPU code runs: every pass is a hand-written sm_103a kernel.
 */
#include "reshape.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef FFTW_FORWARD
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#endif

/* FFTW's complex type: a C99 complex when <complex.h> came first, else double[2]. */
#if !defined(FFTW3_H) && !defined(ORACLE_SHIM_FFTW3_H)
#if defined(complex) && defined(_Complex_I) && !defined(__cplusplus)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif
#endif

struct dmg_split_impl;

/** Split-FFT plan (reference split_fft.h:10-30).  The FFTW plan fields of
 * the reference become the device pass lists held in `impl`; plan_a etc.
 * are non-NULL exactly when the reference would have built that FFTW plan. */
struct split_fft_plan {
  MPI_Comm comm;
  int *A_factors;        /**< A_i per dimension */
  Decomp A;              /**< stage-1 (interleaved) decomposition */
  Decomp B;              /**< stage-2 (blocked) decomposition, NULL when every A_i == 1 */
  Decomp B_flipped;      /**< the reference's output descriptor (see getTransformed) */
  fftw_complex *src;     /**< device pointer to dat (borrowed) */
  fftw_complex *work;    /**< device pointer to the workspace (borrowed) */
  int extent;            /**< largest extent of A and B over the virtual ranks */
  void *plan_a, *plan_b, *plan_a_back, *plan_b_back;
  ReshapePlan start_to_A, A_to_start, A_to_B, B_to_A;
  double **twiddle;      /**< NULL (twiddles live on the device) */
  double *times;         /**< [NUM_TIMERS] accumulated seconds, see dmg_split_collect_times */
  struct dmg_split_impl *impl;
};

/** Timer slots (reference split_fft.h:32-40). */
enum Timers { RESHAPE_1 = 0, FFT_1, TWIDDLE, RESHAPE_2, FFT_2, ALL, NUM_TIMERS };

/** Flags of proposeParallelPlan / buildParallelPlan (reference split_fft.h:42-47). */
enum SearchFlags { NO_FLAGS = 0x00, PREFER_LARGE_FFT = 0x01, PREFER_STAGE1 = 0x02, FORCE_USE_FIRST = 0x04 };

typedef struct split_fft_plan *SplitPlan;

/** Visitor over the local slots of a host copy of one rank's buffer
 * (reference split_fft.h:50).  global_position holds the slot's global
 * coordinate, or -1 entries for a slot that holds no data. */
typedef void (*data_visitor)(int ndim, int *global_position, double *dat);
/** Visit every slot 0..max_local of the buffer of the rank the descriptor
 * describes (the communicator's view rank when it was made), in host memory
 * as interleaved complex doubles (reference split_fft.h:51). */
void visitData(Decomp d, data_visitor vis, double *dat);

/** Build a plan for given factors and grids (reference split_fft.h:52).
 * NULL when the workspace is too small or a flag rejects the plan. */
SplitPlan buildParallelPlan(int flags, int use_first, int use_second, Decomp start, int ndim, int A[], int B[],
                            int L[], int a_grid[], int b_grid[], fftw_complex *dat, int length,
                            fftw_complex workspace[]);
/** Factors B given, grids from makeProcessorGrid (reference split_fft.h:53). */
SplitPlan proposeParallelPlan(int flags, Decomp start, int *initial_factor, fftw_complex *dat, int length,
                              fftw_complex workspace[]);
/** Exhaustive search over factors and grids, timing each candidate on the
 * GPU (reference split_fft.h:54). */
SplitPlan autotuneParallelPlan(Decomp start, fftw_complex *dat, int length, fftw_complex workspace[]);
/** The autotuner for a given element type (DMG_C128 or DMG_C64); full_grid_search = 1 walks every
 * processor grid of A and B as the reference does, 0 takes makeProcessorGrid's.  Besides the factors and
 * the pass schedule it chooses the tile size and the radix schedules (dmg_split_set_tile,
 * dmg_split_set_radix); winners are cached per (dimensions, lengths, virtual ranks, element type, grid
 * search, start decomposition), and a cached choice is built without timing.  The search runs forward
 * transforms over `dat` and `workspace`. */
SplitPlan dmg_autotuneParallelPlanTyped(Decomp start, void *dat, long long length, void *workspace, int dtype,
                                        int full_grid_search);
/** Forget every cached autotuning winner. */
void dmg_autotune_cache_clear(void);
/** Number of cached autotuning winners. */
int dmg_autotune_cache_entries(void);
/** Configurations the last autotuning call timed (0 when it built a cached choice). */
int dmg_autotune_last_timed(void);
/** Slab (slab=1: last dim in stage 2 only) or balanced factors A <= B
 * (reference split_fft.h:55). */
SplitPlan makeSplitPlan(int slab, Decomp start, fftw_complex *dat, int length, fftw_complex workspace[]);
/** proposeParallelPlan(NO_FLAGS, ...) (reference split_fft.h:56). */
SplitPlan makeParallelPlan(Decomp start, int *initial_factor, fftw_complex *dat, int length,
                           fftw_complex workspace[]);

/** The reference's output descriptor, unchanged: factor_reverse(A_i, B_i)
 * over B.  It places frequency k correctly only when A_i == B_i for every
 * dimension (reference split_fft.c:549-556); getTransformedExact() gives the
 * descriptor that is right for every factorisation. */
Decomp getTransformed(SplitPlan plan);
/** Output descriptor that maps every frequency k to the slot holding it:
 * factor_reverse(B_i, A_i) over B (slot s = k/B + A*(k%B)). */
Decomp getTransformedExact(SplitPlan plan);
/** Run forward (FFTW_FORWARD) or inverse (FFTW_BACKWARD) on the current
 * stream (reference split_fft.h:60). */
void runSplitPlan(SplitPlan plan, int direction);
/** Free a plan with its decompositions and device tables; the caller's
 * dat and workspace stay (reference split_fft.h:60). */
void freeSplitPlan(SplitPlan plan);
/** Interleaved decomposition: interleave(block(A_i, grid_i), B_i) packed
 * (reference split_fft.h:62). */
Decomp makeInterleavedDecomp(int ndim, MPI_Comm comm, int A[], int B[], int grid[]);
/** Blocked decomposition: block(A_i*B_i, factor A_i, grid_i) packed
 * (reference split_fft.h:63). */
Decomp makeBlockedDecomp(int ndim, MPI_Comm comm, int A[], int B[], int grid[]);
/** Binary GCD (reference split_fft.h:64). */
unsigned int gcd(unsigned int u, unsigned int v);

/* ---- GB300 additions ---- */
#define DMG_C128 0 /**< complex128 data, FP64 arithmetic */
#define DMG_C64 1  /**< complex64 data, FP32 arithmetic */

/** makeSplitPlan for a given element type (DMG_C128 or DMG_C64); `length`
 * is the per-rank workspace length in elements of that type. */
SplitPlan dmg_makeSplitPlanTyped(int slab, Decomp start, void *dat, long long length, void *workspace, int dtype);
/** makeParallelPlan for a given element type. */
SplitPlan dmg_makeParallelPlanTyped(Decomp start, int *initial_factor, void *dat, long long length,
                                    void *workspace, int dtype);
/* Arithmetic of the device passes.  complex128 plans run in double-float by
 * default: each real is an unevaluated sum of two floats (48-bit
 * significand, relative error around 1e-14 on a 512^3 transform), computed
 * on the FP32 pipes; the input is scaled by a power of two so any FP64
 * magnitude fits.  DMG_ARITH_FP64 computes in native FP64 instead (GB300's
 * FP64 rate is about 1/56 of its FP32 rate).  complex64 plans use FP32 by
 * default; DMG_ARITH_TC16 runs the DFTs of their 1024-point passes as two
 * 32-point DFT products on the tensor cores (FP16 hi + lo operands, three
 * products each, FP32 accumulation, a power-of-two scale per row; other
 * lengths keep the FP32 stages). */
#define DMG_ARITH_FP64 0
#define DMG_ARITH_FP32 1
#define DMG_ARITH_DF 2
#define DMG_ARITH_TC16 3
/** Select the arithmetic of a plan (DMG_ARITH_FP64 or DMG_ARITH_DF for
 * complex128; DMG_ARITH_FP32 or DMG_ARITH_TC16 for complex64). */
int dmg_split_set_arith(SplitPlan plan, int arith);
/** The plan's device status word, read back after the work queued so far
 * (a synchronising copy): 0 when every tensor-core pass completed its
 * products, 1 when one gave up waiting for them (its results are wrong);
 * negative on error. */
int dmg_split_device_status(SplitPlan plan);
/** The arithmetic a plan computes in (DMG_ARITH_*). */
int dmg_split_get_arith(SplitPlan plan);
/* Pass schedule.  Both give the reference's output in the same workspace
 * slots.  LINES: one pass per dimension transforms all L_d points at once
 * and stores them in slot order (one HBM round trip per dimension; needs
 * L_d <= 2048 for complex128, 4096 for complex64).  SPLIT: the reference's
 * two stages, a pass per factor of each dimension with the twiddle between.
 * AUTO (default): LINES when every L_d is at most 1024 (complex128) or 2048
 * (complex64), else SPLIT. */
#define DMG_SCHEDULE_AUTO 0
#define DMG_SCHEDULE_LINES 1
#define DMG_SCHEDULE_SPLIT 2
/** One run of a plan over `count` (at most 16) arrays at once, each with its
 * own dat and workspace (the plan's own buffers are not used), the passes of
 * all jobs sharing persistent launches.  scales[j]: a device int per job
 * for double-float plans (the input's exponent; NULL otherwise).  No
 * counterpart in the reference (which runs one plan per call). */
int dmg_split_run_batch(SplitPlan plan, int direction, void *stream, int count, void *const *dats, void *const *works,
                        int *const *scales);
/** The plan's extent (largest A / B extent over the ranks) as a 64-bit count;
 * the workspace needs 2 * extent per rank. */
long long dmg_split_extent64(SplitPlan plan);
/** Kernel launches of one dmg_split_run_batch call. */
int dmg_split_batch_launches(SplitPlan plan, int direction, int count);
/** Most plans in one dmg_split_run_group call. */
#define DMG_SPLIT_MAXGROUP 16
/** runSplitPlan on up to DMG_SPLIT_MAXGROUP different plans (any sizes,
 * decompositions and pass counts; no counterpart in the reference), each on
 * its own dat and workspace: the k-th passes of all plans share one launch,
 * so a group of small transforms takes as many pass launches as its longest
 * plan has passes.  Every plan must have a runtime radix schedule
 * (DMG_RADIX_PLAN8 or DMG_RADIX_PLAN4) and the same arithmetic; the results
 * are the bits of runSplitPlan on each plan.  Buffers of different plans
 * must not overlap. */
int dmg_split_run_group(int count, SplitPlan const *plans, int direction, void *stream);
/** The same as a job table: plan i transforms njobs[i] (1 to 16) arrays of
 * its shape, as dmg_split_run_batch does for one plan; dats, works and
 * scales (device int words, for double-float plans) list the arrays plan by
 * plan.  The plans' own dat and workspace are not used. */
int dmg_split_run_group_batch(int count, SplitPlan const *plans, const int *njobs, void *const *dats,
                              void *const *works, int *const *scales, int direction, void *stream);
/** Kernel launches of one dmg_split_run_group call (0 if the group is invalid). */
int dmg_split_group_launches(int count, SplitPlan const *plans, int direction);
/** Select the pass schedule (no counterpart in the reference). */
int dmg_split_set_schedule(SplitPlan plan, int schedule);
/** The schedule in use: DMG_SCHEDULE_LINES or DMG_SCHEDULE_SPLIT. */
int dmg_split_get_schedule(SplitPlan plan);
/** Values per pass tile: 0 for the default (4096 for complex64, 2048 for
 * complex128 in double-float, 1024 in native FP64), else a power of two from
 * 64 up to twice that.  Smaller tiles hold fewer lines side by side; larger
 * ones run the FP32 and double-float passes of power-of-two lengths
 * 256...2048 in one 512-thread block per SM (other passes keep the default),
 * so that passes whose lines are strided in memory move longer rows.  Native
 * FP64 passes take at most 1024 values (one line where a line is longer). */
int dmg_split_set_tile(SplitPlan plan, int values);
/** The plan's values per tile as set (0: the default, which gives FP32
 * passes whose lines are strided in memory the wide tiles and the others
 * the two-block kernels' tiles). */
int dmg_split_get_tile(SplitPlan plan);
/* Radix schedules of the passes: DMG_RADIX_FIXED runs the compile-time
 * schedules of the lengths that have one (powers of two 8...2048: radix 8
 * stages, 16 as 4 x 4; the 2,3,5-smooth cube sides) and the plan's radices
 * for the others; DMG_RADIX_PLAN8 and DMG_RADIX_PLAN4 run every pass with
 * the plan's radices in the runtime-length kernel, 8s first or 4s first. */
#define DMG_RADIX_FIXED 0
#define DMG_RADIX_PLAN8 1
#define DMG_RADIX_PLAN4 2
/** Select the passes' radix schedules (DMG_RADIX_*). */
int dmg_split_set_radix(SplitPlan plan, int radix);
/** The plan's radix schedule choice. */
int dmg_split_get_radix(SplitPlan plan);
/** Status-returning run on an explicit stream (NULL = legacy default). */
int dmg_split_run(SplitPlan plan, int direction, void *stream);
/** Rebind the device buffers of a plan (same sizes). */
int dmg_split_set_buffers(SplitPlan plan, void *dat, void *workspace);
/** Per-rank pitch (elements) of the dat array; default extent(start). */
int dmg_split_set_dat_pitch(SplitPlan plan, long long pitch);
/** Kernel launches one run makes. */
int dmg_split_launches(SplitPlan plan, int direction);
/** 5 N log2 N flops of one 3D transform (the conventional count). */
double dmg_split_flops(SplitPlan plan);
/** Turn per-phase CUDA-event timing on or off (off by default). */
int dmg_split_set_timing(SplitPlan plan, int on);
/** Synchronise and add the timed passes of the last timed run into
 * plan->times (FFT_1: stage-1 passes with the fused start->A move and
 * twiddle; FFT_2: stage-2 passes with the fused A->B move; ALL). */
int dmg_split_collect_times(SplitPlan plan);
/** Per-pass milliseconds of the last timed run in `direction` (timing on);
 * returns the number of passes or a negative error. */
int dmg_split_pass_times(SplitPlan plan, int direction, float *ms, int max);
/** Short description of the pass list. */
const char *dmg_split_describe(SplitPlan plan);

/** runSplitPlan for callers that cannot allocate device memory when they
 * run the transform: a real-time loop that must not wait on the allocator,
 * or an application that gives all of HBM to its own pool up front and so
 * has nothing left for a library to cudaMalloc.  It has no counterpart in
 * the reference (whose MPI ranks always own their workspace).
 *
 * The intermediate passes use a fixed device array of 64 MiB instead of
 * the upper half of each rank's workspace; `dat` and the B-layout output in
 * the workspace's lower half are the caller's buffers as usual.  The call
 * allocates nothing and makes no allocating library call:
 *  - the plan's address tables must already be on the device: any earlier
 *    dmg_split_run / runSplitPlan of the plan uploads them, otherwise the
 *    call returns DMG_ERR_ARG;
 *  - that upload also loads the array on the device (a device holds it from
 *    then until the process exits), so the call finds it in place;
 *  - the device the tables were uploaded on must be current, otherwise the
 *    call returns DMG_ERR_ARG;
 *  - plans needing more than 64 MiB of scratch (virtual ranks x extent x
 *    element size) are rejected with DMG_ERR_BOUNDS before any device work.
 * Every call uses the same array, and the passes overwrite whatever an
 * earlier call left there; calls that overlap on the GPU (different
 * streams, no ordering between them) race on it. */
int dmg_split_run_noalloc(SplitPlan plan, int direction, void *stream);
/** Size in bytes of the fixed scratch array used by dmg_split_run_noalloc. */
size_t dmg_noalloc_scratch_bytes(void);

/** Processor grid over the communicator's ranks for `ndim` task counts
 * (reference processor_grid.c:73-97); the caller frees the result. */
int *makeProcessorGrid(MPI_Comm comm, int ndim, int tasks[]);

#ifdef __cplusplus
}
#endif
#endif
