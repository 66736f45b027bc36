/*
 * TEST INFRASTRUCTURE (oracle).  CPU restatement of the reference's reshape
 * and split-FFT algorithms, used only to check results in tests, by the smoke
 * check, and as the benchmark's CPU baseline.  Never linked into the product.
 *
 * Decompositions are given as spec strings (spec.h) over P virtual ranks;
 * arrays are virtual-grid arrays (rank r's buffer at element r * pitch).
 */
#ifndef ORACLE_H
#define ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Per-rank facts of a decomposition: extents[r] (reference extent() on rank
 * r), proc_used.  Returns 0 on success. */
int oracle_decomp_info(int P, const char *spec, long long *extents, int *proc_used);

/* Element offset (within the virtual-grid array of the given pitch) of every
 * global coordinate in C order, -1 when no rank holds it.  `out` has
 * prod(L) entries.  Returns 0 on success. */
int oracle_global_offsets(int P, const char *spec, long long pitch, long long *out);

/* Reshape src -> dst following the reference's message algorithm: per rank,
 * per-peer typemaps built dimension by dimension in sort order, packed by
 * the sender and unpacked by the receiver.  nthreads worker threads.
 * Returns 0 on success, nonzero when the message sizes do not match. */
int oracle_reshape(int P, const char *src_spec, const char *dst_spec, int esize, long long src_pitch,
                   long long dst_pitch, const void *src, void *dst, int nthreads);

/* Processor grid search (reference processor_grid.c:24-97). */
int oracle_processor_grid(int P, int ndim, const int *tasks, int *grid);

/* Split-FFT plan facts (reference split_fft.c:249-614): mode 0 balanced
 * factors, 1 slab, 2 given B.  Fills A[ndim], B[ndim], grid_a, grid_b and
 * returns the spec strings of decompositions A and B (caller frees) through
 * a_spec/b_spec.  Returns 0 on success. */
int oracle_split_factors(int P, const char *start_spec, int mode, const int *Bin, int *A, int *B, int *grid_a,
                         int *grid_b, char *a_spec, char *b_spec, int speclen);

/* Forward split FFT restated on the CPU (reshape start->A, stage-1 FFT,
 * twiddle, reshape A->B, stage-2 FFT), every virtual rank on one of
 * nthreads threads.  dat is the start array (pitch dat_pitch), work the
 * workspace array (per-rank length work_len); the result is left in each
 * rank's work[0 .. extent).  direction -1 forward; +1 runs the
 * mathematically inverse sequence (stage-2 inverse, B->A, conjugate
 * twiddle, stage-1 inverse, A->start into dat).  Returns 0 on success. */
int oracle_split_fft(int P, const char *start_spec, int mode, const int *Bin, long long dat_pitch,
                     long long work_len, double *dat, double *work, int direction, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
