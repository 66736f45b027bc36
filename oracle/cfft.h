/*
 * TEST INFRASTRUCTURE (oracle).  FP64 complex FFT on the CPU: mixed-radix
 * Stockham (radices 4, 2, 3, 5 and a direct DFT for other primes) with
 * twiddles computed in long double.  Used by the FFTW guru-API stub that the
 * reference is built against, and by the CPU restatement of the split FFT.
 * It stands in for FFTW 3, the third-party library the reference calls for
 * its stages (fftw_plan_guru_dft / fftw_execute, split_fft.c:461-534 and
 * 638-723; version not pinned by the reference, Makefile:8 links -lfftw3),
 * with FFTW's conventions: sign -1 forward, unnormalised backward.
 */
#ifndef ORACLE_CFFT_H
#define ORACLE_CFFT_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct cfft_plan cfft_plan;

/* Plan a length-n transform (n >= 1). */
cfft_plan *cfft_make(int n);
void cfft_free(cfft_plan *p);
/* In-place transform of n contiguous complex values (interleaved re, im);
 * sign -1 forward, +1 backward (unnormalised).  `work` holds 2n doubles. */
void cfft_exec(const cfft_plan *p, int sign, double *x, double *work);

/* Multi-dimensional strided transform, FFTW guru semantics: `rank`
 * transform dimensions (n, is, os) and `howmany_rank` loop dimensions, all
 * strides in complex elements.  in and out may be the same array. */
typedef struct {
  int n, is, os;
} cfft_dim;
void cfft_guru(int rank, const cfft_dim *dims, int howmany_rank, const cfft_dim *howmany, const double *in,
               double *out, int sign);

#ifdef __cplusplus
}
#endif
#endif
