/*
 * TEST INFRASTRUCTURE (oracle).  The subset of FFTW 3's API that the
 * reference calls (split_fft.c:428-541, split_plan_test.c:260-262), written
 * for this project and backed by the oracle's FP64 CPU FFT (cfft.c).
 * FFTW itself is not installed; this stub only stands in for it so that the
 * reference's sources build.  As in FFTW, fftw_complex is a C99 complex when
 * <complex.h> was included first, else double[2].
 */
#ifndef ORACLE_SHIM_FFTW3_H
#define ORACLE_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
#if defined(complex) && defined(_Complex_I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif
typedef struct fftw_plan_s *fftw_plan;
typedef struct {
  int n, is, os;
} fftw_iodim;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim *dims, int howmany_rank, const fftw_iodim *howmany_dims,
                             fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
#ifdef __cplusplus
}
#endif
#endif
