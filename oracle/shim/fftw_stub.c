/* TEST INFRASTRUCTURE (oracle).  FFTW guru-API stub; see fftw3.h. */
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"
#include "../cfft.h"

struct fftw_plan_s {
  int rank, howmany_rank;
  cfft_dim dims[16], howmany[16];
  double *in, *out;
  int sign;
};

fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim *dims, int howmany_rank, const fftw_iodim *howmany_dims,
                             fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  if (rank < 0 || rank > 16 || howmany_rank < 0 || howmany_rank > 16) return NULL;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(struct fftw_plan_s));
  p->rank = rank;
  p->howmany_rank = howmany_rank;
  for (int d = 0; d < rank; ++d) {
    p->dims[d].n = dims[d].n;
    p->dims[d].is = dims[d].is;
    p->dims[d].os = dims[d].os;
  }
  for (int d = 0; d < howmany_rank; ++d) {
    p->howmany[d].n = howmany_dims[d].n;
    p->howmany[d].is = howmany_dims[d].is;
    p->howmany[d].os = howmany_dims[d].os;
  }
  p->in = (double *)in;
  p->out = (double *)out;
  p->sign = sign;
  return p;
}

void fftw_execute(const fftw_plan p) {
  if (p) cfft_guru(p->rank, p->dims, p->howmany_rank, p->howmany, p->in, p->out, p->sign);
}
void fftw_destroy_plan(fftw_plan p) { free(p); }
void *fftw_malloc(size_t n) { return malloc(n ? n : 1); }
void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
