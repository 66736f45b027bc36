/*
 * Device visitors (include/dmg_visit.h), the device forms of decomp_scale
 * (reference dimscale.c:7-67) and of test.c:27's index fill: the
 * distributed array is gathered to global C order with the K1 permutation
 * kernel, visited element-wise, and scattered back.  Three passes over the array instead of one, which is
 * fine for initialisation and occasional scaling; the split FFT does not
 * use these (its twiddle is fused into the passes).
 */
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "dmg_io.h"
#include "dmg_visit.h"

int dmg_scale_global_launch(void *g, int complex64, int L0, int L1, int L2, const void *f0, const void *f1,
                            const void *f2, int conj_f, void *stream);
int dmg_iota_launch(void *g, int type_size, long long n, void *stream);

static long long count_of(Decomp d) {
  long long n = 1;
  for (int i = 0; i < d->ndim; ++i) n *= d->dims[i]->decomp->coord_size;
  return n;
}

int dmg_decomp_scale(Decomp d, int complex64, void *data, const void *const *factors, int sign, void *stream) {
  if (!d || !data) return dmg_error(DMG_ERR_ARG, "dmg_decomp_scale: bad arguments");
  if (d->ndim > 3) return dmg_error(DMG_ERR_UNSUPPORTED, "dmg_decomp_scale: %d dimensions (at most 3)", d->ndim);
  const int es = complex64 ? 8 : 16;
  const size_t real = complex64 ? sizeof(float) : sizeof(double);
  int L[3] = {1, 1, 1};
  size_t tab_bytes = 0;
  for (int i = 0; i < d->ndim; ++i) {
    L[i] = d->dims[i]->decomp->coord_size;
    tab_bytes += (size_t)L[i] * 2 * real;
  }
  tab_bytes += 3 * 2 * real; /* length-1 tables of the missing dimensions */
  const long long N = count_of(d);
  char *host = (char *)malloc(tab_bytes);
  if (!host) return dmg_error(DMG_ERR_NOMEM, "dmg_decomp_scale: host memory");
  void *dev_tab = NULL, *g = NULL;
  int st = dmg_dev_alloc(&dev_tab, tab_bytes);
  if (st == DMG_OK) st = dmg_dev_alloc(&g, (size_t)N * es);
  const void *dt[3] = {NULL, NULL, NULL};
  if (st == DMG_OK) {
    size_t pos = 0;
    for (int i = 0; i < 3; ++i) {
      const size_t bytes = (size_t)L[i] * 2 * real;
      if (i < d->ndim && factors && factors[i]) {
        memcpy(host + pos, factors[i], bytes);
      } else {
        for (int x = 0; x < L[i]; ++x) {
          if (complex64) {
            ((float *)(host + pos))[2 * x] = 1.0f;
            ((float *)(host + pos))[2 * x + 1] = 0.0f;
          } else {
            ((double *)(host + pos))[2 * x] = 1.0;
            ((double *)(host + pos))[2 * x + 1] = 0.0;
          }
        }
      }
      dt[i] = (char *)dev_tab + pos;
      pos += bytes;
    }
    st = dmg_dev_upload(dev_tab, host, pos);
  }
  if (st == DMG_OK) st = dmg_io_gather(d, es, data, g, stream);
  if (st == DMG_OK)
    st = dmg_scale_global_launch(g, complex64, L[0], L[1], L[2], dt[0], dt[1], dt[2], sign == 1, stream);
  if (st == DMG_OK) st = dmg_io_scatter(d, es, g, data, stream);
  if (g) dmg_dev_free(g);
  if (dev_tab) dmg_dev_free(dev_tab);
  free(host);
  return st;
}

int dmg_visit_fill_index(Decomp d, int type_size, void *data, void *stream) {
  if (!d || !data || (type_size != 4 && type_size != 8))
    return dmg_error(DMG_ERR_ARG, "dmg_visit_fill_index: bad arguments");
  const long long N = count_of(d);
  void *g = NULL;
  int st = dmg_dev_alloc(&g, (size_t)N * type_size);
  if (st == DMG_OK) st = dmg_iota_launch(g, type_size, N, stream);
  if (st == DMG_OK) st = dmg_io_scatter(d, type_size, g, data, stream);
  if (g) dmg_dev_free(g);
  return st;
}
