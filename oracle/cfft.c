/*
 * TEST INFRASTRUCTURE (oracle).  See cfft.h.
 *
 * Stockham autosort, decimation in time: with the radices r_1 r_2 ... of n,
 * stage s (radix p, Lp = product of earlier radices, L = Lp*p, m = n/L)
 * computes, for j < Lp and k < m,
 *     a_q = w_L^(j*q) * x[j*p*m + q*m + k]        (q < p)
 *     y[(j + s*Lp)*m + k] = sum_q a_q w_p^(q*s)   (s < p)
 * and leaves the transform in natural order after the last stage.
 */
#include "cfft.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

struct cfft_plan {
  int n;
  int nf;
  int fac[64];
  double *tw; /* exp(-2 pi i t / n), t < n */
};

cfft_plan *cfft_make(int n) {
  if (n < 1) return NULL;
  cfft_plan *p = (cfft_plan *)calloc(1, sizeof(cfft_plan));
  p->n = n;
  int m = n;
  while (m % 4 == 0) {
    p->fac[p->nf++] = 4;
    m /= 4;
  }
  while (m % 2 == 0) {
    p->fac[p->nf++] = 2;
    m /= 2;
  }
  for (int f = 3; (long)f * f <= m; f += 2) {
    while (m % f == 0) {
      p->fac[p->nf++] = f;
      m /= f;
    }
  }
  if (m > 1) p->fac[p->nf++] = m;
  p->tw = (double *)malloc(2 * (size_t)n * sizeof(double));
  for (int t = 0; t < n; ++t) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
    p->tw[2 * t] = (double)cosl(a);
    p->tw[2 * t + 1] = (double)sinl(a);
  }
  return p;
}

void cfft_free(cfft_plan *p) {
  if (!p) return;
  free(p->tw);
  free(p);
}

/* w_n^t with the requested sign */
static inline void twid(const cfft_plan *p, long t, int sign, double *re, double *im) {
  t %= p->n;
  *re = p->tw[2 * t];
  *im = sign < 0 ? p->tw[2 * t + 1] : -p->tw[2 * t + 1];
}

void cfft_exec(const cfft_plan *p, int sign, double *x, double *work) {
  const int n = p->n;
  if (n == 1) return;
  double *src = x, *dst = work;
  int Lp = 1;
  double are[64], aim[64];
  for (int f = 0; f < p->nf; ++f) {
    const int r = p->fac[f];
    const int L = Lp * r, m = n / L;
    const long tstep = n / L; /* w_L^1 = w_n^(n/L) */
    for (int j = 0; j < Lp; ++j) {
      for (int k = 0; k < m; ++k) {
        double *ar = are, *ai = aim;
        double big_r[r > 64 ? r : 1], big_i[r > 64 ? r : 1];
        if (r > 64) {
          ar = big_r;
          ai = big_i;
        }
        for (int q = 0; q < r; ++q) {
          const double *v = src + 2 * ((size_t)j * r * m + (size_t)q * m + k);
          double wr, wi;
          twid(p, tstep * j * q, sign, &wr, &wi);
          ar[q] = v[0] * wr - v[1] * wi;
          ai[q] = v[0] * wi + v[1] * wr;
        }
        double *out = dst + 2 * ((size_t)j * m + k);
        const size_t ostep = 2 * (size_t)Lp * m;
        if (r == 2) {
          out[0] = ar[0] + ar[1];
          out[1] = ai[0] + ai[1];
          out[ostep] = ar[0] - ar[1];
          out[ostep + 1] = ai[0] - ai[1];
        } else if (r == 4) {
          double s0r = ar[0] + ar[2], s0i = ai[0] + ai[2];
          double d0r = ar[0] - ar[2], d0i = ai[0] - ai[2];
          double s1r = ar[1] + ar[3], s1i = ai[1] + ai[3];
          double d1r = ar[1] - ar[3], d1i = ai[1] - ai[3];
          /* w_4 = -i (forward) or +i (backward) times d1 */
          double jr = sign < 0 ? d1i : -d1i, ji = sign < 0 ? -d1r : d1r;
          out[0] = s0r + s1r;
          out[1] = s0i + s1i;
          out[ostep] = d0r + jr;
          out[ostep + 1] = d0i + ji;
          out[2 * ostep] = s0r - s1r;
          out[2 * ostep + 1] = s0i - s1i;
          out[3 * ostep] = d0r - jr;
          out[3 * ostep + 1] = d0i - ji;
        } else {
          const long pstep = n / r; /* w_r^1 = w_n^(n/r) */
          for (int s = 0; s < r; ++s) {
            double sr = 0, si = 0;
            for (int q = 0; q < r; ++q) {
              double wr, wi;
              twid(p, pstep * ((long)q * s % r), sign, &wr, &wi);
              sr += ar[q] * wr - ai[q] * wi;
              si += ar[q] * wi + ai[q] * wr;
            }
            out[s * ostep] = sr;
            out[s * ostep + 1] = si;
          }
        }
      }
    }
    double *t = src;
    src = dst;
    dst = t;
    Lp = L;
  }
  if (src != x) memcpy(x, src, 2 * (size_t)n * sizeof(double));
}

void cfft_guru(int rank, const cfft_dim *dims, int howmany_rank, const cfft_dim *howmany, const double *in,
               double *out, int sign) {
  long total = 1;
  int maxn = 1;
  for (int d = 0; d < rank; ++d) {
    total *= dims[d].n;
    if (dims[d].n > maxn) maxn = dims[d].n;
  }
  cfft_plan *plans[16];
  for (int d = 0; d < rank; ++d) plans[d] = cfft_make(dims[d].n);
  double *tmp = (double *)malloc(2 * (size_t)total * sizeof(double));
  double *line = (double *)malloc(2 * (size_t)maxn * sizeof(double));
  double *work = (double *)malloc(2 * (size_t)maxn * sizeof(double));
  long nloop = 1;
  for (int h = 0; h < howmany_rank; ++h) nloop *= howmany[h].n;
  for (long it = 0; it < nloop; ++it) {
    long rem = it, ioff = 0, ooff = 0;
    for (int h = howmany_rank - 1; h >= 0; --h) {
      long c = rem % howmany[h].n;
      rem /= howmany[h].n;
      ioff += c * howmany[h].is;
      ooff += c * howmany[h].os;
    }
    /* gather the sub-array into C order */
    for (long e = 0; e < total; ++e) {
      long r2 = e, off = ioff;
      for (int d = rank - 1; d >= 0; --d) {
        off += (r2 % dims[d].n) * dims[d].is;
        r2 /= dims[d].n;
      }
      tmp[2 * e] = in[2 * off];
      tmp[2 * e + 1] = in[2 * off + 1];
    }
    /* transform each dimension in turn */
    long inner = total;
    for (int d = 0; d < rank; ++d) {
      int n = dims[d].n;
      inner /= n;
      long outer = total / (inner * n);
      for (long o = 0; o < outer; ++o) {
        for (long i = 0; i < inner; ++i) {
          double *base = tmp + 2 * (o * n * inner + i);
          for (int k = 0; k < n; ++k) {
            line[2 * k] = base[2 * k * inner];
            line[2 * k + 1] = base[2 * k * inner + 1];
          }
          cfft_exec(plans[d], sign, line, work);
          for (int k = 0; k < n; ++k) {
            base[2 * k * inner] = line[2 * k];
            base[2 * k * inner + 1] = line[2 * k + 1];
          }
        }
      }
    }
    for (long e = 0; e < total; ++e) {
      long r2 = e, off = ooff;
      for (int d = rank - 1; d >= 0; --d) {
        off += (r2 % dims[d].n) * dims[d].os;
        r2 /= dims[d].n;
      }
      out[2 * off] = tmp[2 * e];
      out[2 * off + 1] = tmp[2 * e + 1];
    }
  }
  for (int d = 0; d < rank; ++d) cfft_free(plans[d]);
  free(tmp);
  free(line);
  free(work);
}
