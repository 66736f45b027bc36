// Batched FFT pass with fused layout change and split twiddle.
//
// One launch transforms every line along one sub-axis t of the split
// coordinates (x_d = y_d + A_d*z_d) and writes the result in another layout.
// A block owns tiles of n x M1 x M2 values: it gathers them from the input
// layout in the order that is contiguous there (through the per-dimension
// address tables), runs a Stockham autosort FFT over the n-long lines in
// shared memory (radix 8, 4, 2, 3, 5 butterflies, other primes by direct
// DFT), optionally multiplies by the split twiddle prod_d exp(-+2 pi i y_d
// k1_d / L_d) from FP64 tables, and scatters the tile to the output layout in
// the order contiguous there.  Launches are persistent over the tiles.
//
// Stockham stage with radix r, Lp = product of earlier radices, m = n/(Lp r):
//   a_q = w_{Lp r}^{j q} * x[j r m + q m + k],  y[(j + s Lp) m + k] = sum_q a_q w_r^{q s}
// (j < Lp, k < m); the result is in natural order after the last stage.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "../host/dmg_internal.h"
#include "../host/fft_params.h"

namespace {

constexpr int NT = 128;
constexpr int TILE_MAX = 4096;  // complex values per tile buffer (one 4096-long line at most)

template <typename T>
using C2 = typename std::conditional<std::is_same<T, double>::value, double2, float2>::type;

template <typename T>
__device__ __forceinline__ C2<T> mk(T x, T y) {
  C2<T> r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename T>
__device__ __forceinline__ C2<T> add(C2<T> a, C2<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T>
__device__ __forceinline__ C2<T> sub(C2<T> a, C2<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T>
__device__ __forceinline__ C2<T> mul(C2<T> a, C2<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ C2<T> scl(C2<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// multiply by sign*i
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> rot90(C2<T> a) {
  return SIGN < 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}

// mathematical constants
#define DMG_SQRT1_2 0.707106781186547524400844362104849039
#define DMG_SQRT3_2 0.866025403784438646763723170752936183
#define DMG_C72 0.309016994374947424102293417182819059   // cos(2 pi / 5)
#define DMG_C144 -0.809016994374947424102293417182819059 // cos(4 pi / 5)
#define DMG_S72 0.951056516295153572116439333379382143   // sin(2 pi / 5)
#define DMG_S144 0.587785252292473129168705954639072769  // sin(4 pi / 5)

template <typename T, int SIGN>
__device__ __forceinline__ void dft4(C2<T> &a0, C2<T> &a1, C2<T> &a2, C2<T> &a3) {
  C2<T> t0 = add<T>(a0, a2), t1 = sub<T>(a0, a2), t2 = add<T>(a1, a3), t3 = rot90<T, SIGN>(sub<T>(a1, a3));
  a0 = add<T>(t0, t2);
  a2 = sub<T>(t0, t2);
  a1 = add<T>(t1, t3);
  a3 = sub<T>(t1, t3);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft8(C2<T> *a) {
  C2<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  C2<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<T, SIGN>(e0, e1, e2, e3);
  dft4<T, SIGN>(o0, o1, o2, o3);
  const T c = (T)DMG_SQRT1_2;
  // o1 *= (1 + sign i) c ; o2 *= sign i ; o3 *= (-1 + sign i) c
  C2<T> w1 = SIGN < 0 ? mk<T>(c * (o1.x + o1.y), c * (o1.y - o1.x)) : mk<T>(c * (o1.x - o1.y), c * (o1.y + o1.x));
  C2<T> w2 = rot90<T, SIGN>(o2);
  C2<T> w3 = SIGN < 0 ? mk<T>(c * (o3.y - o3.x), -c * (o3.x + o3.y)) : mk<T>(-c * (o3.x + o3.y), c * (o3.x - o3.y));
  a[0] = add<T>(e0, o0);
  a[4] = sub<T>(e0, o0);
  a[1] = add<T>(e1, w1);
  a[5] = sub<T>(e1, w1);
  a[2] = add<T>(e2, w2);
  a[6] = sub<T>(e2, w2);
  a[3] = add<T>(e3, w3);
  a[7] = sub<T>(e3, w3);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft3(C2<T> *a) {
  C2<T> s = add<T>(a[1], a[2]);
  C2<T> d = sub<T>(a[1], a[2]);
  C2<T> m = mk<T>(a[0].x - (T)0.5 * s.x, a[0].y - (T)0.5 * s.y);
  C2<T> r = rot90<T, SIGN>(scl<T>(d, (T)DMG_SQRT3_2));
  a[0] = add<T>(a[0], s);
  a[1] = add<T>(m, r);
  a[2] = sub<T>(m, r);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft5(C2<T> *a) {
  C2<T> b1 = add<T>(a[1], a[4]), b2 = add<T>(a[2], a[3]);
  C2<T> d1 = sub<T>(a[1], a[4]), d2 = sub<T>(a[2], a[3]);
  const T c1 = (T)DMG_C72, c2 = (T)DMG_C144, s1 = (T)DMG_S72, s2 = (T)DMG_S144;
  C2<T> p1 = mk<T>(a[0].x + c1 * b1.x + c2 * b2.x, a[0].y + c1 * b1.y + c2 * b2.y);
  C2<T> p2 = mk<T>(a[0].x + c2 * b1.x + c1 * b2.x, a[0].y + c2 * b1.y + c1 * b2.y);
  C2<T> q1 = rot90<T, SIGN>(mk<T>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
  C2<T> q2 = rot90<T, SIGN>(mk<T>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
  a[0] = add<T>(a[0], add<T>(b1, b2));
  a[1] = add<T>(p1, q1);
  a[4] = sub<T>(p1, q1);
  a[2] = add<T>(p2, q2);
  a[3] = sub<T>(p2, q2);
}

template <typename T>
__device__ __forceinline__ int64_t layout_addr(const dmg_fft_layout &L, int ndim, const int *x) {
  if (!L.ranked) {
    int64_t a = L.base;
#pragma unroll
    for (int d = 0; d < DMG_FFT_MAXDIM; ++d)
      if (d < ndim) a += __ldg(L.tab[d] + x[d]);
    return a;
  }
  int32_t R = 0;
#pragma unroll
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d)
    if (d < ndim) R += __ldg(L.rk[d] + x[d]);
  int64_t a = L.base + (int64_t)R * L.pitch;
#pragma unroll
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d)
    if (d < ndim) a += __ldg(L.tab[d] + x[d]) * __ldg(L.rstride + (size_t)d * L.nranks + R);
  return a;
}

// Tile-axis coordinates (c0 = t, c1 = v1, c2 = v2) of a linear index e in an
// order given by each axis's position (0 fastest); selects, no indexing.
__device__ __forceinline__ void tile_coords(int e, const int32_t *pos, int n0, int n1, int n2, int &c0, int &c1,
                                            int &c2) {
  // extents in order: fast, mid
  const int ef = pos[0] == 0 ? n0 : pos[1] == 0 ? n1 : n2;
  const int em = pos[0] == 1 ? n0 : pos[1] == 1 ? n1 : n2;
  const int i_f = e % ef;
  const int rest = e / ef;
  const int i_m = rest % em;
  const int i_s = rest / em;
  c0 = pos[0] == 0 ? i_f : pos[0] == 1 ? i_m : i_s;
  c1 = pos[1] == 0 ? i_f : pos[1] == 1 ? i_m : i_s;
  c2 = pos[2] == 0 ? i_f : pos[2] == 1 ? i_m : i_s;
}

// Global coordinates x_d of the element at tile offsets (c0, c1, c2).
__device__ __forceinline__ void element_x(const dmg_fft_pass &p, const int *yb, const int *zb, int c0, int c1, int c2,
                                          int *x) {
#pragma unroll
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    int y = yb[d], z = zb[d];
    y += (p.kdim[0] == d && !p.kisz[0]) ? c0 : 0;
    z += (p.kdim[0] == d && p.kisz[0]) ? c0 : 0;
    y += (p.kdim[1] == d && !p.kisz[1]) ? c1 : 0;
    z += (p.kdim[1] == d && p.kisz[1]) ? c1 : 0;
    y += (p.kdim[2] == d && !p.kisz[2]) ? c2 : 0;
    z += (p.kdim[2] == d && p.kisz[2]) ? c2 : 0;
    x[d] = y + p.A[d] * z;
  }
}

template <typename T, int SIGN>
__global__ void __launch_bounds__(NT) fft_pass_kernel(const dmg_fft_pass p, const C2<T> *__restrict__ src,
                                                      C2<T> *__restrict__ dst) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int n = p.n;
  const int ld = (n & 1) ? n : n + 1;
  const int nlines = p.M1 * p.M2;
  C2<T> *bufA = reinterpret_cast<C2<T> *>(sm);
  C2<T> *bufB = bufA + (size_t)nlines * ld;
  C2<T> *roots = bufB + (size_t)nlines * ld;
  const int tid = threadIdx.x;
  {
    const C2<T> *gr = reinterpret_cast<const C2<T> *>(p.roots);
    for (int i = tid; i < n; i += NT) {
      C2<T> w = gr[i];
      if (SIGN > 0) w.y = -w.y;
      roots[i] = w;
    }
  }
  __shared__ int s_yb[DMG_FFT_MAXDIM], s_zb[DMG_FFT_MAXDIM];
  __shared__ int s_lim1, s_lim2, s_ytw;
  // the transformed dimension and, for its twiddle, which vector axes carry its y
  const int td = p.t >> 1;
  const C2<T> *twt = reinterpret_cast<const C2<T> *>(p.tw[td]);
  const bool v1_ytd = p.kdim[1] == td && !p.kisz[1];
  const bool v2_ytd = p.kdim[2] == td && !p.kisz[2];

  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    __syncthreads();
    if (tid == 0) {
      int64_t t = tile;
      const int i1 = (int)(t % p.nt1);
      t /= p.nt1;
      const int i2 = (int)(t % p.nt2);
      t /= p.nt2;
      for (int d = 0; d < DMG_FFT_MAXDIM; ++d) s_yb[d] = s_zb[d] = 0;
      for (int b = 0; b < p.nbatch; ++b) {
        const int c = (int)(t % p.blen[b]);
        t /= p.blen[b];
        const int s = p.bsub[b];
        if (s & 1) s_zb[s >> 1] += c;
        else s_yb[s >> 1] += c;
      }
      if (p.v1 >= 0) {
        if (p.v1 & 1) s_zb[p.v1 >> 1] += i1 * p.M1;
        else s_yb[p.v1 >> 1] += i1 * p.M1;
      }
      if (p.v2 >= 0) {
        if (p.v2 & 1) s_zb[p.v2 >> 1] += i2 * p.M2;
        else s_yb[p.v2 >> 1] += i2 * p.M2;
      }
      s_ytw = s_yb[td];
      s_lim1 = p.v1 >= 0 ? min(p.M1, p.nv1 - i1 * p.M1) : 1;
      s_lim2 = p.v2 >= 0 ? min(p.M2, p.nv2 - i2 * p.M2) : 1;
    }
    __syncthreads();
    int yb[DMG_FFT_MAXDIM], zb[DMG_FFT_MAXDIM];
#pragma unroll
    for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
      yb[d] = s_yb[d];
      zb[d] = s_zb[d];
    }
    const int lim1 = s_lim1, lim2 = s_lim2, ytw = s_ytw;
    const int total = n * lim1 * lim2;

    // ---- gather from the input layout ----
    for (int e = tid; e < total; e += NT) {
      int c0, c1, c2;
      tile_coords(e, p.load_pos, n, lim1, lim2, c0, c1, c2);
      int x[DMG_FFT_MAXDIM];
      element_x(p, yb, zb, c0, c1, c2, x);
      C2<T> v = src[layout_addr<T>(p.in, p.ndim, x)];
      if (p.twiddle == 2) {
        const int yv = ytw + (v1_ytd ? c1 : 0) + (v2_ytd ? c2 : 0);
        const int ex = yv * c0;
        if (ex) {
          C2<T> w = twt[ex];
          w.y = -w.y;
          v = mul<T>(v, w);
        }
      }
      bufA[(size_t)(c1 + p.M1 * c2) * ld + c0] = v;
    }
    __syncthreads();

    // ---- Stockham FFT over the lines in shared memory ----
    C2<T> *in = bufA, *out = bufB;
    int Lp = 1;
    for (int f = 0; f < p.nfac; ++f) {
      const int r = p.fac[f];
      const int nr = n / r;
      const int m = nr / Lp;
      const int tstep = n / (Lp * r);  // w_{Lp r}^1 = w_n^tstep
      const int nb = nlines * nr;
      for (int b = tid; b < nb; b += NT) {
        const int l = b / nr;
        const int bb = b - l * nr;
        const int j = bb / m;
        const int k = bb - j * m;
        const C2<T> *xi = in + (size_t)l * ld + j * r * m + k;
        C2<T> *yo = out + (size_t)l * ld + j * m + k;
        const int ostep = Lp * m;
        if (r <= 8) {
          C2<T> a[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            if (q < r) {
              C2<T> v = xi[q * m];
              if (q > 0 && j > 0) v = mul<T>(v, roots[(j * q * tstep) % n]);
              a[q] = v;
            }
          }
          if (r == 8) {
            dft8<T, SIGN>(a);
          } else if (r == 4) {
            dft4<T, SIGN>(a[0], a[1], a[2], a[3]);
          } else if (r == 2) {
            C2<T> t0 = add<T>(a[0], a[1]);
            a[1] = sub<T>(a[0], a[1]);
            a[0] = t0;
          } else if (r == 3) {
            dft3<T, SIGN>(a);
          } else if (r == 5) {
            dft5<T, SIGN>(a);
          } else {  // 7: direct, fully unrolled so that a[] stays in registers
            C2<T> y[8];
#pragma unroll
            for (int s = 0; s < 8; ++s) {
              if (s < r) {
                C2<T> acc = a[0];
#pragma unroll
                for (int q = 1; q < 8; ++q)
                  if (q < r) acc = add<T>(acc, mul<T>(a[q], roots[((q * s) % r) * nr]));
                y[s] = acc;
              }
            }
#pragma unroll
            for (int s = 0; s < 8; ++s)
              if (s < r) a[s] = y[s];
          }
#pragma unroll
          for (int s = 0; s < 8; ++s)
            if (s < r) yo[s * ostep] = a[s];
        } else {
          // direct DFT of a larger prime radix, reading shared memory
          for (int s = 0; s < r; ++s) {
            C2<T> acc = xi[0];
            for (int q = 1; q < r; ++q) {
              C2<T> v = xi[q * m];
              if (j > 0) v = mul<T>(v, roots[(int)(((int64_t)j * q * tstep) % n)]);
              acc = add<T>(acc, mul<T>(v, roots[(int)(((int64_t)q * s % r) * nr)]));
            }
            yo[s * ostep] = acc;
          }
        }
      }
      __syncthreads();
      C2<T> *tmp = in;
      in = out;
      out = tmp;
      Lp *= r;
    }

    // ---- scatter to the output layout ----
    for (int e = tid; e < total; e += NT) {
      int c0, c1, c2;
      tile_coords(e, p.store_pos, n, lim1, lim2, c0, c1, c2);
      C2<T> v = in[(size_t)(c1 + p.M1 * c2) * ld + c0];
      if (p.twiddle == 1) {
        const int yv = ytw + (v1_ytd ? c1 : 0) + (v2_ytd ? c2 : 0);
        const int ex = yv * c0;
        if (ex) v = mul<T>(v, twt[ex]);
      }
      int x[DMG_FFT_MAXDIM];
      element_x(p, yb, zb, c0, c1, c2, x);
      dst[layout_addr<T>(p.out, p.ndim, x)] = v;
    }
  }
}

template <typename T>
size_t pass_smem(const dmg_fft_pass &p) {
  const int ld = (p.n & 1) ? p.n : p.n + 1;
  return sizeof(C2<T>) * ((size_t)2 * p.M1 * p.M2 * ld + p.n);
}

template <typename T, int SIGN>
int launch(const dmg_fft_pass &p, const void *src, void *dst, cudaStream_t s) {
  const size_t smem = pass_smem<T>(p);
  auto k = fft_pass_kernel<T, SIGN>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "fft pass smem %zu: %s", smem, cudaGetErrorString(e));
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, smem);
  if (per_sm < 1) return dmg_error(DMG_ERR_UNSUPPORTED, "fft pass does not fit on an SM (smem %zu)", smem);
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return DMG_OK;
  k<<<(unsigned)grid, NT, smem, s>>>(p, static_cast<const C2<T> *>(src), static_cast<C2<T> *>(dst));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "fft pass launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

}  // namespace

extern "C" size_t dmg_fft_pass_smem(const dmg_fft_pass *p, int dtype) {
  return dtype == 0 ? pass_smem<double>(*p) : pass_smem<float>(*p);
}

extern "C" int dmg_fft_pass_launch(const dmg_fft_pass *p, int dtype, const void *src, void *dst, void *stream) {
  if (p->M1 * p->M2 * p->n > TILE_MAX) return dmg_error(DMG_ERR_ARG, "fft tile %d exceeds %d", p->M1 * p->M2 * p->n, TILE_MAX);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == 0) return p->sign < 0 ? launch<double, -1>(*p, src, dst, s) : launch<double, 1>(*p, src, dst, s);
  return p->sign < 0 ? launch<float, -1>(*p, src, dst, s) : launch<float, 1>(*p, src, dst, s);
}
