// Batched FFT pass with fused layout change and split twiddle.
//
// One launch transforms every line along one sub-axis t of the split
// coordinates (x_d = y_d + A_d*z_d) and writes the result in another layout.
// A block owns tiles of n x M1 x M2 values: it gathers them from the input
// layout in the order that is contiguous there (through the per-dimension
// address tables), runs a Stockham autosort FFT over the n-long lines in
// shared memory (radix 8, 4, 2, 3, 5 butterflies, 7 and larger primes by
// direct DFT), optionally multiplies by the split twiddle of its dimension,
// and scatters the tile to the output layout in the order contiguous there.
// Launches are persistent over the tiles.
//
// Stockham stage with radix r, Lp = product of earlier radices, m = n/(Lp r):
//   a_q = w_{Lp r}^{j q} * x[j r m + q m + k],  y[(j + s Lp) m + k] = sum_q a_q w_r^{q s}
// (j < Lp, k < m); the result is in natural order after the last stage.
//
// Three arithmetics share the code: FP64 (complex128), FP32 (complex64) and
// double-float, where a real is an unevaluated sum hi + lo of two floats
// (48-bit significand) so that complex128 transforms run on the FP32 pipes,
// which GB300 has about 56 times more of than FP64.  Double-float passes keep
// their intermediates as float pairs in HBM; the first pass converts the
// complex128 input after scaling it by 2^-E (E from the input's largest
// exponent, so every value fits FP32's exponent range) and the last pass
// converts back and scales by 2^E.  Error-free transformations used: Knuth's
// two-sum for addition, the FMA product error for multiplication.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "../host/dmg_internal.h"
#include "../host/fft_params.h"

namespace {

constexpr int NT = 128;
constexpr int TILE_MAX = 4096;  // complex values per tile buffer (one 4096-long line at most)

// ---------------------------------------------------------------- double-float reals

struct df {
  float h, l;
};

__device__ __forceinline__ df df_norm(float s, float e) {  // fast two-sum, |s| >= |e|
  const float h = s + e;
  return df{h, e - (h - s)};
}
__device__ __forceinline__ df operator+(df a, df b) {
  const float s = a.h + b.h;
  const float v = s - a.h;
  float e = (a.h - (s - v)) + (b.h - v);
  e += a.l + b.l;
  return df_norm(s, e);
}
__device__ __forceinline__ df operator-(df a) { return df{-a.h, -a.l}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_norm(p, e);
}

// ---------------------------------------------------------------- complex types

struct dfc {
  df x, y;
};
template <typename T>
struct CT;
template <>
struct CT<double> {
  using type = double2;
};
template <>
struct CT<float> {
  using type = float2;
};
template <>
struct CT<df> {
  using type = dfc;
};
template <typename T>
using C2 = typename CT<T>::type;

// a constant in each arithmetic: v for FP64 and FP32, (hi, lo) for double-float
template <typename T>
__device__ __forceinline__ T cst(double v, float hi, float lo);
template <>
__device__ __forceinline__ double cst<double>(double v, float, float) {
  return v;
}
template <>
__device__ __forceinline__ float cst<float>(double v, float, float) {
  return (float)v;
}
template <>
__device__ __forceinline__ df cst<df>(double, float hi, float lo) {
  return df{hi, lo};
}

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
template <typename T>
__device__ __forceinline__ C2<T> conj(C2<T> a) { return mk<T>(a.x, -a.y); }
// multiply by sign*i
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> rot90(C2<T> a) {
  return SIGN < 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}

// mathematical constants and their double-float splits
#define K_SQRT1_2 0.707106781186547524400844362104849039, 0.7071067690849304f, 1.2101617485882343e-08f
#define K_SQRT3_2 0.866025403784438646763723170752936183, 0.8660253882408142f, 1.5543625053737742e-08f
#define K_C72 0.309016994374947424102293417182819059, 0.30901700258255005f, -8.207602597565256e-09f
#define K_C144 -0.809016994374947424102293417182819059, -0.80901700258255f, 8.207602597565256e-09f
#define K_S72 0.951056516295153572116439333379382143, 0.9510565400123596f, -2.3717205976936384e-08f
#define K_S144 0.587785252292473129168705954639072769, 0.5877852439880371f, 8.304436249773062e-09f
#define K_HALF 0.5, 0.5f, 0.0f

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
  const T c = cst<T>(K_SQRT1_2);
  // o1 *= (1 + sign i) c ; o2 *= sign i ; o3 *= (-1 + sign i) c
  C2<T> w1 = SIGN < 0 ? mk<T>(c * (o1.x + o1.y), c * (o1.y - o1.x)) : mk<T>(c * (o1.x - o1.y), c * (o1.y + o1.x));
  C2<T> w2 = rot90<T, SIGN>(o2);
  C2<T> w3 = SIGN < 0 ? mk<T>(c * (o3.y - o3.x), -(c * (o3.x + o3.y))) : mk<T>(-(c * (o3.x + o3.y)), c * (o3.x - o3.y));
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
  const T half = cst<T>(K_HALF);
  C2<T> m = mk<T>(a[0].x - half * s.x, a[0].y - half * s.y);
  C2<T> r = rot90<T, SIGN>(scl<T>(d, cst<T>(K_SQRT3_2)));
  a[0] = add<T>(a[0], s);
  a[1] = add<T>(m, r);
  a[2] = sub<T>(m, r);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft5(C2<T> *a) {
  C2<T> b1 = add<T>(a[1], a[4]), b2 = add<T>(a[2], a[3]);
  C2<T> d1 = sub<T>(a[1], a[4]), d2 = sub<T>(a[2], a[3]);
  const T c1 = cst<T>(K_C72), c2 = cst<T>(K_C144), s1 = cst<T>(K_S72), s2 = cst<T>(K_S144);
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

// ---------------------------------------------------------------- complex128 <-> double-float

// x * 2^-s as a float pair; values pushed below FP64's normal range become 0
__device__ __forceinline__ df to_df(double x, int s) {
  long long b = __double_as_longlong(x);
  const int ef = (int)((b >> 52) & 0x7FF);
  double xs;
  if (ef == 0) {
    // zero or subnormal: scale by two exact power-of-two factors (the result
    // is normal whenever the subnormal matters next to the largest value)
    if ((b & 0x000FFFFFFFFFFFFFll) == 0 || s > 0) return df{0.0f, 0.0f};
    const int s1 = (-s) / 2, s2 = -s - s1;
    xs = x * __longlong_as_double((long long)(1023 + s1) << 52) * __longlong_as_double((long long)(1023 + s2) << 52);
  } else {
    int en = ef - s;
    if (en <= 0) return df{0.0f, 0.0f};
    if (en > 2046) en = 2047;  // stays inf (only when the input held inf or NaN)
    b = (b & ~(0x7FFll << 52)) | ((long long)en << 52);
    xs = __longlong_as_double(b);
  }
  const float h = __double2float_rn(xs);
  const float l = __double2float_rn(xs - (double)h);
  return df{h, l};
}

// (hi + lo) * 2^s as a double
__device__ __forceinline__ double from_df(df v, int s) {
  const double d = (double)v.h + (double)v.l;
  long long b = __double_as_longlong(d);
  const int ef = (int)((b >> 52) & 0x7FF);
  if (ef == 0 || ef == 2047) return d;  // zero (or the inf/NaN of an inf/NaN input)
  const int en = ef + s;
  if (en >= 1 && en <= 2046) return __longlong_as_double((b & ~(0x7FFll << 52)) | ((long long)en << 52));
  // leaves the normal range: two exact power-of-two factors
  const int s1 = s / 2, s2 = s - s1;
  return d * __longlong_as_double((long long)(1023 + s1) << 52) * __longlong_as_double((long long)(1023 + s2) << 52);
}

// ---------------------------------------------------------------- addressing

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

// Walks e = tid, tid + NT, ... through a tile in a given order, keeping the
// (fastest, middle, slowest) coordinates with carries instead of divisions.
struct TileWalk {
  int ef, em, i_f, i_m, i_s, df_, dm, ds;
  __device__ __forceinline__ TileWalk(int tid, const int32_t *pos, int n0, int n1, int n2) {
    ef = pos[0] == 0 ? n0 : pos[1] == 0 ? n1 : n2;
    em = pos[0] == 1 ? n0 : pos[1] == 1 ? n1 : n2;
    i_f = tid % ef;
    const int rest = tid / ef;
    i_m = rest % em;
    i_s = rest / em;
    df_ = NT % ef;
    const int dr = NT / ef;
    dm = dr % em;
    ds = dr / em;
  }
  __device__ __forceinline__ void next() {
    i_f += df_;
    const int c1 = i_f >= ef;
    if (c1) i_f -= ef;
    i_m += dm + c1;
    const int c2 = i_m >= em;
    if (c2) i_m -= em;
    i_s += ds + c2;
  }
  __device__ __forceinline__ int coord(int posk) const { return posk == 0 ? i_f : posk == 1 ? i_m : i_s; }
};

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

// Radix-r butterfly on registers (r <= 8), roots in shared memory.
template <typename T, int SIGN>
__device__ __forceinline__ void butterfly(C2<T> *a, int r, const C2<T> *roots, int nr) {
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
}

// Stockham stages for any n (radices from the pass parameters).
template <typename T, int SIGN>
__device__ __forceinline__ void stockham_runtime(const dmg_fft_pass &p, C2<T> *&in, C2<T> *&out, const C2<T> *roots,
                                                 int nlines, int ld, int tid) {
  const int n = p.n;
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
        butterfly<T, SIGN>(a, r, roots, nr);
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
}

// Radix of the stage after the first LP points of a power-of-two length NF.
__host__ __device__ constexpr int fixed_radix(int nf, int lp) {
  return (nf / lp) % 8 == 0 ? 8 : ((nf / lp) % 4 == 0 ? 4 : 2);
}

// Stockham stages for a power-of-two length known at compile time: index
// arithmetic becomes shifts and masks.
template <typename T, int SIGN, int NF, int LP>
__device__ __forceinline__ void stockham_fixed(C2<T> *&in, C2<T> *&out, const C2<T> *roots, int nlines, int ld,
                                               int tid) {
  if constexpr (LP < NF) {
    constexpr int R = fixed_radix(NF, LP);
    constexpr int NR = NF / R;
    constexpr int M = NR / LP;
    constexpr int TSTEP = NF / (LP * R);
    constexpr int OSTEP = LP * M;
    const int nb = nlines * NR;
    for (int b = tid; b < nb; b += NT) {
      const int l = b / NR;
      const int bb = b % NR;
      const int j = bb / M;
      const int k = bb % M;
      const C2<T> *xi = in + (size_t)l * ld + j * R * M + k;
      C2<T> *yo = out + (size_t)l * ld + j * M + k;
      C2<T> a[8];
#pragma unroll
      for (int q = 0; q < R; ++q) {
        C2<T> v = xi[q * M];
        if (LP > 1 && q > 0) v = mul<T>(v, roots[(j * q * TSTEP) & (NF - 1)]);
        a[q] = v;
      }
      butterfly<T, SIGN>(a, R, roots, NR);
#pragma unroll
      for (int s = 0; s < R; ++s) yo[s * OSTEP] = a[s];
    }
    __syncthreads();
    C2<T> *tmp = in;
    in = out;
    out = tmp;
    stockham_fixed<T, SIGN, NF, LP * R>(in, out, roots, nlines, ld, tid);
  }
}

template <typename T, bool FP64>
__device__ __forceinline__ C2<T> load_elem(const void *src, int64_t a, int s) {
  if constexpr (FP64) {
    const double2 d = reinterpret_cast<const double2 *>(src)[a];
    dfc r;
    r.x = to_df(d.x, s);
    r.y = to_df(d.y, s);
    return r;
  } else {
    (void)s;
    return reinterpret_cast<const C2<T> *>(src)[a];
  }
}

template <typename T, bool FP64>
__device__ __forceinline__ void store_elem(void *dst, int64_t a, C2<T> v, int s) {
  if constexpr (FP64) {
    double2 d;
    d.x = from_df(v.x, s);
    d.y = from_df(v.y, s);
    reinterpret_cast<double2 *>(dst)[a] = d;
  } else {
    (void)s;
    reinterpret_cast<C2<T> *>(dst)[a] = v;
  }
}

// INF / OUTF: the input / output is complex128 converted to and from
// double-float (double-float arithmetic only)
template <typename T, int SIGN, bool INF, bool OUTF, int NF>
__global__ void __launch_bounds__(NT) fft_pass_kernel(const dmg_fft_pass p, const void *__restrict__ src,
                                                      void *__restrict__ dst) {
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
    for (int i = tid; i < n; i += NT) roots[i] = SIGN > 0 ? conj<T>(gr[i]) : gr[i];
  }
  __shared__ int s_yb[DMG_FFT_MAXDIM], s_zb[DMG_FFT_MAXDIM];
  __shared__ int s_lim1, s_lim2, s_ytw;
  // scale exponent of the double-float conversions (bias removed, inputs end below 2)
  int sexp = 0;
  if constexpr (INF || OUTF) sexp = __ldg(p.scale_exp) - 1022;
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
    TileWalk wl(tid, p.load_pos, n, lim1, lim2);
    for (int e = tid; e < total; e += NT, wl.next()) {
      const int c0 = wl.coord(p.load_pos[0]), c1 = wl.coord(p.load_pos[1]), c2 = wl.coord(p.load_pos[2]);
      int x[DMG_FFT_MAXDIM];
      element_x(p, yb, zb, c0, c1, c2, x);
      C2<T> v = load_elem<T, INF>(src, layout_addr(p.in, p.ndim, x), sexp);
      if (p.twiddle == 2) {
        const int yv = ytw + (v1_ytd ? c1 : 0) + (v2_ytd ? c2 : 0);
        const int ex = yv * c0;
        if (ex) v = mul<T>(v, conj<T>(twt[ex]));
      }
      bufA[(size_t)(c1 + p.M1 * c2) * ld + c0] = v;
    }
    __syncthreads();

    // ---- Stockham FFT over the lines in shared memory ----
    C2<T> *in = bufA, *out = bufB;
    if constexpr (NF > 0) {
      stockham_fixed<T, SIGN, NF, 1>(in, out, roots, nlines, ld, tid);
    } else {
      stockham_runtime<T, SIGN>(p, in, out, roots, nlines, ld, tid);
    }

    // ---- scatter to the output layout ----
    TileWalk ws(tid, p.store_pos, n, lim1, lim2);
    for (int e = tid; e < total; e += NT, ws.next()) {
      const int c0 = ws.coord(p.store_pos[0]), c1 = ws.coord(p.store_pos[1]), c2 = ws.coord(p.store_pos[2]);
      C2<T> v = in[(size_t)(c1 + p.M1 * c2) * ld + c0];
      if (p.twiddle == 1) {
        const int yv = ytw + (v1_ytd ? c1 : 0) + (v2_ytd ? c2 : 0);
        const int ex = yv * c0;
        if (ex) v = mul<T>(v, twt[ex]);
      }
      int x[DMG_FFT_MAXDIM];
      element_x(p, yb, zb, c0, c1, c2, x);
      store_elem<T, OUTF>(dst, layout_addr(p.out, p.ndim, x), v, sexp);
    }
  }
}

// Largest biased exponent of max(|re|, |im|) over every element of a layout.
// Coordinates enumerate the global array in C order; dimensions beyond ndim
// have length 1.
__global__ void __launch_bounds__(256) maxexp_kernel(const dmg_fft_layout lay, int ndim, int L0, int L1, int L2,
                                                     const double2 *__restrict__ src, int32_t *out) {
  const int64_t N = (int64_t)L0 * L1 * L2;
  int best = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    int x[DMG_FFT_MAXDIM];
    int64_t r = i;
    x[2] = (int)(r % L2);
    r /= L2;
    x[1] = (int)(r % L1);
    x[0] = (int)(r / L1);
    const double2 v = src[layout_addr(lay, ndim, x)];
    const int ea = (int)((__double_as_longlong(v.x) >> 52) & 0x7FF);
    const int eb = (int)((__double_as_longlong(v.y) >> 52) & 0x7FF);
    best = max(best, max(ea, eb));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(out, best);
}

template <typename T>
size_t pass_smem(const dmg_fft_pass &p) {
  const int ld = (p.n & 1) ? p.n : p.n + 1;
  return sizeof(C2<T>) * ((size_t)2 * p.M1 * p.M2 * ld + p.n);
}

template <typename T, int SIGN, bool INF, bool OUTF, int NF>
int launch_n(const dmg_fft_pass &p, const void *src, void *dst, cudaStream_t s) {
  const size_t smem = pass_smem<T>(p);
  auto k = fft_pass_kernel<T, SIGN, INF, OUTF, NF>;
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
  k<<<(unsigned)grid, NT, smem, s>>>(p, src, dst);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "fft pass launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

// lines of 16 and 32 points (the split factors of 256, 512 and 1024) get
// specialised kernels; every other length runs the general one
template <typename T, int SIGN, bool INF, bool OUTF>
int launch(const dmg_fft_pass &p, const void *src, void *dst, cudaStream_t s) {
  if (p.n == 32) return launch_n<T, SIGN, INF, OUTF, 32>(p, src, dst, s);
  if (p.n == 16) return launch_n<T, SIGN, INF, OUTF, 16>(p, src, dst, s);
  return launch_n<T, SIGN, INF, OUTF, 0>(p, src, dst, s);
}

template <typename T, int SIGN>
int launch_fmt(const dmg_fft_pass &p, const void *src, void *dst, cudaStream_t s) {
  if constexpr (std::is_same<T, df>::value) {
    if (p.in_fp64 && p.out_fp64) return launch<T, SIGN, true, true>(p, src, dst, s);
    if (p.in_fp64) return launch<T, SIGN, true, false>(p, src, dst, s);
    if (p.out_fp64) return launch<T, SIGN, false, true>(p, src, dst, s);
  }
  return launch<T, SIGN, false, false>(p, src, dst, s);
}

}  // namespace

extern "C" size_t dmg_fft_pass_smem(const dmg_fft_pass *p, int dtype) {
  return dtype == 1 ? pass_smem<float>(*p) : pass_smem<double>(*p);
}

extern "C" int dmg_fft_pass_launch(const dmg_fft_pass *p, int dtype, const void *src, void *dst, void *stream) {
  if (p->M1 * p->M2 * p->n > TILE_MAX) return dmg_error(DMG_ERR_ARG, "fft tile %d exceeds %d", p->M1 * p->M2 * p->n, TILE_MAX);
  if (dtype == 2 && (p->in_fp64 || p->out_fp64) && !p->scale_exp)
    return dmg_error(DMG_ERR_ARG, "double-float pass without a scale exponent");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (dtype) {
    case 0: return p->sign < 0 ? launch_fmt<double, -1>(*p, src, dst, s) : launch_fmt<double, 1>(*p, src, dst, s);
    case 1: return p->sign < 0 ? launch_fmt<float, -1>(*p, src, dst, s) : launch_fmt<float, 1>(*p, src, dst, s);
    case 2: return p->sign < 0 ? launch_fmt<df, -1>(*p, src, dst, s) : launch_fmt<df, 1>(*p, src, dst, s);
    default: return dmg_error(DMG_ERR_ARG, "fft dtype %d", dtype);
  }
}

extern "C" int dmg_fft_maxexp_launch(const dmg_fft_layout *lay, int ndim, const int32_t *A, const int32_t *L,
                                     const void *src, int32_t *out, void *stream) {
  (void)A;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "maxexp memset: %s", cudaGetErrorString(e));
  const int L0 = L[0], L1 = ndim > 1 ? L[1] : 1, L2 = ndim > 2 ? L[2] : 1;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  maxexp_kernel<<<nsm * 8, 256, 0, s>>>(*lay, ndim, L0, L1, L2, static_cast<const double2 *>(src), out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "maxexp launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}
