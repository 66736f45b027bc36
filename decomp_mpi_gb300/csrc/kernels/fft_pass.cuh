// Batched FFT pass with fused layout change (shared by the translation units
// fft_pass_{f64,f32,df}{,_inv}{,_mixed}.cu: one per arithmetic, direction and
// group of lengths).
//
// One launch transforms every line along one axis and writes the result in
// another layout: one pass does the work of a reshape (runReshapePlan), a
// batch of FFTW transforms and the twiddle (decomp_scale) of the reference's
// runSplitPlan (split_fft.c:622-744).  A block owns tiles of n x M1 x M2 values, persistent over
// the tiles, in a three-buffer pipeline: the gather copies tile i+1 from the
// input layout into a staging buffer with asynchronous copies (cp.async, in
// the order contiguous in the input) while tile i goes through its Stockham
// stages between two other buffers; the scatter stores the result to the
// output layout in the order contiguous there, optionally multiplied by a
// split twiddle, and in the split FFT's slot order for whole-dimension
// passes.  A block steps through its tiles by adding the digits of the grid
// size to the tile index's mixed-radix digits, and the next tile's address
// parts load asynchronously behind the current tile's first stage.  The
// pass body takes its block index and block count as arguments, so that a
// grouped launch can give each of several passes (of different plans and
// lengths) a range of its blocks.
//
// Stockham stage with radix r, Lp = product of earlier radices, m = n/(Lp r):
//   a_q = w_{Lp r}^{j q} * x[j r m + q m + k],  y[(j + s Lp) m + k] = sum_q a_q w_r^{q s}
// (j < Lp, k < m); the result is in natural order after the last stage.
// Lengths known at compile time (powers of two 8...2048, the 2,3,5-smooth
// cube sides 48...480) have fixed radix schedules.  The power-of-two ones
// keep the tile between stages in per-hop XOR-swizzled layouts (one XOR per
// access, bank-conflict free) and read twiddles from per-stage tables staged
// in shared memory; the others swizzle line positions (i ^ ((i / V) mod V),
// V values per 128 bytes) and read the pass's root table.  Other lengths
// take radices 8, 4, 2, 3, 5, 7 and direct DFTs of larger primes from the
// pass.  The staging buffer and the buffer the scatter reads are
// line-padded (odd pitch) with swizzled line positions.
//
// Addresses: a side whose address is separable over the tile axes keeps,
// per tile, the part of the two vector axes in shared memory and reads the
// transform axis's part from its table; the usual axis orders walk with the
// axes' roles fixed at compile time.  Ranked layouts are evaluated per
// value.  Values every phase needs live in shared memory and are re-read
// after barriers, so none holds a register through the stages.
//
// Three arithmetics share the code: FP64 (complex128), FP32 (complex64) and
// double-float, where a real is an unevaluated sum hi + lo of two floats
// (48-bit significand) so that complex128 transforms run on the FP32 pipes,
// which GB300 has about 56 times more of than FP64.  Double-float passes keep
// their intermediates as float pairs in HBM; the first pass converts the
// complex128 input after scaling it by 2^-E (E from the input's largest
// exponent, so every value fits FP32's exponent range) and the last pass
// converts back and scales by 2^E, both with integer operations.
// Error-free transformations used: Knuth's two-sum for addition, the FMA
// product error for multiplication.  FP32 and double-float complex values
// keep (re, im) in one float pair, so that their arithmetic runs as
// Blackwell's paired FP32 instructions (one instruction per pair).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "../host/dmg_internal.h"
#include "../host/fft_params.h"
#include "tc_sm100.cuh"

namespace {

constexpr int NT = DMG_FFT_NT;
constexpr int TILE_MAX = DMG_FFT_TILE_MAX;

// ---------------------------------------------------------------- paired FP32 operations

// Blackwell's two-wide FP32 instructions (FADD2, FMUL2, FFMA2): each runs
// one operation on both floats of a pair, rounding each as its scalar form.
// Complex values keep (re, im) in one pair so that every complex operation
// is a sequence of paired instructions.
__device__ __forceinline__ float2 p2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 splat(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as an FMA with -1 (exact product, one rounding: the same as a subtraction)
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, splat(-1.0f), a); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

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

// A double-float complex number: the leading parts (re, im) in one pair and
// the trailing parts in another, so that the two-sum and product-error steps
// of the real and imaginary parts run as paired instructions.  Stored in
// shared memory and HBM in the same order (re.hi, im.hi, re.lo, im.lo),
// 16-byte aligned so that a value moves with one 16-byte access.
struct __align__(16) dfc {
  float2 h, l;
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

// a real constant in each arithmetic: v for FP64 and FP32, (hi, lo) for double-float
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

// --- FP64: scalar ---
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cscl(double2 a, double c) { return make_double2(a.x * c, a.y * c); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
template <int SIGN>
__device__ __forceinline__ double2 crot(double2 a) {  // multiply by sign * i
  return SIGN < 0 ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

// --- FP32: paired ---
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return padd(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return psub(a, b); }
// a * b = a.x * (b.x, b.y) + a.y * (-b.y, b.x)
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return pfma(splat(a.y), p2(-b.y, b.x), pmul(splat(a.x), b));
}
__device__ __forceinline__ float2 cscl(float2 a, float c) { return pmul(a, splat(c)); }
__device__ __forceinline__ float2 cconj(float2 a) { return p2(a.x, -a.y); }
template <int SIGN>
__device__ __forceinline__ float2 crot(float2 a) {
  return SIGN < 0 ? p2(a.y, -a.x) : p2(-a.y, a.x);
}

// --- double-float: paired two-sum / FMA product error ---
__device__ __forceinline__ dfc dnorm(float2 s, float2 e) {  // fast two-sum of both lanes, |s| >= |e|
  const float2 h = padd(s, e);
  return dfc{h, psub(e, psub(h, s))};
}
// sum with the result left unnormalised (two-sum of the leading parts plus
// the trailing parts); for results that only feed further additions
__device__ __forceinline__ dfc cadd_lazy(dfc a, dfc b) {
  const float2 s = padd(a.h, b.h);
  const float2 v = psub(s, a.h);
  float2 e = padd(psub(a.h, psub(s, v)), psub(b.h, v));
  e = padd(e, padd(a.l, b.l));
  return dfc{s, e};
}
__device__ __forceinline__ dfc cadd(dfc a, dfc b) {
  const dfc r = cadd_lazy(a, b);
  return dnorm(r.h, r.l);
}
// difference: the two-sum of a and -b
__device__ __forceinline__ dfc csub_lazy(dfc a, dfc b) {
  const float2 s = psub(a.h, b.h);
  const float2 v = psub(s, a.h);
  const float2 e = psub(psub(a.h, psub(s, v)), padd(b.h, v));
  return dfc{s, padd(e, psub(a.l, b.l))};
}
__device__ __forceinline__ dfc csub(dfc a, dfc b) {
  const dfc r = csub_lazy(a, b);
  return dnorm(r.h, r.l);
}
// a * b = a.re * b + a.im * (i b): the leading products and their exact
// errors (FMA), the exact sum of the leading products (two-sum), the cross
// terms; the lo*lo terms (2^-48 of the result) are dropped
__device__ __forceinline__ dfc cmul(dfc a, dfc b) {
  const float2 bh_i = p2(-b.h.y, b.h.x), bl_i = p2(-b.l.y, b.l.x);
  const float2 xh = splat(a.h.x), yh = splat(a.h.y), xl = splat(a.l.x), yl = splat(a.l.y);
  const float2 q1 = pmul(xh, b.h);
  const float2 q2 = pmul(yh, bh_i);
  const float2 e1 = pfma(xh, b.h, p2(-q1.x, -q1.y));
  const float2 e2 = pfma(yh, bh_i, p2(-q2.x, -q2.y));
  const float2 s = padd(q1, q2);
  const float2 v = psub(s, q1);
  float2 t = padd(psub(q1, psub(s, v)), psub(q2, v));
  t = padd(t, padd(e1, e2));
  t = pfma(xh, b.l, t);
  t = pfma(xl, b.h, t);
  t = pfma(yh, bl_i, t);
  t = pfma(yl, bh_i, t);
  return dnorm(s, t);
}
// a * c for a real double-float constant c
__device__ __forceinline__ dfc cscl(dfc a, df c) {
  const float2 ch = splat(c.h);
  const float2 p = pmul(a.h, ch);
  float2 e = pfma(a.h, ch, p2(-p.x, -p.y));
  e = pfma(a.h, splat(c.l), e);
  e = pfma(a.l, ch, e);
  return dnorm(p, e);
}
__device__ __forceinline__ dfc cconj(dfc a) { return dfc{p2(a.h.x, -a.h.y), p2(a.l.x, -a.l.y)}; }
template <int SIGN>
__device__ __forceinline__ dfc crot(dfc a) {
  return SIGN < 0 ? dfc{p2(a.h.y, -a.h.x), p2(a.l.y, -a.l.x)} : dfc{p2(-a.h.y, a.h.x), p2(-a.l.y, a.l.x)};
}

// The generic names the stages use.
template <typename T>
__device__ __forceinline__ C2<T> add(C2<T> a, C2<T> b) { return cadd(a, b); }
template <typename T>
__device__ __forceinline__ C2<T> sub(C2<T> a, C2<T> b) { return csub(a, b); }
template <typename T>
__device__ __forceinline__ C2<T> mul(C2<T> a, C2<T> b) { return cmul(a, b); }
template <typename T>
__device__ __forceinline__ C2<T> scl(C2<T> a, T c) { return cscl(a, c); }
template <typename T>
__device__ __forceinline__ C2<T> conj(C2<T> a) { return cconj(a); }
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> rot90(C2<T> a) { return crot<SIGN>(a); }
// unnormalised sum / difference for double-float (FP64 and FP32 exact forms unaffected)
template <typename T>
__device__ __forceinline__ C2<T> addl(C2<T> a, C2<T> b) {
  if constexpr (std::is_same<T, df>::value) {
    return cadd_lazy(a, b);
  } else {
    return cadd(a, b);
  }
}
template <typename T>
__device__ __forceinline__ C2<T> subl(C2<T> a, C2<T> b) {
  if constexpr (std::is_same<T, df>::value) {
    return csub_lazy(a, b);
  } else {
    return csub(a, b);
  }
}

// mathematical constants and their double-float splits
#define K_SQRT1_2 0.707106781186547524400844362104849039, 0.7071067690849304f, 1.2101617485882343e-08f
#define K_SQRT3_2 0.866025403784438646763723170752936183, 0.8660253882408142f, 1.5543625053737742e-08f
#define K_C72 0.309016994374947424102293417182819059, 0.30901700258255005f, -8.207602597565256e-09f
#define K_C144 -0.809016994374947424102293417182819059, -0.80901700258255f, 8.207602597565256e-09f
#define K_S72 0.951056516295153572116439333379382143, 0.9510565400123596f, -2.3717205976936384e-08f
#define K_S144 0.587785252292473129168705954639072769, 0.5877852439880371f, 8.304436249773062e-09f
#define K_HALF 0.5, 0.5f, 0.0f

// Butterflies written with complex operations only (so that each maps to
// paired instructions).
// LAZY: outputs left unnormalised (double-float), for callers that only add
// them or scale them further
template <typename T, int SIGN, bool LAZY = false>
__device__ __forceinline__ void dft4(C2<T> &a0, C2<T> &a1, C2<T> &a2, C2<T> &a3) {
  C2<T> t0 = addl<T>(a0, a2), t1 = subl<T>(a0, a2), t2 = addl<T>(a1, a3), t3 = rot90<T, SIGN>(subl<T>(a1, a3));
  if constexpr (LAZY) {
    a0 = addl<T>(t0, t2);
    a2 = subl<T>(t0, t2);
    a1 = addl<T>(t1, t3);
    a3 = subl<T>(t1, t3);
  } else {
    a0 = add<T>(t0, t2);
    a2 = sub<T>(t0, t2);
    a1 = add<T>(t1, t3);
    a3 = sub<T>(t1, t3);
  }
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft8(C2<T> *a) {
  C2<T> e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  C2<T> o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  // the inner sums stay unnormalised (double-float): only the outputs are normalised
  dft4<T, SIGN, true>(e0, e1, e2, e3);
  dft4<T, SIGN, true>(o0, o1, o2, o3);
  const T c = cst<T>(K_SQRT1_2);
  // o1 *= (1 + sign i) c ; o2 *= sign i ; o3 *= (-1 + sign i) c
  const C2<T> w1 = scl<T>(addl<T>(o1, rot90<T, SIGN>(o1)), c);
  const C2<T> w2 = rot90<T, SIGN>(o2);
  const C2<T> w3 = scl<T>(subl<T>(rot90<T, SIGN>(o3), o3), c);
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
  const C2<T> s = add<T>(a[1], a[2]);
  const C2<T> d = sub<T>(a[1], a[2]);
  const C2<T> m = sub<T>(a[0], scl<T>(s, cst<T>(K_HALF)));
  const C2<T> r = rot90<T, SIGN>(scl<T>(d, cst<T>(K_SQRT3_2)));
  a[0] = add<T>(a[0], s);
  a[1] = add<T>(m, r);
  a[2] = sub<T>(m, r);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft5(C2<T> *a) {
  const C2<T> b1 = add<T>(a[1], a[4]), b2 = add<T>(a[2], a[3]);
  const C2<T> d1 = sub<T>(a[1], a[4]), d2 = sub<T>(a[2], a[3]);
  const T c1 = cst<T>(K_C72), c2 = cst<T>(K_C144), s1 = cst<T>(K_S72), s2 = cst<T>(K_S144);
  const C2<T> p1 = add<T>(a[0], add<T>(scl<T>(b1, c1), scl<T>(b2, c2)));
  const C2<T> p2_ = add<T>(a[0], add<T>(scl<T>(b1, c2), scl<T>(b2, c1)));
  const C2<T> q1 = rot90<T, SIGN>(add<T>(scl<T>(d1, s1), scl<T>(d2, s2)));
  const C2<T> q2 = rot90<T, SIGN>(sub<T>(scl<T>(d1, s2), scl<T>(d2, s1)));
  a[0] = add<T>(a[0], add<T>(b1, b2));
  a[1] = add<T>(p1, q1);
  a[4] = sub<T>(p1, q1);
  a[2] = add<T>(p2_, q2);
  a[3] = sub<T>(p2_, q2);
}

// ---------------------------------------------------------------- complex128 <-> double-float

// x * 2^-s as a float pair with FP64 arithmetic (any x); values pushed below
// FP64's normal range become 0
__device__ __noinline__ df to_df_slow(double x, int s) {
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

// (hi + lo) * 2^s as a double with FP64 arithmetic (any pair)
__device__ __noinline__ double from_df_slow(df v, int s) {
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

// The same conversions with integer operations only (GB300 runs FP64 and
// FP32<->FP64 conversions at 1/64 of its FP32 rate).  A normal double's
// 53-bit significand m splits exactly into its 24-bit rounding mh (the
// float hi) and the remainder r = m - mh * 2^29 (|r| <= 2^28, converted to
// the float lo); back, lo rounded to the places of hi's double is added to
// that double's bit pattern.  Values whose pair would leave FP32's
// normal range, zeros, subnormals, infinities and NaNs take the FP64 path.
__device__ __forceinline__ df to_df(double x, int s) {
  // in 32-bit halves: hi's 23 stored significand bits are the double's top
  // 23, rounded by the next bit (added to hi's bit pattern, so that a carry
  // moves into the exponent); the remaining 29 bits, less 2^29 when hi
  // rounded up, are lo in units of 2^(fe - 179)
  const unsigned hb = (unsigned)__double2hiint(x), lb = (unsigned)__double2loint(x);
  const int E = (int)((hb >> 20) & 0x7FF);
  const int fe = E - s - 896;  // float biased exponent of hi before rounding
  if (E == 0 || E == 0x7FF || fe < 53 || fe > 253) return to_df_slow(x, s);
  const unsigned top = ((hb & 0xFFFFFu) << 3) | (lb >> 29);
  const unsigned rb = (lb >> 28) & 1u;
  const int r = (int)(lb & 0x1FFFFFFFu) - (int)(rb << 29);
  const unsigned sign = hb & 0x80000000u;
  const float h = __uint_as_float((sign | ((unsigned)fe << 23) | top) + rb);
  // fe >= 53 keeps the power of two normal
  const float l = (float)r * __uint_as_float(((unsigned)(fe - 52) << 23) | sign);
  return df{h, l};
}

__device__ __forceinline__ double from_df(df v, int s) {
  // the double of hi (exponent rebiased, scaled by 2^s) plus lo counted in
  // that double's last places: an integer r added to its bit pattern, which
  // carries into the exponent by itself; just below a power of two (hi's
  // significand all zeros, r < 0) the places are half as large, so 2r
  const unsigned hb = __float_as_uint(v.h);
  const int fe = (int)((hb >> 23) & 0xFF);
  const int E = fe + 896 + s;
  const float ls = v.l * __uint_as_float(((unsigned)(306 - fe) << 23) | (hb & 0x80000000u));
  if (fe < 52 || fe == 0xFF || E < 2 || E > 2046 || !(fabsf(ls) < 1073741824.0f)) return from_df_slow(v, s);
  const int r = __float2int_rn(ls);
  const unsigned mant = hb & 0x7FFFFFu;
  const long long hi = (long long)(((unsigned long long)(hb >> 31) << 63) | ((unsigned long long)E << 52) |
                                   ((unsigned long long)mant << 29));
  return __longlong_as_double(hi + ((mant == 0 && r < 0) ? 2ll * r : (long long)r));
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

// a root of the pass's table, conjugated for the inverse
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> root_at(const C2<T> *roots, int i) {
  C2<T> w;
  if constexpr (std::is_same<T, df>::value) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(roots) + i);
    w.h = make_float2(v.x, v.y);
    w.l = make_float2(v.z, v.w);
  } else {
    w = __ldg(roots + i);
  }
  return SIGN > 0 ? conj<T>(w) : w;
}

// FP64 radix-8 stage with its input twiddles w^q (w = w_{8 LP}^j), as three
// layers of radix-2 butterflies y0 = a + t b, y1 = 2 a - y0 whose twiddle t
// is a single complex number: six FMAs per butterfly, 72 per eight values
// against 80 for seven twiddle products and the 8-point DFT.  With
// A_q = x_q + w^4 x_{q+4} (B: minus), the even outputs are the 4-point DFT of
// w^q A_q and the odd ones that of (w W8)^q B_q; the same split again leaves
// twiddles w^2 and w^2 W4 for the second layer and w, w W4, w W8, w W8 W4 for
// the third (W8 = w_8 in the transform's direction, W4 = W8^2: multiplying by
// it is a swap and a sign).  v = w W8 comes from the pass's root table.
template <int SIGN>
__device__ __forceinline__ void bfly_tw(double2 &a, double2 &b, double tx, double ty) {
  const double y0x = __fma_rn(tx, b.x, __fma_rn(-ty, b.y, a.x));
  const double y0y = __fma_rn(tx, b.y, __fma_rn(ty, b.x, a.y));
  b.x = __fma_rn(2.0, a.x, -y0x);
  b.y = __fma_rn(2.0, a.y, -y0y);
  a.x = y0x;
  a.y = y0y;
}
// the same with twiddle t W4
template <int SIGN>
__device__ __forceinline__ void bfly_tw_rot(double2 &a, double2 &b, double tx, double ty) {
  if (SIGN < 0) {
    bfly_tw<SIGN>(a, b, ty, -tx);  // t (-i)
  } else {
    bfly_tw<SIGN>(a, b, -ty, tx);  // t i
  }
}
template <int SIGN>
__device__ __forceinline__ void dft8_tw_fma(double2 *a, double2 w1, double2 w2, double2 w4, double2 v) {
#pragma unroll
  for (int q = 0; q < 4; ++q) bfly_tw<SIGN>(a[q], a[q + 4], w4.x, w4.y);
  bfly_tw<SIGN>(a[0], a[2], w2.x, w2.y);
  bfly_tw<SIGN>(a[1], a[3], w2.x, w2.y);
  bfly_tw_rot<SIGN>(a[4], a[6], w2.x, w2.y);
  bfly_tw_rot<SIGN>(a[5], a[7], w2.x, w2.y);
  bfly_tw<SIGN>(a[0], a[1], w1.x, w1.y);
  bfly_tw_rot<SIGN>(a[2], a[3], w1.x, w1.y);
  bfly_tw<SIGN>(a[4], a[5], v.x, v.y);
  bfly_tw_rot<SIGN>(a[6], a[7], v.x, v.y);
  // outputs in bit-reversed places: y0 y4 y2 y6 y1 y5 y3 y7
  const double2 y1 = a[4], y2 = a[2], y3 = a[6], y4 = a[1], y6 = a[3];
  a[1] = y1;
  a[2] = y2;
  a[3] = y3;
  a[4] = y4;
  a[6] = y6;
}

// The radix-4 stage the same way: A_q = x_q + w^2 x_{q+2} (B: minus), then
// y0, y2 = A_0 +- w A_1 and y1, y3 = B_0 +- w W4 B_1 (24 FMAs against 28).
template <int SIGN>
__device__ __forceinline__ void dft4_tw_fma(double2 *a, double2 w1, double2 w2) {
  bfly_tw<SIGN>(a[0], a[2], w2.x, w2.y);
  bfly_tw<SIGN>(a[1], a[3], w2.x, w2.y);
  bfly_tw<SIGN>(a[0], a[1], w1.x, w1.y);
  bfly_tw_rot<SIGN>(a[2], a[3], w1.x, w1.y);
  const double2 y1 = a[2];  // y0 y2 y1 y3 in place
  a[2] = a[1];
  a[1] = y1;
}

// Radix-r butterfly on registers (r <= 8), roots from the pass's table.
template <typename T, int SIGN>
__device__ __forceinline__ void butterfly(C2<T> *a, int r, const C2<T> *roots, int nr) {
  // (roots: the pass's global table of exp(-2 pi i k / n), conjugated here for the inverse)
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
          if (q < r) acc = add<T>(acc, mul<T>(a[q], root_at<T, SIGN>(roots, ((q * s) % r) * nr)));
        y[s] = acc;
      }
    }
#pragma unroll
    for (int s = 0; s < 8; ++s)
      if (s < r) a[s] = y[s];
  }
}

// Radix-R butterfly for R = 2, 3, 4, 5, 8 known at compile time.
template <typename T, int SIGN, int R>
__device__ __forceinline__ void bfly_fixed(C2<T> *a) {
  if constexpr (R == 8) {
    dft8<T, SIGN>(a);
  } else if constexpr (R == 4) {
    dft4<T, SIGN>(a[0], a[1], a[2], a[3]);
  } else if constexpr (R == 3) {
    dft3<T, SIGN>(a);
  } else if constexpr (R == 5) {
    dft5<T, SIGN>(a);
  } else {
    static_assert(R == 2, "radix 2, 3, 4, 5 or 8");
    C2<T> t0 = add<T>(a[0], a[1]);
    a[1] = sub<T>(a[0], a[1]);
    a[0] = t0;
  }
}

// One Stockham stage of radix r = p.fac[f] after the first Lp points, for
// any n (radices from the pass), from `in` to `out`.
template <typename T, int SIGN>
__device__ __forceinline__ void stage_runtime(const dmg_fft_pass &p, int f, int Lp, const C2<T> *in, C2<T> *out,
                                              const C2<T> *roots, int nlines, int ld, int tid) {
  const int n = p.n;
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
          if (q > 0 && j > 0) v = mul<T>(v, root_at<T, SIGN>(roots, (j * q * tstep) % n));
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
          if (j > 0) v = mul<T>(v, root_at<T, SIGN>(roots, (int)(((int64_t)j * q * tstep) % n)));
          acc = add<T>(acc, mul<T>(v, root_at<T, SIGN>(roots, (int)(((int64_t)q * s % r) * nr))));
        }
        yo[s * ostep] = acc;
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- stages of a length known at compile time

// log2 of the values per 128 bytes: the swizzle period
template <typename T>
__host__ __device__ constexpr int swz_shift() {
  return sizeof(C2<T>) == 8 ? 4 : 3;
}
// position of value i of an NF-point line: the low bits of i XOR the next
// ones, when NF is a multiple of the period (else i); NF = 0: i
template <typename T, int NF>
__device__ __forceinline__ int swz(int i) {
  constexpr int S = swz_shift<T>();
  if constexpr (NF > 0 && NF % (1 << S) == 0) {
    return i ^ ((i >> S) & ((1 << S) - 1));
  } else {
    return i;
  }
}

// Roots of the compile-time-length stages: staged in shared memory when
// DMG_FFT_SMEM_ROOTS is set (the kernel copies the pass's table at start;
// shared loads wait less than L1 loads), else read through L1 from the
// global table.
#ifndef DMG_FFT_SMEM_ROOTS
#define DMG_FFT_SMEM_ROOTS 1
#endif
template <typename T, int SIGN>
__device__ __forceinline__ C2<T> root_fx(const C2<T> *roots, int i) {
  if constexpr (DMG_FFT_SMEM_ROOTS) {
    const C2<T> w = roots[i];
    return SIGN > 0 ? conj<T>(w) : w;
  } else {
    return root_at<T, SIGN>(roots, i);
  }
}

// radix of the stage after the first LP points of NF (2, 3, 5-smooth): 8s
// while the power-of-two part allows (16 done as 4 x 4), then 4, 2, 3, 5
__host__ __device__ constexpr int fixed_radix(int nf, int lp) {
  const int rem = nf / lp;
  const int p2 = rem & -rem;
  if (p2 >= 8) return p2 == 16 ? 4 : 8;
  if (p2 == 4) return 4;
  if (p2 == 2) return 2;
  if (rem % 3 == 0) return 3;
  if (rem % 5 == 0) return 5;
  return rem;
}

// ---- power-of-two lengths: stage buffers addressed by XOR constants ----
//
// Between two stages of a power-of-two length the tile is kept in a layout
// of its own: value x = line * NF + i (the line-major tile index) sits at
// g(x) = x ^ ((x >> A1) & (V - 1)) [^ ((x >> A2) & (V - 1))], V values per
// 128 bytes, with A1 = log2 of the consuming stage's radix.  g is linear over
// GF(2) and the stage's index splits into disjoint bit fields (a thread's
// butterfly base, the radix digit q * M, the output digit s * NR), so every
// position is g(base) ^ g(digit) with g(digit) a compile-time constant: one
// XOR per value instead of the index arithmetic.  The bank model this was
// chosen with (16 lanes x 8 bytes or 8 lanes x 16 bytes per shared-memory
// wavefront) gives one wavefront per access for every stage of the
// lengths 16 ... 2048; length 32 needs its own terms.  The staging buffer the
// gather fills and the buffer the scatter reads keep the line-padded layout.
__host__ __device__ constexpr bool pow2_length(int n) { return n >= 8 && n <= 2048 && (n & (n - 1)) == 0; }
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
// bytes per stage buffer of a power-of-two length kernel: the largest tile
// of the pass in the line-padded layout (one line where a line is longer
// than the tile target)
__host__ __device__ constexpr size_t pow2_stride(size_t es, int n) {
  return ((size_t)(DMG_FFT_TILE_TARGET(es) / n > 0 ? DMG_FFT_TILE_TARGET(es) / n : 1) * (size_t)(n | 1) * es + 15) &
         ~(size_t)15;
}
// the most lines side by side a power-of-two length kernel's buffers hold
__host__ __device__ constexpr int pow2_lines(size_t es, int n) {
  return DMG_FFT_TILE_TARGET(es) / n > 0 ? DMG_FFT_TILE_TARGET(es) / n : 1;
}
template <typename T, int NF, int LPC>  // LPC: the consuming stage's LP
struct HopSwz {
  static constexpr int S = swz_shift<T>();
  static constexpr int A1 = NF == 32 ? (S == 3 ? 3 : 1) : ilog2(fixed_radix(NF, LPC));
  static constexpr int A2 = (NF == 32 && S == 4) ? 3 : 0;
  __host__ __device__ static constexpr int g(int x) {
    return x ^ ((x >> A1) & ((1 << S) - 1)) ^ (A2 ? ((x >> A2) & ((1 << S) - 1)) : 0);
  }
};
// value at swizzled index gx ^ c (c a compile-time constant) of a stage buffer
template <typename T>
__device__ __forceinline__ const C2<T> &at_xor(const C2<T> *buf, int gxb, int cb) {
  return *reinterpret_cast<const C2<T> *>(reinterpret_cast<const unsigned char *>(buf) + (gxb ^ cb));
}
template <typename T>
__device__ __forceinline__ C2<T> &at_xor(C2<T> *buf, int gxb, int cb) {
  return *reinterpret_cast<C2<T> *>(reinterpret_cast<unsigned char *>(buf) + (gxb ^ cb));
}

// Lengths whose twiddle tables would crowd a block's shared memory (16 KB
// and more, which costs the second block per SM; for 8-byte values 8 KB,
// which leaves the room the transform-axis offsets need) read the twiddles
// through L1 from the pass's root table instead.
__host__ __device__ constexpr bool global_twiddles(int n, size_t es) {
  return (size_t)n * es >= (es == 8 ? 8192u : 16384u);
}

// Twiddles of the power-of-two stages, staged in shared memory once per
// block: stage (LP, R) keeps w_{LP R}^{j q} (conjugated for the inverse) at
// LP - 1 + (q - 1) LP + j, so that a thread's R - 1 twiddles sit at
// compile-time offsets from its j and neighbouring threads read neighbouring
// entries.  The stages' tables add up to NF - 1 entries (the first stage's
// are ones and unused).
template <typename T, int SIGN, int NF>
__device__ __forceinline__ void pow2_twiddles(const C2<T> *roots, C2<T> *tws, int tid) {
  for (int e = tid; e < NF - 1; e += NT) {
    int lp = 1;
#pragma unroll
    for (int s = 0; s < 12; ++s) {
      const int r = fixed_radix(NF, lp);
      if (e + 1 < lp * r) break;
      lp *= r;
    }
    const int r = fixed_radix(NF, lp);
    const int e2 = e - (lp - 1);
    const int q = e2 / lp + 1, j = e2 % lp;
    const C2<T> w = roots[j * q * (NF / (lp * r))];
    tws[e] = SIGN > 0 ? conj<T>(w) : w;
  }
}

// The Stockham stage after the first LP points of a power-of-two NF: from
// the line-padded staging layout (first stage) or the previous stage's
// swizzled layout, to the next stage's swizzled layout or (last stage) the
// line-padded layout the scatter reads.  tws: the tables above.
template <typename T, int SIGN, int NF, int LP>
__device__ __forceinline__ void stage_pow2(const C2<T> *in, C2<T> *out, const C2<T> *tws, int nlines, int ld, int tid,
                                           bool conv, int sexp, const C2<T> *groots = nullptr) {
  constexpr int R = fixed_radix(NF, LP);
  constexpr int NR = NF / R;
  constexpr int M = NR / LP;
  constexpr int LGNR = ilog2(NR), LGM = ilog2(M), LGNF = ilog2(NF);
  constexpr int ES = (int)sizeof(C2<T>);
  constexpr bool IN_SWZ = LP > 1, OUT_SWZ = LP * R < NF;
  using Gin = HopSwz<T, NF, LP>;
  using Gout = HopSwz<T, NF, (LP * R < NF ? LP * R : LP)>;
  const C2<T> *tw = tws + (LP - 1);
  const int nb = nlines * NR;
  for (int b = tid; b < nb; b += NT) {
    const int l = b >> LGNR;
    const int bb = b & (NR - 1);
    const int j = bb >> LGM;
    const int k = bb & (M - 1);
    C2<T> a[R];
    constexpr bool FMA8 = std::is_same<T, double>::value && (R == 8 || R == 4) && IN_SWZ;
    if constexpr (FMA8) {
      // native FP64, twiddled radix 8 or 4: the twiddles go into the butterflies
      const int gxb = Gin::g((l << LGNF) + j * R * M + k) * ES;
#pragma unroll
      for (int q = 0; q < R; ++q) a[q] = at_xor<T>(in, gxb, Gin::g(q * M) * ES);
      constexpr int TSTEP = NF / (LP * R);
      C2<T> w1, w2;
      if constexpr (global_twiddles(NF, sizeof(C2<T>))) {
        w1 = root_at<T, SIGN>(tws, j * TSTEP);
        w2 = root_at<T, SIGN>(tws, 2 * j * TSTEP);
      } else {
        w1 = tw[j];
        w2 = tw[LP + j];
      }
      if constexpr (R == 8) {
        const C2<T> w4 = global_twiddles(NF, sizeof(C2<T>)) ? root_at<T, SIGN>(tws, 4 * j * TSTEP) : tw[3 * LP + j];
        const C2<T> v = root_at<T, SIGN>(groots, j * TSTEP + NF / 8);
        dft8_tw_fma<SIGN>(a, w1, w2, w4, v);
      } else {
        dft4_tw_fma<SIGN>(a, w1, w2);
      }
    } else if constexpr (IN_SWZ) {
      const int gxb = Gin::g((l << LGNF) + j * R * M + k) * ES;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        C2<T> v = at_xor<T>(in, gxb, Gin::g(q * M) * ES);
        if constexpr (global_twiddles(NF, sizeof(C2<T>))) {
          // tws: the pass's root table exp(-2 pi i k / NF)
          if (q > 0) v = mul<T>(v, root_at<T, SIGN>(tws, j * q * (NF / (LP * R))));
        } else {
          if (q > 0) v = mul<T>(v, tw[(q - 1) * LP + j]);
        }
        a[q] = v;
      }
    } else {
      const int lo = l * ld;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int pos = lo + swz<T, NF>(q * M + k);
        C2<T> v;
        if constexpr (std::is_same<T, df>::value) {
          if (conv) {
            const double2 d = reinterpret_cast<const double2 *>(in)[pos];
            const df re = to_df(d.x, sexp), im = to_df(d.y, sexp);
            v = dfc{make_float2(re.h, im.h), make_float2(re.l, im.l)};
          } else {
            v = in[pos];
          }
        } else {
          (void)conv;
          (void)sexp;
          v = in[pos];
        }
        a[q] = v;
      }
    }
    if constexpr (!FMA8) bfly_fixed<T, SIGN, R>(a);
    if constexpr (OUT_SWZ) {
      const int gyb = Gout::g((l << LGNF) + bb) * ES;
#pragma unroll
      for (int s = 0; s < R; ++s) at_xor<T>(out, gyb, Gout::g(s * NR) * ES) = a[s];
    } else {
      const int lo = l * ld;
#pragma unroll
      for (int s = 0; s < R; ++s) out[lo + swz<T, NF>(bb + s * NR)] = a[s];
    }
  }
  __syncthreads();
}

// The Stockham stage after the first LP points of NF, from `in` to `out`.
// roots: the pass's global table.
// conv (first stage of a double-float pass that reads complex128): the
// staging buffer holds raw complex128 values, converted here with the scale
// exponent sexp as they are loaded.
template <typename T, int SIGN, int NF, int LP>
__device__ __forceinline__ void stage_fixed(const C2<T> *in, C2<T> *out, const C2<T> *roots, int nlines, int ld,
                                            int tid, bool conv = false, int sexp = 0) {
  constexpr int R = fixed_radix(NF, LP);
  constexpr int NR = NF / R;
  constexpr int M = NR / LP;
  constexpr int TSTEP = NF / (LP * R);
  const int nb = nlines * NR;
  for (int b = tid; b < nb; b += NT) {
    const int l = b / NR;
    const int bb = b % NR;
    const int j = bb / M;
    const int k = bb % M;
    const int lo = l * ld;
    C2<T> a[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int pos = lo + swz<T, NF>(j * R * M + q * M + k);
      C2<T> v;
      if constexpr (std::is_same<T, df>::value && LP == 1) {
        if (conv) {
          const double2 d = reinterpret_cast<const double2 *>(in)[pos];
          const df re = to_df(d.x, sexp), im = to_df(d.y, sexp);
          v = dfc{make_float2(re.h, im.h), make_float2(re.l, im.l)};
        } else {
          v = in[pos];
        }
      } else {
        (void)conv;
        (void)sexp;
        v = in[pos];
      }
      // (native FP64 radix 8 and 4: the twiddles go into the butterflies below)
      if (LP > 1 && q > 0 && !(std::is_same<T, double>::value && (R == 8 || R == 4)))
        v = mul<T>(v, root_fx<T, SIGN>(roots, j * q * TSTEP));
      a[q] = v;
    }
    if constexpr (std::is_same<T, double>::value && (R == 8 || R == 4) && LP > 1) {
      const C2<T> w1 = root_fx<T, SIGN>(roots, j * TSTEP), w2 = root_fx<T, SIGN>(roots, 2 * j * TSTEP);
      if constexpr (R == 8) {
        dft8_tw_fma<SIGN>(a, w1, w2, root_fx<T, SIGN>(roots, 4 * j * TSTEP),
                          root_fx<T, SIGN>(roots, j * TSTEP + NF / 8));
      } else {
        dft4_tw_fma<SIGN>(a, w1, w2);
      }
    } else {
      bfly_fixed<T, SIGN, R>(a);
    }
#pragma unroll
    for (int s = 0; s < R; ++s) out[lo + swz<T, NF>((j + s * LP) * M + k)] = a[s];
  }
  __syncthreads();
}

// Stages from LP on: `in` to `out`, then back and forth between `out` and
// `spare`; returns the buffer holding the result.
template <typename T, int SIGN, int NF, int LP>
__device__ __forceinline__ C2<T> *stages_fixed(C2<T> *in, C2<T> *out, C2<T> *spare, const C2<T> *roots, int nlines,
                                               int ld, int tid, const C2<T> *groots = nullptr) {
  if constexpr (LP < NF) {
    if constexpr (pow2_length(NF)) {
      stage_pow2<T, SIGN, NF, LP>(in, out, roots, nlines, ld, tid, false, 0, groots);
    } else {
      stage_fixed<T, SIGN, NF, LP>(in, out, roots, nlines, ld, tid);
    }
    return stages_fixed<T, SIGN, NF, LP * fixed_radix(NF, LP)>(out, spare, out, roots, nlines, ld, tid, groots);
  } else {
    (void)out;
    (void)spare;
    return in;
  }
}

// A value of the pass's input: complex128 converted to double-float (scaled
// by 2^-s) when the double-float pass reads complex128, else as stored.
template <typename T>
__device__ __forceinline__ C2<T> load_elem(const void *src, int64_t a, bool fp64, int s) {
  if constexpr (std::is_same<T, df>::value) {
    if (fp64) {
      const double2 d = reinterpret_cast<const double2 *>(src)[a];
      const df re = to_df(d.x, s), im = to_df(d.y, s);
      return dfc{make_float2(re.h, im.h), make_float2(re.l, im.l)};
    }
  }
  (void)fp64;
  (void)s;
  return reinterpret_cast<const C2<T> *>(src)[a];
}

template <typename T>
__device__ __forceinline__ void store_elem(void *dst, int64_t a, C2<T> v, bool fp64, int s) {
  if constexpr (std::is_same<T, df>::value) {
    if (fp64) {
      double2 d;
      d.x = from_df(df{v.h.x, v.l.x}, s);
      d.y = from_df(df{v.h.y, v.l.y}, s);
      reinterpret_cast<double2 *>(dst)[a] = d;
      return;
    }
  }
  (void)fp64;
  (void)s;
  reinterpret_cast<C2<T> *>(dst)[a] = v;
}

// ---------------------------------------------------------------- shared memory

// the largest dynamic shared memory per block with which the shared
// transform-axis offsets are kept: two blocks per SM, each at most 112 KB
// with its 1 KB reserve and static shared memory (measured: at 115 KB the
// 1024-point FP32 passes fell to one block per SM)
#ifndef DMG_FFT_T0_SMEM_LIMIT
#define DMG_FFT_T0_SMEM_LIMIT 113328
#endif

// int64 entries of one side's separable address parts for a tile: unused,
// M1 entries of v1's dimension, M2 of v2's, 3 of the dimensions no tile axis
// covers
__host__ __device__ inline int parts_len(const dmg_fft_pass &p) { return 4 + p.M1 + p.M2; }

// Carve-up of a pass block's dynamic shared memory (host and device agree):
// the staging buffer the gather copies the next tile into, two buffers the
// stages go between, then small tables (twiddles or roots, address parts,
// buffer positions along the transform axis).
struct SmemLayout {
  int ld;             // line pitch in values (odd)
  size_t buf_a, buf_b; // byte offsets of the stage buffers (the staging buffer is at 0)
  size_t roots_off;   // compile-time lengths: the per-stage twiddle tables (powers of two) or the n roots
  size_t contrib_off; // separable address parts (parts_len int64 each): gather side, then two scatter-side areas
  size_t spos_off;    // int16 buffer positions of the transform axis's coordinates: gather side, then scatter side
  size_t t0_off;      // int32 transform-axis address offsets: gather side (has_t0_in), then scatter side (has_t0_out)
  int has_t0_in, has_t0_out;
  size_t total;
};

// Lengths with their own kernels: powers of two 8 ... 2048 and the 2, 3,
// 5-smooth cube sides 48 ... 480.
__host__ __device__ constexpr bool fixed_length(int n) {
  return n == 8 || n == 16 || n == 32 || n == 64 || n == 128 || n == 256 || n == 512 || n == 1024 || n == 2048 ||
         n == 48 || n == 96 || n == 120 || n == 160 || n == 192 || n == 240 || n == 320 || n == 384 || n == 480;
}

// The tensor-core form of the 1024-point FP32 pass (tc = true) keeps, after
// the staging buffer, an area of TC_AREA bytes (aligned at run time to 1024
// bytes inside it): the two A operands of a product (hi and lo halves, 16 KB
// each; the line-padded result after the second product), the two B operands
// (the 32-point DFT matrix's hi and lo halves, 8 KB each) and the rows' scale
// exponents.
constexpr size_t TC_A_BYTES = 33792;  // >= 32 KB of operands and >= 4 lines x 1025 x 8 bytes of result
constexpr size_t TC_B_BYTES = 16384;
constexpr size_t TC_EXP_BYTES = 1024;
constexpr size_t TC_AREA = 1024 + TC_A_BYTES + TC_B_BYTES + TC_EXP_BYTES;

template <typename T>
__host__ __device__ inline SmemLayout smem_layout(const dmg_fft_pass &p, bool fixed, bool tc = false) {
  SmemLayout s;
  const size_t es = sizeof(C2<T>);
  const int n = p.n;
  s.ld = n | 1;
  const size_t one = fixed && pow2_length(n) ? pow2_stride(es, n) : (size_t)p.M1 * p.M2 * s.ld * es;
  s.buf_a = one;
  s.buf_b = 2 * one;
  size_t pos = tc ? ((one + TC_AREA + 15) & ~(size_t)15) : ((3 * one + 15) & ~(size_t)15);
  s.roots_off = pos;
  if (!tc && fixed && (pow2_length(n) ? !global_twiddles(n, es) : DMG_FFT_SMEM_ROOTS)) pos += (size_t)n * es;
  s.contrib_off = pos;
  pos += (size_t)3 * parts_len(p) * sizeof(int64_t);
  s.spos_off = pos;
  pos += (size_t)2 * n * sizeof(int16_t);
  // the transform axis's address offsets in shared memory where a side
  // qualifies and two blocks per SM still fit
  pos = (pos + 15) & ~(size_t)15;
  s.t0_off = pos;
  s.has_t0_in = p.t0_rel_in && pos + (size_t)n * sizeof(int32_t) <= DMG_FFT_T0_SMEM_LIMIT;
  if (s.has_t0_in) pos += (size_t)n * sizeof(int32_t);
  s.has_t0_out = p.t0_rel_out && pos + (size_t)n * sizeof(int32_t) <= DMG_FFT_T0_SMEM_LIMIT;
  if (s.has_t0_out) pos += (size_t)n * sizeof(int32_t);
  s.total = (pos + 15) & ~(size_t)15;
  return s;
}

template <typename T>
__host__ __device__ inline bool use_fixed(const dmg_fft_pass &p) {
  return fixed_length(p.n) && !p.radix_runtime;
}


// ---------------------------------------------------------------- asynchronous copies

// global -> shared copy of one value that completes in the background
// (cp.async, 16 bytes through L2 only, 8 bytes through L1)
// (sa: a shared-window address)
template <int BYTES>
__device__ __forceinline__ void copy_async_sa(unsigned sa, const void *gmem) {
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
  } else {
    static_assert(BYTES == 8, "8- or 16-byte values");
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
  }
}
template <int BYTES>
__device__ __forceinline__ void copy_async(void *smem, const void *gmem) {
  copy_async_sa<BYTES>((unsigned)__cvta_generic_to_shared(smem), gmem);
}
__device__ __forceinline__ void copy_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void copy_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Start the copies of one side's separable address parts for a tile (table
// entries, asynchronously; part has parts_len entries): part[1 + c] and
// part[1 + M1 + c] the entries of the v1 and v2 dimensions (0 past the tile's
// extent), part[1 + M1 + M2 + u] that of dimension u when no tile axis
// covers it (else 0), and part[0] the paired dimension's entry at the
// tile's start (pair: that dimension holds two tile axes and a sum of parts
// along them; else 0).  The side's address is then L.base + the last three
// - part[0] + the tables of the tile axes.
__device__ __forceinline__ void sep_parts_async(const dmg_fft_layout &L, const dmg_fft_pass &p, const int *yb,
                                                const int *zb, int lim1, int lim2, int tid, int64_t *part,
                                                bool semi = false, bool pair = false) {
  const int M1 = p.M1;
  const int E = 1 + M1 + p.M2;
  for (int i = tid; i < E + 3; i += NT) {
    if (i == 0) {
      if (pair) {
        const int d = p.kdim[p.semi_a];
        copy_async<8>(part, L.tab[d] + (yb[d] + p.A[d] * zb[d]));
      } else {
        part[0] = 0;
      }
    } else if (i >= E) {
      const int d = i - E;
      if (d < p.ndim && d != p.kdim[0] && d != p.kdim[1] && d != p.kdim[2])
        copy_async<8>(part + i, L.tab[d] + (yb[d] + p.A[d] * zb[d]));
      else
        part[i] = 0;
    } else {
      const int k = i <= M1 ? 1 : 2;
      const int c = k == 1 ? i - 1 : i - 1 - M1;
      const int d = p.kdim[k];
      // (a side with two axes in one dimension reads that dimension per value)
      const bool paired = semi && (k == p.semi_a || k == p.semi_b);
      if (d >= 0 && !paired && c < (k == 1 ? lim1 : lim2)) {
        const int x = yb[d] + p.A[d] * zb[d] + (p.kisz[k] ? p.A[d] * c : c);
        copy_async<8>(part + i, L.tab[d] + x);
      } else {
        part[i] = 0;
      }
    }
  }
}
// A side with two tile axes in one dimension: that dimension's table and the
// coordinate's start and steps along the two axes (x = x0 + sa ca + sb cb),
// for a tile.
struct SharedDim {
  const int64_t *tab;
  int x0, sa, sb;
  bool t_paired;  // the transform axis is one of the two
};
__device__ __forceinline__ SharedDim shared_dim(const dmg_fft_layout &L, const dmg_fft_pass &p, const int *yb,
                                                const int *zb) {
  const int d = p.kdim[p.semi_a];
  SharedDim s;
  s.tab = L.tab[d];
  s.x0 = yb[d] + p.A[d] * zb[d];
  s.sa = p.kisz[p.semi_a] ? p.A[d] : 1;
  s.sb = p.kisz[p.semi_b] ? p.A[d] : 1;
  s.t_paired = p.semi_a == 0;
  return s;
}
// the shared dimension's table entry at tile offsets (c0, c1, c2)
__device__ __forceinline__ int64_t shared_dim_part(const SharedDim &s, const dmg_fft_pass &p, int c0, int c1, int c2) {
  const int ca = p.semi_a == 0 ? c0 : c1;  // semi_a < semi_b
  const int cb = p.semi_b == 1 ? c1 : c2;
  return __ldg(s.tab + s.x0 + s.sa * ca + s.sb * cb);
}

// the base of a separable side's addresses in a tile (parts complete)
__device__ __forceinline__ int64_t sep_base(const dmg_fft_layout &L, const dmg_fft_pass &p, const int64_t *part) {
  const int E = 1 + p.M1 + p.M2;
  return L.base + part[E] + part[E + 1] + part[E + 2] - part[0];
}

// ---------------------------------------------------------------- the pass kernel

#ifndef DMG_FFT_EPT
#define DMG_FFT_EPT 4
#endif
constexpr int EPT = DMG_FFT_EPT;  // values a thread stores per scatter round
#ifndef DMG_FFT_MINB
#define DMG_FFT_MINB 2
#endif
constexpr int MINB = DMG_FFT_MINB;  // resident blocks per SM the register budget allows

// A tile's place in the pass (and which job of the batch it belongs to).
struct TileState {
  int yb[DMG_FFT_MAXDIM], zb[DMG_FFT_MAXDIM];
  int lim1, lim2, ytw;
  int job, sexp;
};

// The tile index as digits (v1 tile, v2 tile, the batch sub-axes, the job;
// radices nt1, nt2, blen[], count): a block steps through its tiles by
// adding the digits of the grid size, without dividing.
constexpr int NDIG = 9;

// Values every phase needs.  They live in shared memory and each phase
// reads them after a barrier, so that none of them holds a register through
// the FFT stages.
struct PassConsts {
  int ld, M1, d0, mult0, td, v1_ytd, v2_ytd, in64, out64;
  int tw_kmaj;  // the store walk steps along y first: read the k-major twiddle table
  unsigned buf_a, buf_b, roots_off, contrib_off, spos_off, t0_off;
  int t0_in, t0_out;              // the sides whose transform-axis offsets are in shared memory
  int64_t t0base_in, t0base_out;  // their first entries
  int ndig, rad[NDIG], inc[NDIG], dig[NDIG];
  TileState ts[3];  // the tile being transformed, the one being gathered, the one after
  // tensor-core form: the MMA completion barrier, the tensor-memory columns, a wait that gave up
  uint64_t tc_bar;
  uint32_t tc_taddr;
  int tc_fail;
};

__device__ __forceinline__ void tile_digits(const int *rad, int nd, int64_t t, int *dig) {
  for (int i = 0; i < nd; ++i) {
    dig[i] = (int)(t % rad[i]);
    t /= rad[i];
  }
}
__device__ __forceinline__ void digits_add(int *dig, const int *inc, const int *rad, int nd) {
  int carry = 0;
  for (int i = 0; i < nd; ++i) {
    const int v = dig[i] + inc[i] + carry;
    carry = v >= rad[i];
    dig[i] = carry ? v - rad[i] : v;
  }
}

// A tile's place from its digits.
template <typename T>
__device__ __forceinline__ void tile_state_digits(const dmg_fft_pass &p, const dmg_fft_batch &bt, const int *dig,
                                                  TileState &st) {
  const int i1 = dig[0], i2 = dig[1];
  st.job = dig[2 + p.nbatch];
  // scale exponent of the double-float conversions (bias removed, inputs end below 2)
  st.sexp = (std::is_same<T, df>::value && (p.in_fp64 || p.out_fp64)) ? __ldg(bt.scale_exp[st.job]) - 1022 : 0;
  int yb[DMG_FFT_MAXDIM] = {0, 0, 0}, zb[DMG_FFT_MAXDIM] = {0, 0, 0};
  for (int b = 0; b < p.nbatch; ++b) {
    const int c = dig[2 + b];
    const int s = p.bsub[b];
    if (s & 1) zb[s >> 1] += c;
    else yb[s >> 1] += c;
  }
  if (p.v1 >= 0) {
    if (p.v1 & 1) zb[p.v1 >> 1] += i1 * p.M1;
    else yb[p.v1 >> 1] += i1 * p.M1;
  }
  if (p.v2 >= 0) {
    if (p.v2 & 1) zb[p.v2 >> 1] += i2 * p.M2;
    else yb[p.v2 >> 1] += i2 * p.M2;
  }
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    st.yb[d] = yb[d];
    st.zb[d] = zb[d];
  }
  st.ytw = yb[p.t >> 1];
  st.lim1 = p.v1 >= 0 ? min(p.M1, p.nv1 - i1 * p.M1) : 1;
  st.lim2 = p.v2 >= 0 ? min(p.M2, p.nv2 - i2 * p.M2) : 1;
}


// Visits the values of a tile that thread `tid` owns on a separable side,
// calling f(address, staging position, c0, c1, c2).  Warps run along the
// walk's fastest axis (order[0], the one contiguous in the layout).  When that
// axis is at most NT long, each thread keeps one fast coordinate (and its
// address part) for the whole tile and steps over rows; when it is longer,
// each thread keeps up to 8 fast coordinates and loops over rows.  Address
// parts: the transform axis's from its table (tab0, step mult0), the vector
// axes' from the per-tile table `part`.  Returns false (visiting nothing)
// when the fast axis is longer than 8 * NT.
// The same walk for the usual axis orders (ORD 0: t, v1, v2 fastest first;
// 1: v1, t, v2; 2: v1, v2, t) with the axes' roles fixed at compile time, so
// that a value costs its table reads and additions only.  Returns false
// (visiting nothing) where it does not apply.
__host__ __device__ constexpr int walk_order_code(int a, int b, int c) {
  return (a == 0 && b == 1 && c == 2) ? 0 : (a == 1 && b == 0 && c == 2) ? 1 : (a == 1 && b == 2 && c == 0) ? 2 : -1;
}
// REL: the transform axis's entries come from shared memory (t0rel, offsets
// from t0base) instead of the table.
template <typename T, int NF, int ORD, bool REL, typename F>
__device__ __forceinline__ bool sep_walk_ord(int n, int lim1, int lim2, int M1, int ld, const int64_t *tab0, int mult0,
                                             int64_t base, const int64_t *part, const int16_t *spos, int tid, F &&f,
                                             const int32_t *t0rel, int64_t t0base) {
  // table reads in flight per thread: 8-byte values can afford more registers
  constexpr int WALK_UNROLL = sizeof(C2<T>) == 8 ? 8 : 4;
  const int nn = NF > 0 ? NF : n;
  auto T0 = [&](int i) -> int64_t {
    if constexpr (REL) {
      return t0base + t0rel[i];
    } else {
      return __ldg(tab0 + i * mult0);
    }
  };
  if constexpr (ORD == 0) {
    if constexpr (NF > 0 && NF >= NT && NF % NT == 0 && NF / NT <= 8) {
      // each thread keeps NF / NT coordinates along t; rows are the tile's lines
      constexpr int J = NF / NT;
      int64_t af[J];
      int sf[J];
#pragma unroll
      for (int j = 0; j < J; ++j) {
        af[j] = base + T0(tid + j * NT);
        sf[j] = spos[tid + j * NT];
      }
      for (int i_s = 0; i_s < lim2; ++i_s) {
        const int64_t a2 = part[1 + M1 + i_s];
        for (int i_m = 0; i_m < lim1; ++i_m) {
          const int64_t ar = a2 + part[1 + i_m];
          const int sr = (i_m + M1 * i_s) * ld;
#pragma unroll
          for (int j = 0; j < J; ++j) f(af[j] + ar, sf[j] + sr, tid + j * NT, i_m, i_s);
        }
      }
      return true;
    } else {
      return false;
    }
  } else {
    // v1 fastest: each thread keeps one v1 coordinate; rows run over the
    // other two axes (t then v2 for ORD 1, v2 then t for ORD 2)
    const int ef = lim1;
    if (ef > NT) return false;
    const int rstep = NT / ef;
    if (tid >= rstep * ef) return true;
    const int i_f = tid % ef;
    const int r0 = tid / ef;
    const int64_t af = base + part[1 + i_f];
    const int sf = i_f * ld;
    if constexpr (ORD == 1) {
      if (nn % rstep == 0) {
        // rows r0 + k rstep: t = r0 + k rstep for k < nn / rstep within each v2 row
        const int kn = nn / rstep;
        for (int i_s = 0; i_s < lim2; ++i_s) {
          const int64_t a2 = af + part[1 + M1 + i_s];
          const int s2 = sf + i_s * M1 * ld;
#pragma unroll WALK_UNROLL
          for (int k = 0; k < kn; ++k) {
            const int t = r0 + k * rstep;
            f(a2 + T0(t), s2 + spos[t], t, i_f, i_s);
          }
        }
      } else {
        int t = r0 % nn, i_s = r0 / nn;
        const int dm = rstep % nn, ds = rstep / nn;
        while (i_s < lim2) {
          f(af + T0(t) + part[1 + M1 + i_s], sf + spos[t] + i_s * M1 * ld, t, i_f, i_s);
          t += dm;
          i_s += ds;
          if (t >= nn) {
            t -= nn;
            ++i_s;
          }
        }
      }
    } else if (lim2 == 1 && nn % rstep == 0) {
      // one v2 value: rows are t = r0 + k rstep
      const int kn = nn / rstep;
      const int64_t a2 = af + part[1 + M1];
#pragma unroll WALK_UNROLL
      for (int k = 0; k < kn; ++k) {
        const int t = r0 + k * rstep;
        f(a2 + T0(t), sf + spos[t], t, i_f, 0);
      }
    } else {
      // rows (v2, t): v2 = r % lim2, t = r / lim2
      int i_m = r0 % lim2, t = r0 / lim2;
      const int dm = rstep % lim2, ds = rstep / lim2;
      while (t < nn) {
        f(af + part[1 + M1 + i_m] + T0(t), sf + i_m * M1 * ld + spos[t], t, i_f, i_m);
        i_m += dm;
        t += ds;
        if (i_m >= lim2) {
          i_m -= lim2;
          ++t;
        }
      }
    }
    return true;
  }
}
// walk by the side's order: a specialised form where one applies
template <typename T, int NF, typename F>
__device__ __forceinline__ bool sep_walk_any(const int32_t *order, int n, int lim1, int lim2, int M1, int ld,
                                             const int64_t *tab0, int mult0, int64_t base, const int64_t *part,
                                             const int16_t *spos, int tid, F &&f, const int32_t *t0rel,
                                             int64_t t0base);

template <typename T, int NF, typename F>
__device__ __forceinline__ bool sep_walk(const int32_t *order, int n, int lim1, int lim2, int M1, int ld,
                                         const int64_t *tab0, int mult0, int64_t base, const int64_t *part,
                                         const int16_t *spos, int tid, F &&f) {
  const int kf = order[0], km = order[1], ks = order[2];
  auto E = [&](int k) { return k == 0 ? n : (k == 1 ? lim1 : lim2); };
  auto AP = [&](int k, int i) -> int64_t { return k == 0 ? __ldg(tab0 + i * mult0) : part[k == 1 ? 1 + i : 1 + M1 + i]; };
  auto SP = [&](int k, int i) -> int {
    return k == 0 ? (int)spos[i] : (k == 1 ? i * ld : i * M1 * ld);
  };
  auto C = [&](int k, int i_f, int i_m, int i_s) { return kf == k ? i_f : (km == k ? i_m : i_s); };
  const int ef = E(kf), em = E(km), es = E(ks);
  const int rows = em * es;
  if (ef <= NT) {
    const int rstep = NT / ef;
    if (tid >= rstep * ef) return true;
    const int i_f = tid % ef;
    const int64_t af = base + AP(kf, i_f);
    const int sf = SP(kf, i_f);
    if (es == 1) {
      const int64_t a1 = af + AP(ks, 0);
      const int s1 = sf + SP(ks, 0);
#pragma unroll 4
      for (int r = tid / ef; r < rows; r += rstep)
        f(a1 + AP(km, r), s1 + SP(km, r), C(0, i_f, r, 0), C(1, i_f, r, 0), C(2, i_f, r, 0));
    } else {
      // rows r = tid / ef + k * rstep as (i_m, i_s) = (r % em, r / em), stepped without dividing
      const int r0 = tid / ef;
      int i_m = r0 % em, i_s = r0 / em;
      const int dm = rstep % em, ds = rstep / em;
      while (i_s < es) {
        f(af + AP(km, i_m) + AP(ks, i_s), sf + SP(km, i_m) + SP(ks, i_s), C(0, i_f, i_m, i_s), C(1, i_f, i_m, i_s),
          C(2, i_f, i_m, i_s));
        i_m += dm;
        i_s += ds;
        if (i_m >= em) {
          i_m -= em;
          ++i_s;
        }
      }
    }
    return true;
  }
  if (ef > 8 * NT) return false;
  int64_t af[8];
  int sf[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int i_f = tid + j * NT;
    if (i_f < ef) {
      af[j] = base + AP(kf, i_f);
      sf[j] = SP(kf, i_f);
    }
  }
  for (int i_m = 0, i_s = 0; i_s < es;) {
    const int64_t ar = AP(km, i_m) + AP(ks, i_s);
    const int sr = SP(km, i_m) + SP(ks, i_s);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int i_f = tid + j * NT;
      if (i_f < ef) f(af[j] + ar, sf[j] + sr, C(0, i_f, i_m, i_s), C(1, i_f, i_m, i_s), C(2, i_f, i_m, i_s));
    }
    if (++i_m == em) {
      i_m = 0;
      ++i_s;
    }
  }
  return true;
}

template <typename T, int NF, typename F>
__device__ __forceinline__ bool sep_walk_any(const int32_t *order, int n, int lim1, int lim2, int M1, int ld,
                                             const int64_t *tab0, int mult0, int64_t base, const int64_t *part,
                                             const int16_t *spos, int tid, F &&f, const int32_t *t0rel,
                                             int64_t t0base) {
  const int code = walk_order_code(order[0], order[1], order[2]);
  if (code == 0 &&
      sep_walk_ord<T, NF, 0, false>(n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f, t0rel, t0base))
    return true;
  if (code == 1 && t0rel &&
      sep_walk_ord<T, NF, 1, true>(n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f, t0rel, t0base))
    return true;
  if (code == 1 && !t0rel &&
      sep_walk_ord<T, NF, 1, false>(n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f, t0rel, t0base))
    return true;
  if (code == 2 && t0rel &&
      sep_walk_ord<T, NF, 2, true>(n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f, t0rel, t0base))
    return true;
  if (code == 2 && !t0rel &&
      sep_walk_ord<T, NF, 2, false>(n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f, t0rel, t0base))
    return true;
  return sep_walk<T, NF>(order, n, lim1, lim2, M1, ld, tab0, mult0, base, part, spos, tid, f);
}

// Start the copies of a tile into the staging buffer (raw values: a
// complex128 input of a double-float pass is converted once it is there).
template <typename T, int NF>
__device__ __forceinline__ void gather_async(const dmg_fft_pass &p, const PassConsts &kc, const TileState &st,
                                             const unsigned char *sm, const int64_t *pin, const dmg_fft_batch &bt,
                                             int tid) {
  constexpr bool FIXED = NF > 0;
  const int n = FIXED ? NF : p.n;
  const int ld = kc.ld, M1 = kc.M1;
  int yb[DMG_FFT_MAXDIM], zb[DMG_FFT_MAXDIM];
#pragma unroll
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    yb[d] = st.yb[d];
    zb[d] = st.zb[d];
  }
  const int lim1 = st.lim1, lim2 = st.lim2;
  const int total = n * lim1 * lim2;
  const int d0 = kc.d0, mult0 = kc.mult0;
  const int16_t *spos = reinterpret_cast<const int16_t *>(sm + kc.spos_off);
  const int64_t *tab0 = p.in.tab[d0] + (yb[d0] + p.A[d0] * zb[d0]);
  const int64_t in0 = (p.sep_in || p.semi_in) ? sep_base(p.in, p, pin) : 0;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(sm);  // the staging buffer
  const unsigned char *gsrc = static_cast<const unsigned char *>(bt.src[st.job]);
  if (p.sep_in &&
      sep_walk_any<T, NF>(p.load_order, n, lim1, lim2, M1, ld, tab0, mult0, in0, pin, spos, tid,
                          [&](int64_t ad, int sp, int, int, int) {
                        copy_async_sa<sizeof(C2<T>)>(sbase + (unsigned)(sp * (int)sizeof(C2<T>)),
                                                     gsrc + ad * (int64_t)sizeof(C2<T>));
                      },
                          kc.t0_in ? reinterpret_cast<const int32_t *>(sm + kc.t0_off) : nullptr, kc.t0base_in)) {
    copy_async_commit();
    return;
  }
  const SharedDim sd = p.semi_in ? shared_dim(p.in, p, yb, zb) : SharedDim{};
  TileWalk w(tid, p.load_pos, n, lim1, lim2);
  for (int e = tid; e < total; e += NT, w.next()) {
    const int c0 = w.coord(p.load_pos[0]), c1 = w.coord(p.load_pos[1]), c2 = w.coord(p.load_pos[2]);
    int64_t ad;
    if (p.sep_in) {
      ad = in0 + __ldg(tab0 + c0 * mult0) + pin[1 + c1] + pin[1 + M1 + c2];
    } else if (p.semi_in) {
      // the paired axes' parts are zero in pin
      ad = in0 + shared_dim_part(sd, p, c0, c1, c2) + (sd.t_paired ? 0 : __ldg(tab0 + c0 * mult0)) + pin[1 + c1] +
           pin[1 + M1 + c2];
    } else {
      int x[DMG_FFT_MAXDIM];
      element_x(p, yb, zb, c0, c1, c2, x);
      ad = layout_addr(p.in, p.ndim, x);
    }
    const int sp = (c1 + M1 * c2) * ld + spos[c0];
    copy_async_sa<sizeof(C2<T>)>(sbase + (unsigned)(sp * (int)sizeof(C2<T>)), gsrc + ad * (int64_t)sizeof(C2<T>));
  }
  copy_async_commit();
}

// ---------------------------------------------------------------- tensor-core stages (1024-point FP32 lines)
//
// The 1024-point DFT of a line as two 32-point DFT products on the tensor
// cores (four-step: t = t1 + 32 t2, k = k2 + 32 k1):
//   Z[t1, k2] = sum_t2 x[t1 + 32 t2] w32^(t2 k2)                 (product 1)
//   X[k2 + 32 k1] = sum_t1 (Z[t1, k2] w1024^(t1 k2)) w32^(t1 k1)  (product 2)
// A tile's four lines give M = 4 x 32 = 128 rows (row = line * 32 + t1, then
// line * 32 + k2); a complex value is two real columns (re, im), so each
// product is D[128 x 64] = A[128 x 64] B[64 x 64]^T with B the real form of
// the 32-point DFT matrix ([c, -s; s, c] blocks).  Operands are split into
// FP16 hi + lo parts and D = Al Bh + Ah Bl + Ah Bh accumulates in FP32 in
// tensor memory; each row is scaled by a power of two first so that its
// largest magnitude lies in [2^14, 2^15) (FP16's range), and the product is
// scaled back as it leaves tensor memory.  The twiddle w1024^(t1 k2) is
// applied in FP32 between the products.

// MMA completion waits give up after this many polls (a fault, not a slow
// product: one product takes well under a microsecond)
constexpr uint32_t TC_WAIT_LIMIT = 1u << 22;

// 2^e as a float, e in [-126, 126]
__device__ __forceinline__ float tc_pow2(int e) { return __uint_as_float((uint32_t)(127 + e) << 23); }

// scale exponent of a row whose largest |component| has the bit pattern m
__device__ __forceinline__ int tc_row_exp(uint32_t m) {
  if (m == 0) return 0;
  const int e = (int)(m >> 23) - 127 - 14;
  return e < -126 ? -126 : (e > 126 ? 126 : e);
}

__device__ __forceinline__ uint32_t tc_bits(__half2 h) {
  uint32_t u;
  memcpy(&u, &h, sizeof(u));
  return u;
}

// v * 2^-e split into FP16 hi and lo pairs (re, im each)
__device__ __forceinline__ void tc_split(float2 v, float sc, __half2 &hi, __half2 &lo) {
  const float2 xs = pmul(v, splat(sc));
  hi = __float22half2_rn(xs);
  const float2 back = __half22float2(hi);
  lo = __float22half2_rn(psub(xs, back));
}

// The real form of the 32-point DFT matrix (conjugated for the inverse) as
// the B operand, hi and lo halves: row n = 2 k + a, column 2 t + b.
// roots: the pass's 1024 roots exp(-2 pi i m / 1024).
template <int SIGN>
__device__ __forceinline__ void tc_build_dft32(const float2 *roots, unsigned char *Bm, int tid) {
  for (int e = tid; e < 64 * 64; e += NT) {
    const int n = e >> 6, kk = e & 63;
    const int k = n >> 1, a = n & 1, t = kk >> 1, b = kk & 1;
    float2 w = __ldg(roots + 32 * ((t * k) & 31));
    if (SIGN > 0) w.y = -w.y;
    const float val = a == 0 ? (b == 0 ? w.x : -w.y) : (b == 0 ? w.y : w.x);
    const __half hi = __float2half_rn(val);
    const __half lo = __float2half_rn(val - __half2float(hi));
    *reinterpret_cast<__half *>(Bm + tc::sw128_offset(n, kk)) = hi;
    *reinterpret_cast<__half *>(Bm + TC_B_BYTES / 2 + tc::sw128_offset(n, kk)) = lo;
  }
}

// D = Al Bh + Ah Bl + Ah Bh over K = 64 (four slices of 16), then a commit
// to the barrier; one thread issues it.  The small cross terms go first: the
// accumulator rounds after every MMA, and this way only the last four
// additions round at the full magnitude of the result.
__device__ __forceinline__ void tc_issue(uint32_t taddr, uint32_t a_sa, uint32_t b_sa, uint32_t bar) {
  constexpr uint32_t ID = tc::idesc_f16_f32(128, 64);
  constexpr uint32_t LO_A = 16384, LO_B = (uint32_t)(TC_B_BYTES / 2);
  static_assert(TC_A_BYTES >= 2 * LO_A, "two A operands");
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
    tc::mma_f16(taddr, tc::desc_sw128(a_sa + LO_A + 32 * kk), tc::desc_sw128(b_sa + 32 * kk), ID, kk > 0);
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
    tc::mma_f16(taddr, tc::desc_sw128(a_sa + 32 * kk), tc::desc_sw128(b_sa + LO_B + 32 * kk), ID, 1);
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
    tc::mma_f16(taddr, tc::desc_sw128(a_sa + 32 * kk), tc::desc_sw128(b_sa + 32 * kk), ID, 1);
  tc::mma_commit(bar);
}

// Product 1's operand from the staging buffer (line l, value t at
// l * ld + swz(t)): thread pairs own rows (l, t1), each thread 16 of the 32
// values x[t1 + 32 t2]; lines >= nlines are zero.  Ends with the operands
// visible to the tensor cores and a barrier.
__device__ __forceinline__ void tc_operand1(const float2 *stg, int ld, unsigned char *A, int *exp1, int nlines,
                                            int tid) {
  const int r = tid >> 1, h = tid & 1;
  const int l = r >> 5, t1 = r & 31;
  float2 x[16];
  uint32_t mx = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    x[i] = l < nlines ? stg[l * ld + swz<float, 1024>(t1 + 32 * (16 * h + i))] : make_float2(0.f, 0.f);
    mx = max(mx, max(__float_as_uint(x[i].x) & 0x7FFFFFFFu, __float_as_uint(x[i].y) & 0x7FFFFFFFu));
  }
  mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, 1));
  const int e = tc_row_exp(mx);
  const float sc = tc_pow2(-e);
  const uint32_t rowb = (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t hb[4], lb[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      __half2 hv, lv;
      tc_split(x[4 * j + q], sc, hv, lv);
      hb[q] = tc_bits(hv);
      lb[q] = tc_bits(lv);
    }
    const uint32_t off = rowb + ((uint32_t)((4 * h + j) ^ (r & 7)) << 4);
    *reinterpret_cast<uint4 *>(A + off) = make_uint4(hb[0], hb[1], hb[2], hb[3]);
    *reinterpret_cast<uint4 *>(A + 16384 + off) = make_uint4(lb[0], lb[1], lb[2], lb[3]);
  }
  if (h == 0) exp1[r] = e;
  tc::fence_proxy_async();
  __syncthreads();
}

// Waits for product 1, applies the row scale and the twiddle, builds product
// 2's operand (rows (l, k2), columns t1), waits for product 2 and writes the
// lines, scaled back, in natural order (value k at l * ld + swz(k)) over the
// A area.  Warp w reads tensor-memory lanes 32 (w % 4) .. + 31 (line w % 4,
// t1 or k2 = lane) and the column half w / 4.  Product 2's operand has one
// scale per line: |Z[t1, k2]| <= 32 max_t2 |x[t1 + 32 t2]| < 2^(20 + e1[t1]),
// so the exponent e2 = max_t1 e1[t1] + 5 keeps every value of the line below
// 2^15 (and a power-of-two scale leaves the hi + lo split's relative
// accuracy as it is).  Ends with a barrier.
template <int SIGN>
__device__ __forceinline__ const float2 *tc_finish(unsigned char *A, uint32_t a_sa, uint32_t b_sa, const int *exp1,
                                                   const float2 *roots, int ld, uint32_t taddr, uint32_t bar,
                                                   uint32_t &phase, int &fail, int tid) {
  const int w = tid >> 5, lane = tid & 31, l = w & 3, hf = w >> 2;
  const uint32_t lane_addr = taddr + ((uint32_t)(32 * l) << 16) + (uint32_t)(32 * hf);
  bool ok = !fail && tc::mbar_wait(bar, phase & 1u, TC_WAIT_LIMIT);
  ++phase;
  tc::fence_after_sync();
  float d[32];
  if (ok) {
    tc::tmem_ld32(lane_addr, d);
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) d[i] = 0.f;
  }
  const int e1 = exp1[32 * l + lane];
  const int e2 = min(__reduce_max_sync(0xFFFFFFFFu, e1) + 5, 126);
  {
    // back to the line's values (2^e1), then into product 2's range (2^-e2): two exact scalings, since
    // 2^(e1 - e2) alone may lie below FP32's normal range
    const float s1 = tc_pow2(e1), s2i = tc_pow2(-e2);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int k2 = 16 * hf + j;
      float2 wt = __ldg(roots + lane * k2);
      if (SIGN > 0) wt.y = -wt.y;
      const float2 z = cmul(pmul(pmul(make_float2(d[2 * j], d[2 * j + 1]), splat(s1)), splat(s2i)), wt);
      const __half2 hv = __float22half2_rn(z);
      const __half2 lv = __float22half2_rn(psub(z, __half22float2(hv)));
      const int r2 = 32 * l + k2;
      const uint32_t off = (uint32_t)(r2 >> 3) * 1024u + (uint32_t)(r2 & 7) * 128u +
                           ((uint32_t)((lane >> 2) ^ (r2 & 7)) << 4) + (uint32_t)(lane & 3) * 4u;
      *reinterpret_cast<__half2 *>(A + off) = hv;
      *reinterpret_cast<__half2 *>(A + 16384 + off) = lv;
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  if (tid == 0 && ok) {
    tc::fence_after_sync();
    tc_issue(taddr, a_sa, b_sa, bar);
  }
  ok = ok && tc::mbar_wait(bar, phase & 1u, TC_WAIT_LIMIT);
  ++phase;
  tc::fence_after_sync();
  if (ok) {
    tc::tmem_ld32(lane_addr, d);
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) d[i] = 0.f;
  }
  float2 *res = reinterpret_cast<float2 *>(A);
  const float s2 = tc_pow2(e2);
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int k = lane + 32 * (16 * hf + j);
    res[l * ld + swz<float, 1024>(k)] = pmul(make_float2(d[2 * j], d[2 * j + 1]), splat(s2));
  }
  if (!ok) fail = 1;
  tc::fence_before_sync();
  __syncthreads();
  return res;
}

// NF > 0: length NF with a compile-time schedule; NF == 0: any length.
// TC: the 1024-point FP32 pass with its DFT on the tensor cores (see above).
// The pass as block `bid` of `nblk` persistent blocks (a launch's grid, or a
// job's share of a grouped launch).
template <typename T, int SIGN, int NF, bool TC = false>
__device__ __forceinline__ void pass_body(const dmg_fft_pass &p, const dmg_fft_batch &bt, const int64_t bid,
                                          const int64_t nblk) {
  static_assert(!TC || (std::is_same<T, float>::value && NF == 1024), "tensor-core stages: 1024-point FP32");
  constexpr bool FIXED = NF > 0;
  // power-of-two lengths: buffers at compile-time offsets (staging, A, B, twiddle tables)
  constexpr bool POW2 = pow2_length(NF);
  constexpr size_t PSTRIDE = POW2 ? pow2_stride(sizeof(C2<T>), NF) : 0;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ PassConsts kc;
  const int tid = threadIdx.x;
  const int64_t ntiles_all = p.ntiles * bt.count;
  if (tid == 0) {
    const SmemLayout S = smem_layout<T>(p, FIXED, TC);
    kc.ld = S.ld;
    kc.M1 = p.M1;
    kc.buf_a = (unsigned)S.buf_a;
    kc.buf_b = (unsigned)S.buf_b;
    kc.roots_off = (unsigned)S.roots_off;
    kc.contrib_off = (unsigned)S.contrib_off;
    kc.spos_off = (unsigned)S.spos_off;
    kc.t0_off = (unsigned)S.t0_off;
    kc.t0_in = S.has_t0_in;
    kc.t0_out = S.has_t0_out;
    kc.t0base_in = kc.t0_in ? __ldg(p.in.tab[p.kdim[0]]) : 0;
    kc.t0base_out = kc.t0_out ? __ldg(p.out.tab[p.kdim[0]]) : 0;
    // the transform axis's dimension and step (separable sides)
    kc.d0 = p.kdim[0];
    kc.mult0 = p.kisz[0] ? p.A[p.kdim[0]] : 1;
    // the transformed dimension and, for its twiddle, which vector axes carry its y
    const int td = p.t >> 1;
    kc.td = td;
    kc.v1_ytd = p.kdim[1] == td && !p.kisz[1];
    kc.v2_ytd = p.kdim[2] == td && !p.kisz[2];
    kc.tw_kmaj = (p.store_order[0] == 1 && kc.v1_ytd) || (p.store_order[0] == 2 && kc.v2_ytd);
    kc.in64 = p.in_fp64 != 0;
    kc.out64 = p.out_fp64 != 0;
    // this block's first two tiles, and the digits of the stride between its tiles
    const int nd = 3 + p.nbatch;
    kc.ndig = nd;
    kc.rad[0] = p.nt1;
    kc.rad[1] = p.nt2;
    for (int b = 0; b < p.nbatch; ++b) kc.rad[2 + b] = p.blen[b];
    kc.rad[2 + p.nbatch] = bt.count;
    tile_digits(kc.rad, nd, bid, kc.dig);
    tile_digits(kc.rad, nd, nblk, kc.inc);
    if (bid < ntiles_all) {
      tile_state_digits<T>(p, bt, kc.dig, kc.ts[0]);
      digits_add(kc.dig, kc.inc, kc.rad, nd);
      if (bid + nblk < ntiles_all) tile_state_digits<T>(p, bt, kc.dig, kc.ts[1]);
    }
    if constexpr (TC) {
      kc.tc_fail = 0;
      tc::mbar_init(tc::smem_u32(&kc.tc_bar), 1);
    }
  }
  // tensor-core form: the area after the staging buffer, 1024-byte aligned; 64 tensor-memory columns (one
  // 128 x 64 FP32 accumulator)
  unsigned char *tcA = nullptr, *tcB = nullptr;
  int *tcE1 = nullptr;
  uint32_t tc_phase = 0;
  if constexpr (TC) {
    const uint32_t at = tc::smem_u32(sm) + (uint32_t)PSTRIDE;
    tcA = sm + PSTRIDE + ((1024u - (at & 1023u)) & 1023u);
    tcB = tcA + TC_A_BYTES;
    tcE1 = reinterpret_cast<int *>(tcB + TC_B_BYTES);
    if (tid < 32) tc::tmem_alloc(tc::smem_u32(&kc.tc_taddr), 64);
    tc_build_dft32<SIGN>(reinterpret_cast<const float2 *>(p.roots), tcB, tid);
    tc::fence_before_sync();
  }
  __syncthreads();
  if constexpr (TC) tc::fence_after_sync();
  // separable address parts: gather side, two scatter-side areas (tiles alternate)
  int64_t *const parts_in = reinterpret_cast<int64_t *>(sm + kc.contrib_off);
  int64_t *const parts_out0 = parts_in + parts_len(p);
  {
    const int n = FIXED ? NF : p.n;
    if constexpr (POW2) {
      if (!global_twiddles(NF, sizeof(C2<T>)))
        pow2_twiddles<T, SIGN, NF>(reinterpret_cast<const C2<T> *>(p.roots), reinterpret_cast<C2<T> *>(sm + 3 * PSTRIDE),
                                 tid);
    } else if constexpr (FIXED && DMG_FFT_SMEM_ROOTS) {
      C2<T> *sr = reinterpret_cast<C2<T> *>(sm + kc.roots_off);
      const C2<T> *gr = reinterpret_cast<const C2<T> *>(p.roots);
      for (int i = tid; i < n; i += NT) sr[i] = gr[i];
    }
    {
      // buffer position of transform coordinate i on each side: the line
      // position of slot i where that side is in slot order, swizzled
      int16_t *spos = reinterpret_cast<int16_t *>(sm + kc.spos_off);
      for (int i = tid; i < n; i += NT) {
        const int slot = (p.perm_in || p.perm_out) ? i / p.perm_a + p.perm_b * (i % p.perm_a) : i;
        spos[i] = (int16_t)swz<T, NF>(p.perm_in ? slot : i);
        spos[n + i] = (int16_t)swz<T, NF>(p.perm_out ? slot : i);
      }
      // transform-axis address offsets (every tile's: no batch sub-axis in that dimension)
      int32_t *t0 = reinterpret_cast<int32_t *>(sm + kc.t0_off);
      const int d0 = p.kdim[0], m0 = kc.mult0;
      if (kc.t0_in)
        for (int i = tid; i < n; i += NT) t0[i] = (int32_t)(__ldg(p.in.tab[d0] + i * m0) - kc.t0base_in);
      int32_t *t0o = t0 + (kc.t0_in ? n : 0);
      if (kc.t0_out)
        for (int i = tid; i < n; i += NT) t0o[i] = (int32_t)(__ldg(p.out.tab[d0] + i * m0) - kc.t0base_out);
    }
    if (bid < ntiles_all) {
      const TileState &st = kc.ts[0];
      if (p.sep_in || p.semi_in)
        sep_parts_async(p.in, p, st.yb, st.zb, st.lim1, st.lim2, tid, parts_in, p.semi_in, p.pair_in);
      if (p.sep_out || p.semi_out)
        sep_parts_async(p.out, p, st.yb, st.zb, st.lim1, st.lim2, tid, parts_out0, p.semi_out, p.pair_out);
      copy_async_commit();
    }
  }
  copy_async_wait_all();
  __syncthreads();
  if (bid < ntiles_all) gather_async<T, NF>(p, kc, kc.ts[0], sm, parts_in, bt, tid);

  int it = 0;
  for (int64_t tile = bid; tile < ntiles_all; tile += nblk, ++it) {
    const int64_t next = tile + nblk;
    const int cur = it % 3, nxt = (it + 1) % 3;  // state slots of this tile and the next
    // ---- the tile's values are in the staging buffer ----
    copy_async_wait_all();
    __syncthreads();
    // the state of the tile after the next (read after later barriers)
    if (tid == 0 && next + nblk < ntiles_all) {
      digits_add(kc.dig, kc.inc, kc.rad, kc.ndig);
      tile_state_digits<T>(p, bt, kc.dig, kc.ts[(it + 2) % 3]);
    }
    // the next tile's address parts start loading: gather side, and the
    // scatter side into the area this tile's scatter does not read
    if (next < ntiles_all) {
      const TileState &sn = kc.ts[nxt];
      if (p.sep_in || p.semi_in)
        sep_parts_async(p.in, p, sn.yb, sn.zb, sn.lim1, sn.lim2, tid, parts_in, p.semi_in, p.pair_in);
      if (p.sep_out || p.semi_out)
        sep_parts_async(p.out, p, sn.yb, sn.zb, sn.lim1, sn.lim2, tid, parts_out0 + ((it + 1) & 1) * parts_len(p),
                        p.semi_out, p.pair_out);
      copy_async_commit();
    }
    // convert a complex128 input to double-float, apply the inverse split
    // twiddle (the compile-time-length kernels convert inside their first
    // stage unless a twiddle is due here as well)
    const bool conv_first = FIXED && std::is_same<T, df>::value && kc.in64 && p.twiddle != 2;
    if ((std::is_same<T, df>::value && kc.in64 && !conv_first) || p.twiddle == 2) {
      const int n = FIXED ? NF : p.n;
      const int ld = kc.ld, M1 = kc.M1;
      const TileState &st = kc.ts[cur];
      const int lim1 = st.lim1, lim2 = st.lim2;
      const int sexp = st.sexp;
      const C2<T> *twt = reinterpret_cast<const C2<T> *>(p.twy[kc.td]);  // lanes step along k
      C2<T> *stg = reinterpret_cast<C2<T> *>(sm);
      const int total = n * M1 * p.M2;
      for (int e = tid; e < total; e += NT) {
        const int l = e / n, i = e - (e / n) * n;
        const int c1 = l % M1, c2 = l / M1;
        if (c1 >= lim1 || c2 >= lim2) continue;
        const int sp = l * ld + swz<T, NF>(i);
        C2<T> v;
        if constexpr (std::is_same<T, df>::value) {
          if (kc.in64) {
            const double2 d = *reinterpret_cast<const double2 *>(stg + sp);
            const df re = to_df(d.x, sexp), im = to_df(d.y, sexp);
            v = dfc{make_float2(re.h, im.h), make_float2(re.l, im.l)};
          } else {
            v = stg[sp];
          }
        } else {
          v = stg[sp];
        }
        if (p.twiddle == 2) {
          const int y = st.ytw + (kc.v1_ytd ? c1 : 0) + (kc.v2_ytd ? c2 : 0);
          if (y && i) v = mul<T>(v, conj<T>(twt[y * n + i]));
        }
        stg[sp] = v;
      }
      __syncthreads();
    }

    // ---- first Stockham stage: staging buffer -> A; then the next tile's copies start ----
    {
      const int ld = kc.ld;
      const int nlines = p.M1 * p.M2;
      const C2<T> *stg = reinterpret_cast<const C2<T> *>(sm);
      C2<T> *bufA = reinterpret_cast<C2<T> *>(sm + (POW2 ? PSTRIDE : kc.buf_a));
      if constexpr (TC) {
        (void)bufA;
        tc_operand1(reinterpret_cast<const float2 *>(stg), ld, tcA, tcE1, nlines, tid);
        if (tid == 0 && !kc.tc_fail) {
          tc::fence_after_sync();
          tc_issue(kc.tc_taddr, tc::smem_u32(tcA), tc::smem_u32(tcB), tc::smem_u32(&kc.tc_bar));
        }
      } else if constexpr (POW2) {
        stage_pow2<T, SIGN, NF, 1>(stg, bufA, reinterpret_cast<const C2<T> *>(sm + 3 * PSTRIDE), nlines, ld, tid,
                                   conv_first, kc.ts[cur].sexp);
      } else if constexpr (FIXED) {
        stage_fixed<T, SIGN, NF, 1>(stg, bufA, reinterpret_cast<const C2<T> *>(p.roots), nlines, ld, tid, conv_first,
                                    kc.ts[cur].sexp);
      } else {
        stage_runtime<T, SIGN>(p, 0, 1, stg, bufA, reinterpret_cast<const C2<T> *>(p.roots), nlines, ld, tid);
      }
    }
    if (next < ntiles_all) {
      copy_async_wait_all();  // the next tile's address parts
      __syncthreads();
      gather_async<T, NF>(p, kc, kc.ts[nxt], sm, parts_in, bt, tid);
    }

    // ---- the other stages: between A and B ----
    const C2<T> *res;
    {
      const int ld = kc.ld;
      const int nlines = p.M1 * p.M2;
      C2<T> *bufA = reinterpret_cast<C2<T> *>(sm + (POW2 ? PSTRIDE : kc.buf_a));
      C2<T> *bufB = reinterpret_cast<C2<T> *>(sm + (POW2 ? 2 * PSTRIDE : kc.buf_b));
      if constexpr (TC) {
        (void)bufA;
        (void)bufB;
        res = reinterpret_cast<const C2<T> *>(tc_finish<SIGN>(tcA, tc::smem_u32(tcA), tc::smem_u32(tcB), tcE1,
                                                               reinterpret_cast<const float2 *>(p.roots), ld,
                                                               kc.tc_taddr, tc::smem_u32(&kc.tc_bar), tc_phase,
                                                               kc.tc_fail, tid));
      } else if constexpr (FIXED) {
        const C2<T> *rts = POW2 ? (global_twiddles(NF, sizeof(C2<T>)) ? reinterpret_cast<const C2<T> *>(p.roots)
                                                                      : reinterpret_cast<const C2<T> *>(sm + 3 * PSTRIDE))
                           : DMG_FFT_SMEM_ROOTS ? reinterpret_cast<const C2<T> *>(sm + kc.roots_off)
                                                : reinterpret_cast<const C2<T> *>(p.roots);
        res = stages_fixed<T, SIGN, NF, fixed_radix(NF, 1)>(bufA, bufB, bufA, rts, nlines, ld, tid,
                                                            reinterpret_cast<const C2<T> *>(p.roots));
      } else {
        const C2<T> *groots = reinterpret_cast<const C2<T> *>(p.roots);
        C2<T> *in = bufA, *out = bufB;
        int Lp = p.fac[0];
        for (int f = 1; f < p.nfac; ++f) {
          stage_runtime<T, SIGN>(p, f, Lp, in, out, groots, nlines, ld, tid);
          Lp *= p.fac[f];
          C2<T> *t = in;
          in = out;
          out = t;
        }
        res = in;
      }
    }

    // ---- scatter to the output layout: every read and address, then every store ----
    {
      const int n = FIXED ? NF : p.n;
      const int ld = kc.ld, M1 = kc.M1;
      const TileState &st = kc.ts[cur];
      int yb[DMG_FFT_MAXDIM], zb[DMG_FFT_MAXDIM];
#pragma unroll
      for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
        yb[d] = st.yb[d];
        zb[d] = st.zb[d];
      }
      const int lim1 = st.lim1, lim2 = st.lim2;
      const int total = n * lim1 * lim2;
      const int d0 = kc.d0, mult0 = kc.mult0;
      const int64_t *pout = parts_out0 + (it & 1) * parts_len(p);
      const int16_t *spos = reinterpret_cast<const int16_t *>(sm + kc.spos_off) + n;
      const int64_t *tab0 = p.out.tab[d0] + (yb[d0] + p.A[d0] * zb[d0]);
      const int64_t out0 = (p.sep_out || p.semi_out) ? sep_base(p.out, p, pout) : 0;
      const bool out64 = kc.out64;
      const int sexp = st.sexp;
      void *dst = bt.dst[st.job];
      // split twiddle of output (y, k = c0): entry k A + y or y n + k, whichever the walk's lanes step along
      // (the table's order and A are re-read where a twiddle is due, so that no register holds them
      // through the walks)
      const C2<T> *twt = reinterpret_cast<const C2<T> *>(kc.tw_kmaj ? p.twk[kc.td] : p.twy[kc.td]);
      const bool tw1 = p.twiddle == 1;
      const int ytw = st.ytw, v1y = kc.v1_ytd, v2y = kc.v2_ytd;
      bool done = p.sep_out &&
                  sep_walk_any<T, NF>(p.store_order, n, lim1, lim2, M1, ld, tab0, mult0, out0, pout, spos, tid,
                                      [&](int64_t ad, int sp, int c0, int c1, int c2) {
                                    C2<T> x = res[sp];
                                    if (tw1) {
                                      const int y = ytw + (v1y ? c1 : 0) + (v2y ? c2 : 0);
                                      if (y && c0)
                                        x = mul<T>(x, twt[kc.tw_kmaj ? c0 * p.A[kc.td] + y : y * n + c0]);
                                    }
                                    store_elem<T>(dst, ad, x, out64, sexp);
                                  },
                                  kc.t0_out ? reinterpret_cast<const int32_t *>(sm + kc.t0_off) + (kc.t0_in ? n : 0)
                                            : nullptr,
                                  kc.t0base_out);
      const SharedDim sdo = p.semi_out ? shared_dim(p.out, p, yb, zb) : SharedDim{};
      TileWalk w(tid, p.store_pos, n, lim1, lim2);
      for (int e0 = 0; !done && e0 < total; e0 += NT * EPT) {
        int64_t ad[EPT];
        C2<T> v[EPT];
        bool ok[EPT];
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          ok[u] = e0 + tid + u * NT < total;
          if (ok[u]) {
            const int c0 = w.coord(p.store_pos[0]), c1 = w.coord(p.store_pos[1]), c2 = w.coord(p.store_pos[2]);
            C2<T> x = res[(c1 + M1 * c2) * ld + spos[c0]];
            if (tw1) {
              const int y = ytw + (v1y ? c1 : 0) + (v2y ? c2 : 0);
              if (y && c0) x = mul<T>(x, twt[kc.tw_kmaj ? c0 * p.A[kc.td] + y : y * n + c0]);
            }
            v[u] = x;
            if (p.sep_out) {
              ad[u] = out0 + __ldg(tab0 + c0 * mult0) + pout[1 + c1] + pout[1 + M1 + c2];
            } else if (p.semi_out) {
              ad[u] = out0 + shared_dim_part(sdo, p, c0, c1, c2) + (sdo.t_paired ? 0 : __ldg(tab0 + c0 * mult0)) +
                      pout[1 + c1] + pout[1 + M1 + c2];
            } else {
              int xg[DMG_FFT_MAXDIM];
              element_x(p, yb, zb, c0, c1, c2, xg);
              ad[u] = layout_addr(p.out, p.ndim, xg);
            }
          }
          w.next();
        }
#pragma unroll
        for (int u = 0; u < EPT; ++u)
          if (ok[u]) store_elem<T>(dst, ad[u], v[u], out64, sexp);
      }
    }
    __syncthreads();
  }
  if constexpr (TC) {
    // every tensor-memory read is done (each tile ends with a barrier): give the columns back
    tc::fence_after_sync();
    if (tid < 32) tc::tmem_dealloc(kc.tc_taddr, 64);
    if (tid == 0 && kc.tc_fail && p.status) atomicExch(p.status, 1);
  }
}

template <typename T, int SIGN, int NF, bool TC = false>
__global__ void __launch_bounds__(NT, MINB) fft_pass_kernel(const dmg_fft_pass p, const dmg_fft_batch bt) {
  pass_body<T, SIGN, NF, TC>(p, bt, blockIdx.x, gridDim.x);
}

// Passes of several plans (any lengths, with the runtime-length stages) in
// one launch: job j owns blocks first_block .. first_block + nblocks - 1 and
// runs its pass with them as its own grid.
template <typename T, int SIGN>
__global__ void __launch_bounds__(NT, MINB) fft_pass_group_kernel(const __grid_constant__ dmg_fft_group g) {
  int j = 0;
  while (j + 1 < g.count && (int64_t)blockIdx.x >= g.job[j + 1].first_block) ++j;
  const dmg_fft_group_job &job = g.job[j];
  pass_body<T, SIGN, 0, false>(job.p, job.bt, (int64_t)blockIdx.x - job.first_block, job.nblocks);
}

// One grouped launch: every job gets blocks in proportion to its tiles (at
// least one, at most its tile count) out of the blocks that fill the SMs at
// the largest job's shared memory.
template <typename T, int SIGN>
int launch_group(dmg_fft_group g, cudaStream_t s) {
  size_t smem = 0;
  int64_t tiles = 0;
  for (int j = 0; j < g.count; ++j) {
    const size_t sj = smem_layout<T>(g.job[j].p, false).total;
    smem = sj > smem ? sj : smem;
    tiles += g.job[j].p.ntiles * g.job[j].bt.count;
  }
  auto k = fft_pass_group_kernel<T, SIGN>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "grouped fft pass smem %zu: %s", smem, cudaGetErrorString(e));
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, smem);
  if (per_sm < 1) return dmg_error(DMG_ERR_UNSUPPORTED, "grouped fft pass does not fit on an SM (smem %zu)", smem);
  const int64_t budget = (int64_t)nsm * per_sm;
  int64_t first = 0;
  for (int j = 0; j < g.count; ++j) {
    const int64_t tj = g.job[j].p.ntiles * g.job[j].bt.count;
    int64_t nb = tiles > 0 ? (budget * tj + tiles - 1) / tiles : 1;
    if (nb > tj) nb = tj;
    if (nb < 1) nb = 1;
    g.job[j].first_block = first;
    g.job[j].nblocks = nb;
    first += nb;
  }
  k<<<(unsigned)first, NT, smem, s>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "grouped fft pass launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

template <typename T, int SIGN, int NF, bool TC = false>
int launch_k(const dmg_fft_pass &p, const dmg_fft_batch &bt, cudaStream_t s) {
  const size_t smem = smem_layout<T>(p, NF > 0, TC).total;
  auto k = fft_pass_kernel<T, SIGN, NF, TC>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "fft pass smem %zu: %s", smem, cudaGetErrorString(e));
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, smem);
  if (per_sm < 1) return dmg_error(DMG_ERR_UNSUPPORTED, "fft pass does not fit on an SM (smem %zu)", smem);
  if constexpr (TC) {
    // the occupancy query answers one block per SM for kernels that allocate tensor memory; two blocks of
    // this kernel fit (64 of the SM's 512 tensor-memory columns each, and shared memory and registers for
    // two), and run together
    cudaFuncAttributes fa;
    int smem_sm = 0, reserve = 0;
    if (cudaFuncGetAttributes(&fa, k) == cudaSuccess &&
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess) {
      const size_t per_block = smem + fa.sharedSizeBytes + (size_t)reserve;
      const int fit = (int)((size_t)smem_sm / per_block);
      per_sm = max(per_sm, min(fit, MINB));
    }
  }
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > p.ntiles * bt.count) grid = p.ntiles * bt.count;
  if (grid < 1) return DMG_OK;
  k<<<(unsigned)grid, NT, smem, s>>>(p, bt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "fft pass launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

// The compile-time lengths fall in two groups, each compiled in its own
// translation unit per arithmetic and direction so that the build runs them
// in parallel: the powers of two from 8 to 2048, and the other lengths with
// the runtime-length kernel.
__host__ __device__ constexpr bool pow2_group(int n) { return n >= 8 && n <= 2048 && (n & (n - 1)) == 0; }

template <typename T, int SIGN>
int launch_pow2_group(const dmg_fft_pass &p, const dmg_fft_batch &bt, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (p.n) {
    case 8: return launch_k<T, SIGN, 8>(p, bt, s);
    case 16: return launch_k<T, SIGN, 16>(p, bt, s);
    case 32: return launch_k<T, SIGN, 32>(p, bt, s);
    case 64: return launch_k<T, SIGN, 64>(p, bt, s);
    case 128: return launch_k<T, SIGN, 128>(p, bt, s);
    case 256: return launch_k<T, SIGN, 256>(p, bt, s);
    case 512: return launch_k<T, SIGN, 512>(p, bt, s);
    case 1024: return launch_k<T, SIGN, 1024>(p, bt, s);
    case 2048: return launch_k<T, SIGN, 2048>(p, bt, s);
    default: return dmg_error(DMG_ERR_ARG, "fft pass: length %d is not a power of two from 8 to 2048", p.n);
  }
}

template <typename T, int SIGN>
int launch_other_group(const dmg_fft_pass &p, const dmg_fft_batch &bt, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p.radix_runtime) return launch_k<T, SIGN, 0>(p, bt, s);
  switch (p.n) {
    case 48: return launch_k<T, SIGN, 48>(p, bt, s);
    case 96: return launch_k<T, SIGN, 96>(p, bt, s);
    case 120: return launch_k<T, SIGN, 120>(p, bt, s);
    case 160: return launch_k<T, SIGN, 160>(p, bt, s);
    case 192: return launch_k<T, SIGN, 192>(p, bt, s);
    case 240: return launch_k<T, SIGN, 240>(p, bt, s);
    case 320: return launch_k<T, SIGN, 320>(p, bt, s);
    case 384: return launch_k<T, SIGN, 384>(p, bt, s);
    case 480: return launch_k<T, SIGN, 480>(p, bt, s);
    default: return launch_k<T, SIGN, 0>(p, bt, s);
  }
}

// Checks of a pass launch over a batch of jobs in arithmetic T, before the
// launch in the direction p.sign goes to the translation unit of its group.
template <typename T>
int check_batch(const dmg_fft_pass &p, const dmg_fft_batch &bt) {
  if (bt.count < 1 || bt.count > DMG_FFT_MAXBATCH)
    return dmg_error(DMG_ERR_ARG, "fft pass: batch of %d jobs (1 to %d)", bt.count, DMG_FFT_MAXBATCH);
  for (int j = 0; j < bt.count; ++j) {
    // the gather copies whole values asynchronously: both arrays need their natural alignment
    if ((reinterpret_cast<uintptr_t>(bt.src[j]) | reinterpret_cast<uintptr_t>(bt.dst[j])) % sizeof(C2<T>) != 0)
      return dmg_error(DMG_ERR_ARG, "fft pass: buffers must be aligned to %zu bytes", sizeof(C2<T>));
    if (std::is_same<T, df>::value && (p.in_fp64 || p.out_fp64) && !bt.scale_exp[j])
      return dmg_error(DMG_ERR_ARG, "double-float pass without a scale exponent");
  }
  return DMG_OK;
}

template <typename T>
size_t pass_smem(const dmg_fft_pass &p) {
  return smem_layout<T>(p, use_fixed<T>(p)).total;
}

}  // namespace
