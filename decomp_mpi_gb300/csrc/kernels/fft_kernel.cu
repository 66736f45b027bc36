// Entry points of the FFT passes (dispatch by arithmetic) and the exponent
// pre-pass of double-float runs.  The passes are the execution of
// runSplitPlan (reference split_fft.c:622-744).
#include "fft_pass.cuh"

// per-arithmetic launchers (fft_pass_f64.cu, fft_pass_f32.cu, fft_pass_df.cu)
size_t dmg_fft_pass_smem_f64(const dmg_fft_pass *p);
size_t dmg_fft_pass_smem_f32(const dmg_fft_pass *p);
size_t dmg_fft_pass_smem_df(const dmg_fft_pass *p);
size_t dmg_fft_pass_smem_tc(const dmg_fft_pass *p);
int dmg_fft_pass_launch_tc(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_launch_f64(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_launch_f32(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_launch_df(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
// grouped runtime-length passes (fft_pass_*_mixed.cu)
int dmg_fft_pass_f64_fwd_group(const dmg_fft_group *g, void *stream);
int dmg_fft_pass_f64_inv_group(const dmg_fft_group *g, void *stream);
int dmg_fft_pass_f32_fwd_group(const dmg_fft_group *g, void *stream);
int dmg_fft_pass_f32_inv_group(const dmg_fft_group *g, void *stream);
int dmg_fft_pass_df_fwd_group(const dmg_fft_group *g, void *stream);
int dmg_fft_pass_df_inv_group(const dmg_fft_group *g, void *stream);

namespace {

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

// The same over a separable layout, a block per row of the last dimension
// at a time: the row's address part is formed once, the threads run along
// the row (contiguous in the usual layouts).
__global__ void __launch_bounds__(256) maxexp_rows_kernel(const dmg_fft_layout lay, int ndim, int L0, int L1, int L2,
                                                          const double2 *__restrict__ src, int32_t *out) {
  const int64_t rows = (int64_t)L0 * L1;
  int best = 0;
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const int x0 = (int)(r / L1), x1 = (int)(r - (int64_t)x0 * L1);
    const int64_t base = lay.base + __ldg(lay.tab[0] + x0) + (ndim > 1 ? __ldg(lay.tab[1] + x1) : 0);
    for (int x2 = threadIdx.x; x2 < L2; x2 += blockDim.x) {
      const double2 v = src[base + (ndim > 2 ? __ldg(lay.tab[2] + x2) : 0)];
      const int ea = (int)((__double_as_longlong(v.x) >> 52) & 0x7FF);
      const int eb = (int)((__double_as_longlong(v.y) >> 52) & 0x7FF);
      best = max(best, max(ea, eb));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(out, best);
}

}  // namespace

extern "C" size_t dmg_fft_pass_smem(const dmg_fft_pass *p, int dtype) {
  return dtype == 0 ? dmg_fft_pass_smem_f64(p)
                    : dtype == 1 ? dmg_fft_pass_smem_f32(p)
                                 : dtype == 2 ? dmg_fft_pass_smem_df(p) : dmg_fft_pass_smem_tc(p);
}

extern "C" int dmg_fft_pass_launch_batch(const dmg_fft_pass *p, int dtype, const dmg_fft_batch *b, void *stream) {
  const int64_t most = p->wide ? 2 * DMG_FFT_TILE_MAX : DMG_FFT_TILE_MAX;
  if ((int64_t)p->M1 * p->M2 * p->n > most)
    return dmg_error(DMG_ERR_ARG, "fft tile %d exceeds %lld", p->M1 * p->M2 * p->n, (long long)most);
  if (p->wide && (dtype == 0 || (dtype == 3 && p->n == 1024) || p->radix_runtime || p->n < 8 || p->n > 2048 ||
                  (p->n & (p->n - 1))))
    return dmg_error(DMG_ERR_ARG, "fft pass: wide tiles for length %d in arithmetic %d", p->n, dtype);
  if ((p->perm_in || p->perm_out) && (p->perm_a < 1 || p->perm_b < 1 || (int64_t)p->perm_a * p->perm_b != p->n))
    return dmg_error(DMG_ERR_ARG, "fft slot order %d x %d does not match length %d", p->perm_a, p->perm_b, p->n);
  switch (dtype) {
    case 0: return dmg_fft_pass_launch_f64(p, b, stream);
    case 1: return dmg_fft_pass_launch_f32(p, b, stream);
    case 2: return dmg_fft_pass_launch_df(p, b, stream);
    case 3: return dmg_fft_pass_launch_tc(p, b, stream);
    default: return dmg_error(DMG_ERR_ARG, "fft dtype %d", dtype);
  }
}

extern "C" int dmg_fft_pass_launch_group(const dmg_fft_group *g, int dtype, void *stream) {
  if (g->count < 1 || g->count > DMG_FFT_MAXGROUP)
    return dmg_error(DMG_ERR_ARG, "grouped fft pass: %d passes (1 to %d)", g->count, DMG_FFT_MAXGROUP);
  const int sign = g->job[0].p.sign;
  for (int j = 0; j < g->count; ++j) {
    const dmg_fft_pass &p = g->job[j].p;
    if (!p.radix_runtime || p.wide || p.sign != sign)
      return dmg_error(DMG_ERR_ARG, "grouped fft pass %d: needs runtime stages, plain tiles and one direction", j);
    if ((int64_t)p.M1 * p.M2 * p.n > DMG_FFT_TILE_MAX)
      return dmg_error(DMG_ERR_ARG, "fft tile %d exceeds %d", p.M1 * p.M2 * p.n, DMG_FFT_TILE_MAX);
    if ((p.perm_in || p.perm_out) && (p.perm_a < 1 || p.perm_b < 1 || (int64_t)p.perm_a * p.perm_b != p.n))
      return dmg_error(DMG_ERR_ARG, "fft slot order %d x %d does not match length %d", p.perm_a, p.perm_b, p.n);
    const int st = dtype == 0 ? check_batch<double>(p, g->job[j].bt)
                              : dtype == 2 ? check_batch<df>(p, g->job[j].bt) : check_batch<float>(p, g->job[j].bt);
    if (st != DMG_OK) return st;
  }
  const bool inv = sign > 0;
  switch (dtype) {
    case 0: return inv ? dmg_fft_pass_f64_inv_group(g, stream) : dmg_fft_pass_f64_fwd_group(g, stream);
    case 1:
    case 3:  // the tensor-core form has no runtime-length kernel: its passes run in FP32
      return inv ? dmg_fft_pass_f32_inv_group(g, stream) : dmg_fft_pass_f32_fwd_group(g, stream);
    case 2: return inv ? dmg_fft_pass_df_inv_group(g, stream) : dmg_fft_pass_df_fwd_group(g, stream);
    default: return dmg_error(DMG_ERR_ARG, "fft dtype %d", dtype);
  }
}

extern "C" int dmg_fft_pass_launch(const dmg_fft_pass *p, int dtype, const void *src, void *dst, void *stream) {
  dmg_fft_batch b;
  b.count = 1;
  b.src[0] = src;
  b.dst[0] = dst;
  b.scale_exp[0] = p->scale_exp;
  return dmg_fft_pass_launch_batch(p, dtype, &b, stream);
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
  if (!lay->ranked) {
    const int64_t rows = (int64_t)L0 * L1;
    const int64_t grid = rows < (int64_t)nsm * 8 ? rows : (int64_t)nsm * 8;
    maxexp_rows_kernel<<<(unsigned)grid, 256, 0, s>>>(*lay, ndim, L0, L1, L2, static_cast<const double2 *>(src), out);
  } else {
    maxexp_kernel<<<nsm * 8, 256, 0, s>>>(*lay, ndim, L0, L1, L2, static_cast<const double2 *>(src), out);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "maxexp launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}
