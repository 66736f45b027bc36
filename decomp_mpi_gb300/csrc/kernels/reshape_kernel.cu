// Reshape permutation kernel: the data movement of runReshapePlan
// (reference reshape.c:461-492), whose per-peer typemaps (typelist.c:74-119)
// and MPI exchange become one permutation over the virtual grid.
//
// One launch moves a whole virtual-grid array from one decomposition to
// another: dst[addr_dst(g)] = src[addr_src(g)] for every global coordinate g
// held by both sides.  Addresses come from per-axis tables (k1_params.h).
//
// Work is split into 2-D tiles over two axes: ax0, along which the source is
// contiguous, and ax1, along which the destination is contiguous.  A block
// reads its tile in source order into shared memory and writes it out in
// destination order, so both the HBM reads and the HBM writes are coalesced
// even when the decompositions transpose the fast axis.  When both sides are
// contiguous along the same axis the planner widens the unit (up to 16 bytes)
// and the tile is read and written in the same order.  The launch is
// persistent: a grid sized to fill the SMs walks the tiles in order, so
// neighbouring tiles are in flight together and share L2 lines.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include "../host/dmg_internal.h"
#include "../host/k1_params.h"

namespace {

constexpr int NT = 256;      // threads per block
constexpr int MAXITEMS = 8;  // tile elements per thread per phase (tile <= 2048 units)

struct u8x1 { uint8_t v; };
struct u16x1 { uint16_t v; };

template <bool RANKED>
struct SideSlices {
  int64_t *t0, *t1;  // tile slices of the ax0 / ax1 tables
  int32_t *r0, *r1;  // ranked: rank parts
};

template <bool RANKED>
__device__ __forceinline__ int64_t side_addr(const dmg_k1_side &s, const SideSlices<RANKED> &sl, int64_t base,
                                             int32_t rbase, const int64_t *bto, int nbatch, const int32_t *bax,
                                             int ax0, int ax1, int i0, int i1) {
  if constexpr (!RANKED) {
    return base + sl.t0[i0] + sl.t1[i1];
  } else {
    int32_t R = rbase + sl.r0[i0] + sl.r1[i1];
    if (R < 0) return -1;
    const int64_t *rs = s.rstride;
    const int P = s.nranks;
    int64_t a = (int64_t)R * s.pitch + sl.t0[i0] * __ldg(rs + (size_t)ax0 * P + R);
    if (ax1 >= 0) a += sl.t1[i1] * __ldg(rs + (size_t)ax1 * P + R);
    for (int b = 0; b < nbatch; ++b) a += bto[b] * __ldg(rs + (size_t)bax[b] * P + R);
    return a;
  }
}

template <typename U, bool SR, bool DR>
__global__ void __launch_bounds__(NT) k1_permute(const dmg_k1_params p, const U *__restrict__ src, U *__restrict__ dst) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ int64_t s_base, d_base;
  __shared__ int32_t s_rb, d_rb;
  __shared__ int64_t s_bto[DMG_MAXAX], d_bto[DMG_MAXAX];
  __shared__ int32_t s_bax[DMG_MAXAX];
  __shared__ int32_t s_g0, s_g1, s_lim0, s_lim1;

  const int e0 = p.e0, e1 = p.e1;
  const int ld = e0 + 1;  // padded row length of the tile buffer
  U *buf = reinterpret_cast<U *>(sm);
  size_t off = sizeof(U) * (size_t)e1 * ld;
  off = (off + 15) & ~size_t(15);
  int64_t *st0 = reinterpret_cast<int64_t *>(sm + off);
  int64_t *st1 = st0 + e0;
  int64_t *dt0 = st1 + e1;
  int64_t *dt1 = dt0 + e0;
  int32_t *sr0 = reinterpret_cast<int32_t *>(dt1 + e1);
  int32_t *sr1 = sr0 + e0;
  int32_t *dr0 = sr1 + e1;
  int32_t *dr1 = dr0 + e0;
  SideSlices<SR> ssl{st0, st1, sr0, sr1};
  SideSlices<DR> dsl{dt0, dt1, dr0, dr1};

  const int ax0 = p.ax0, ax1 = p.ax1;
  const int tid = threadIdx.x;
  if (tid < DMG_MAXAX) s_bax[tid] = tid < p.nbatch ? p.batch_ax[tid] : 0;

  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    __syncthreads();  // the previous tile is done with shared memory
    if (tid == 0) {
      int64_t t = tile;
      int t0 = (int)(t % p.nt0);
      t /= p.nt0;
      int t1 = 0;
      if (ax1 >= 0) {
        t1 = (int)(t % p.nt1);
        t /= p.nt1;
      }
      int64_t sb = 0, db = 0;
      int32_t rs = 0, rd = 0;
      for (int b = 0; b < p.nbatch; ++b) {
        int a = p.batch_ax[b];
        int c = (int)(t % p.len[a]);
        t /= p.len[a];
        if constexpr (SR) {
          rs += p.src.rk[a][c];
          s_bto[b] = p.src.tab[a][c];
        } else {
          sb += p.src.tab[a][c];
        }
        if constexpr (DR) {
          rd += p.dst.rk[a][c];
          d_bto[b] = p.dst.tab[a][c];
        } else {
          db += p.dst.tab[a][c];
        }
      }
      s_base = sb;
      d_base = db;
      s_rb = rs;
      d_rb = rd;
      int g0 = t0 * e0, g1 = t1 * e1;
      s_g0 = g0;
      s_g1 = g1;
      s_lim0 = min(e0, p.len[ax0] - g0);
      s_lim1 = ax1 >= 0 ? min(e1, p.len[ax1] - g1) : 1;
    }
    __syncthreads();
    const int g0 = s_g0, g1 = s_g1, lim0 = s_lim0, lim1 = s_lim1;
    for (int i = tid; i < lim0; i += NT) {
      st0[i] = __ldg(p.src.tab[ax0] + g0 + i);
      dt0[i] = __ldg(p.dst.tab[ax0] + g0 + i);
      if constexpr (SR) sr0[i] = __ldg(p.src.rk[ax0] + g0 + i);
      if constexpr (DR) dr0[i] = __ldg(p.dst.rk[ax0] + g0 + i);
    }
    if (ax1 >= 0) {
      for (int i = tid; i < lim1; i += NT) {
        st1[i] = __ldg(p.src.tab[ax1] + g1 + i);
        dt1[i] = __ldg(p.dst.tab[ax1] + g1 + i);
        if constexpr (SR) sr1[i] = __ldg(p.src.rk[ax1] + g1 + i);
        if constexpr (DR) dr1[i] = __ldg(p.dst.rk[ax1] + g1 + i);
      }
    } else if (tid == 0) {
      st1[0] = 0;
      dt1[0] = 0;
      sr1[0] = 0;
      dr1[0] = 0;
    }
    __syncthreads();
    const int64_t sb = s_base, db = d_base;
    const int32_t rsb = s_rb, rdb = d_rb;
    // a batch coordinate that a side does not hold empties the whole tile
    bool skip = (SR ? rsb < 0 : sb < 0) || (DR ? rdb < 0 : db < 0);
    if (skip) continue;
    const int n = lim0 * lim1;

    // ---- load: source order ----
    {
      const int F = p.load_fast == 0 ? lim0 : lim1;
      int q = tid / F, r = tid - (tid / F) * F;
      const int dq = NT / F, dr = NT - (NT / F) * F;
      U v[MAXITEMS];
      int idx[MAXITEMS];
#pragma unroll
      for (int j = 0; j < MAXITEMS; ++j) {
        int k = tid + j * NT;
        idx[j] = -1;
        if (k < n) {
          int i0 = p.load_fast == 0 ? r : q;
          int i1 = p.load_fast == 0 ? q : r;
          int64_t a = side_addr<SR>(p.src, ssl, sb, rsb, s_bto, p.nbatch, s_bax, ax0, ax1, i0, i1);
          if (a >= 0) {
            v[j] = src[a];
            idx[j] = i1 * ld + i0;
          }
        }
        r += dr;
        q += dq;
        if (r >= F) {
          r -= F;
          q += 1;
        }
      }
#pragma unroll
      for (int j = 0; j < MAXITEMS; ++j)
        if (idx[j] >= 0) buf[idx[j]] = v[j];
    }
    __syncthreads();
    // ---- store: destination order ----
    {
      const int F = p.store_fast == 0 ? lim0 : lim1;
      int q = tid / F, r = tid - (tid / F) * F;
      const int dq = NT / F, dr = NT - (NT / F) * F;
#pragma unroll
      for (int j = 0; j < MAXITEMS; ++j) {
        int k = tid + j * NT;
        if (k < n) {
          int i0 = p.store_fast == 0 ? r : q;
          int i1 = p.store_fast == 0 ? q : r;
          int64_t da = side_addr<DR>(p.dst, dsl, db, rdb, d_bto, p.nbatch, s_bax, ax0, ax1, i0, i1);
          if (da >= 0) {
            int64_t sa = side_addr<SR>(p.src, ssl, sb, rsb, s_bto, p.nbatch, s_bax, ax0, ax1, i0, i1);
            if (sa >= 0) dst[da] = buf[i1 * ld + i0];
          }
        }
        r += dr;
        q += dq;
        if (r >= F) {
          r -= F;
          q += 1;
        }
      }
    }
  }
}

// Address of (i0, i1) of a tile from global tables (direct kernel).
template <bool RANKED>
__device__ __forceinline__ int64_t direct_addr(const dmg_k1_side &s, int64_t base, int32_t rbase, const int64_t *bto,
                                               const int32_t *bax, int nbatch, int ax0, int ax1, int g0, int g1) {
  if constexpr (!RANKED) {
    int64_t a = base + __ldg(s.tab[ax0] + g0);
    if (ax1 >= 0) a += __ldg(s.tab[ax1] + g1);
    return a;
  } else {
    int32_t R = rbase + __ldg(s.rk[ax0] + g0);
    if (ax1 >= 0) R += __ldg(s.rk[ax1] + g1);
    if (R < 0) return -1;
    const int64_t *rs = s.rstride;
    const int P = s.nranks;
    int64_t a = (int64_t)R * s.pitch + __ldg(s.tab[ax0] + g0) * __ldg(rs + (size_t)ax0 * P + R);
    if (ax1 >= 0) a += __ldg(s.tab[ax1] + g1) * __ldg(rs + (size_t)ax1 * P + R);
    for (int b = 0; b < nbatch; ++b) a += bto[b] * __ldg(rs + (size_t)bax[b] * P + R);
    return a;
  }
}

// Same fast axis on both sides: every thread moves its own elements straight
// from source to destination, MAXITEMS loads in flight before the stores,
// with no shared memory and no barrier.  Tiles run along ax0 (contiguous on
// both sides) and ax1.  One tile of one array:
template <typename U, bool SR, bool DR>
__device__ __forceinline__ void direct_tile(const dmg_k1_params &p, const U *__restrict__ src, U *__restrict__ dst,
                                            int64_t tile) {
  const int ax0 = p.ax0, ax1 = p.ax1;
  const int e0 = p.e0, e1 = p.e1;
  const int tid = threadIdx.x;
  int64_t t = tile;
  const int t0 = (int)(t % p.nt0);
  t /= p.nt0;
  int t1 = 0;
  if (ax1 >= 0) {
    t1 = (int)(t % p.nt1);
    t /= p.nt1;
  }
  int64_t sb = 0, db = 0;
  int32_t rs = 0, rd = 0;
  int64_t sbto[DMG_MAXAX], dbto[DMG_MAXAX];
  int32_t bax[DMG_MAXAX];
#pragma unroll
  for (int b = 0; b < DMG_MAXAX; ++b) {
    if (b < p.nbatch) {
      const int a = p.batch_ax[b];
      const int c = (int)(t % p.len[a]);
      t /= p.len[a];
      bax[b] = a;
      if constexpr (SR) {
        rs += __ldg(p.src.rk[a] + c);
        sbto[b] = __ldg(p.src.tab[a] + c);
      } else {
        sb += __ldg(p.src.tab[a] + c);
      }
      if constexpr (DR) {
        rd += __ldg(p.dst.rk[a] + c);
        dbto[b] = __ldg(p.dst.tab[a] + c);
      } else {
        db += __ldg(p.dst.tab[a] + c);
      }
    }
  }
  if ((SR ? rs < 0 : sb < 0) || (DR ? rd < 0 : db < 0)) return;
  const int g0 = t0 * e0, g1 = t1 * e1;
  const int lim0 = min(e0, p.len[ax0] - g0);
  const int lim1 = ax1 >= 0 ? min(e1, p.len[ax1] - g1) : 1;
  const int n = lim0 * lim1;
  int q = tid / lim0, r = tid - q * lim0;
  const int dq = NT / lim0, dr = NT - (NT / lim0) * lim0;
  U v[MAXITEMS];
  int64_t da[MAXITEMS];
#pragma unroll
  for (int j = 0; j < MAXITEMS; ++j) {
    da[j] = -1;
    if (tid + j * NT < n) {
      int64_t d = direct_addr<DR>(p.dst, db, rd, dbto, bax, p.nbatch, ax0, ax1, g0 + r, g1 + q);
      int64_t s = direct_addr<SR>(p.src, sb, rs, sbto, bax, p.nbatch, ax0, ax1, g0 + r, g1 + q);
      if (d >= 0 && s >= 0) {
        v[j] = src[s];
        da[j] = d;
      }
    }
    r += dr;
    q += dq;
    if (r >= lim0) {
      r -= lim0;
      q += 1;
    }
  }
#pragma unroll
  for (int j = 0; j < MAXITEMS; ++j)
    if (da[j] >= 0) dst[da[j]] = v[j];
}

template <typename U, bool SR, bool DR>
__global__ void __launch_bounds__(NT, 4) k1_direct(const dmg_k1_params p, const U *__restrict__ src, U *__restrict__ dst) {
  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) direct_tile<U, SR, DR>(p, src, dst, tile);
}

// Several reshapes, of any sizes and decompositions, in one persistent
// launch: the tiles of all jobs form one sequence (job j's tiles from
// first_tile), and a block finds the job of each of its tiles.  Every job
// moves units of the same size and has the same ranked / separable sides.
template <typename U, bool SR, bool DR>
__global__ void __launch_bounds__(NT, 4) k1_direct_group(const dmg_k1_group g) {
  for (int64_t tile = blockIdx.x; tile < g.total_tiles; tile += gridDim.x) {
    int j = 0;
    while (j + 1 < g.count && tile >= g.job[j + 1].first_tile) ++j;
    const dmg_k1_group_job &job = g.job[j];
    direct_tile<U, SR, DR>(job.p, static_cast<const U *>(job.src), static_cast<U *>(job.dst), tile - job.first_tile);
  }
}

template <typename U, bool SR, bool DR>
int launch_direct_group(const dmg_k1_group &g, cudaStream_t stream) {
  auto kern = k1_direct_group<U, SR, DR>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, 0);
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > g.total_tiles) grid = g.total_tiles;
  if (grid < 1) return DMG_OK;
  kern<<<(unsigned)grid, NT, 0, stream>>>(g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "grouped reshape kernel launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

template <typename U>
int launch_group_unit(const dmg_k1_group &g, cudaStream_t stream) {
  const bool sr = g.job[0].p.src.ranked, dr = g.job[0].p.dst.ranked;
  if (sr && dr) return launch_direct_group<U, true, true>(g, stream);
  if (sr) return launch_direct_group<U, true, false>(g, stream);
  if (dr) return launch_direct_group<U, false, true>(g, stream);
  return launch_direct_group<U, false, false>(g, stream);
}

template <typename U, bool SR, bool DR>
int launch_direct(const dmg_k1_params &p, const void *src, void *dst, cudaStream_t stream) {
  auto kern = k1_direct<U, SR, DR>;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, 0);
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return DMG_OK;
  kern<<<(unsigned)grid, NT, 0, stream>>>(p, static_cast<const U *>(src), static_cast<U *>(dst));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "reshape kernel launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

template <typename U, bool SR, bool DR>
int launch_typed(const dmg_k1_params &p, const void *src, void *dst, cudaStream_t stream) {
  if (p.load_fast == p.store_fast) return launch_direct<U, SR, DR>(p, src, dst, stream);
  const size_t tilebytes = (sizeof(U) * (size_t)p.e1 * (p.e0 + 1) + 15) & ~size_t(15);
  const size_t smem = tilebytes + (size_t)(p.e0 + p.e1) * 2 * (sizeof(int64_t) + sizeof(int32_t));
  auto kern = k1_permute<U, SR, DR>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "reshape kernel smem attribute: %s", cudaGetErrorString(e));
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return DMG_OK;
  kern<<<(unsigned)grid, NT, smem, stream>>>(p, static_cast<const U *>(src), static_cast<U *>(dst));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "reshape kernel launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

template <typename U>
int launch_unit(const dmg_k1_params &p, const void *src, void *dst, cudaStream_t stream) {
  if (p.src.ranked && p.dst.ranked) return launch_typed<U, true, true>(p, src, dst, stream);
  if (p.src.ranked) return launch_typed<U, true, false>(p, src, dst, stream);
  if (p.dst.ranked) return launch_typed<U, false, true>(p, src, dst, stream);
  return launch_typed<U, false, false>(p, src, dst, stream);
}

}  // namespace

extern "C" int dmg_k1_launch(const dmg_k1_params *p, int unit, const void *src, void *dst, void *stream) {
  if (p->e0 * p->e1 > NT * MAXITEMS)
    return dmg_error(DMG_ERR_ARG, "reshape tile %dx%d exceeds %d units", p->e0, p->e1, NT * MAXITEMS);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (unit) {
    case 1: return launch_unit<u8x1>(*p, src, dst, s);
    case 2: return launch_unit<u16x1>(*p, src, dst, s);
    case 4: return launch_unit<uint32_t>(*p, src, dst, s);
    case 8: return launch_unit<uint2>(*p, src, dst, s);
    case 16: return launch_unit<uint4>(*p, src, dst, s);
    default: return dmg_error(DMG_ERR_ARG, "reshape unit %d bytes unsupported", unit);
  }
}

extern "C" int dmg_k1_launch_group(const dmg_k1_group *g, int unit, void *stream) {
  if (g->count < 1 || g->count > DMG_K1_MAXGROUP)
    return dmg_error(DMG_ERR_ARG, "grouped reshape: %d jobs (1 to %d)", g->count, DMG_K1_MAXGROUP);
  for (int j = 0; j < g->count; ++j) {
    const dmg_k1_params &p = g->job[j].p;
    if (p.e0 * p.e1 > NT * MAXITEMS || p.load_fast != p.store_fast || p.src.ranked != g->job[0].p.src.ranked ||
        p.dst.ranked != g->job[0].p.dst.ranked)
      return dmg_error(DMG_ERR_ARG, "grouped reshape: job %d does not fit the group's kernel", j);
    if (g->job[j].first_tile != (j ? g->job[j - 1].first_tile + g->job[j - 1].p.ntiles : 0))
      return dmg_error(DMG_ERR_ARG, "grouped reshape: job %d's tiles do not follow job %d's", j, j - 1);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (unit) {
    case 1: return launch_group_unit<u8x1>(*g, s);
    case 2: return launch_group_unit<u16x1>(*g, s);
    case 4: return launch_group_unit<uint32_t>(*g, s);
    case 8: return launch_group_unit<uint2>(*g, s);
    case 16: return launch_group_unit<uint4>(*g, s);
    default: return dmg_error(DMG_ERR_ARG, "reshape unit %d bytes unsupported", unit);
  }
}
