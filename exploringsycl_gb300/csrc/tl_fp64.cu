/*
 * tl_fp64.cu -- double-precision kernels of the GB300 TeaLeaf backend: the
 * drop-in replacements of the reference's SYCL kernels and the persistent
 * CG solve. Compiled with --fmad=false: every product and sum is rounded
 * separately, as a sequential evaluation of the reference's expressions
 * would round it, so the results match the CPU oracle bit for bit.
 *
 * Launch shapes
 *  - map kernels: 256 threads, one cell per thread, grid-stride;
 *  - reducing kernels: 256 threads (8 warps) per 4096-cell tile, one warp per
 *    8 of its 64-cell groups (two cells per lane per group; the five upper
 *    tree levels of the 8 groups shared out among the lanes,
 *    warp_sum8_groups); the last block to finish reduces the tile partials in
 *    the reference order and writes the scalar straight into pinned host
 *    memory, so one launch and one stream synchronisation return a dot
 *    product (the reference issues 1 + ceil(log64 n) kernels and a blocking
 *    host read, TeaLeaf/c_kernels/sycl/sycl_shared.hpp:35-79);
 *  - the persistent CG kernel: one 1024-thread block per SM (cooperative
 *    launch), three grid barriers per CG step, scalars alpha/beta computed
 *    redundantly (and identically) by every block.
 */
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "tl_internal.cuh"
#include "tl_dmul.cuh"

namespace {

constexpr int kMapThreads = 256;
constexpr int kRedThreads = 256;
constexpr int kPersistThreads = 1024;
/* Which multiplications of the persistent CG run on the integer pipes
 * (tl_dmul.cuh; the products are the same IEEE-rounded values): 0 none, 1 the
 * exact contract's stencil, 2 all of the exact contract's, 3 also the plain
 * products of the fused contract. */
#ifndef TL_INT_DMUL
#define TL_INT_DMUL 3
#endif
constexpr int kIntMul = TL_INT_DMUL;

/* Exact-contract products: on the integer pipes at the given level. */
template <int kLevel>
__device__ __forceinline__ double xmul(double a, double b) {
  if constexpr (kIntMul >= kLevel) return tl_dmul(a, b);
  return a * b;
}

/* ------------------------------------------------------------ helpers */

__device__ __forceinline__ bool interior(int kk, int jj, int x, int y, int hd) {
  return kk >= hd && kk < x - hd && jj >= hd && jj < y - hd;
}

/* The 5-point operator of TeaLeaf/shared.h:59-63 with the reference's
 * grouping: ((1 + (kx1+kx0)) + (ky1+ky0))*a - (kx1*a1 + kx0*a-1)
 * - (ky1*a+x + ky0*a-x). The five products run on the integer pipes (the
 * same IEEE products; these kernels are bound by the FP64 pipe). */
template <class Load>
__device__ __forceinline__ double smvp(Load a, const double* __restrict__ kx,
                                       const double* __restrict__ ky,
                                       unsigned i, int x) {
  const double kx0 = kx[i], kx1 = kx[i + 1];
  const double ky0 = ky[i], ky1 = ky[i + x];
  return xmul<1>(1.0 + (kx1 + kx0) + (ky1 + ky0), a(i)) -
         (xmul<1>(kx1, a(i + 1)) + xmul<1>(kx0, a(i - 1))) -
         (xmul<1>(ky1, a(i + x)) + xmul<1>(ky0, a(i - x)));
}

struct PlainLoad {
  const double* p;
  __device__ __forceinline__ double operator()(unsigned i) const { return p[i]; }
};

/* ---------------------------------------------------------- map kernels */

template <class Op>
__global__ void __launch_bounds__(kMapThreads) map_kernel(Op op, int x, int y) {
  const unsigned len = (unsigned)x * (unsigned)y;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    op(i, kk, jj);
  }
}

template <class Op>
int launch_map(tl_context* ctx, const Op& op, int x, int y) {
  const unsigned len = (unsigned)x * (unsigned)y;
  unsigned blocks = (len + kMapThreads - 1) / kMapThreads;
  const unsigned cap = (unsigned)ctx->num_sms * 16u;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  map_kernel<Op><<<blocks, kMapThreads, 0, ctx->stream>>>(op, x, y);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

/* Sums of 8 consecutive 64-cell groups held by one warp, two cells per lane
 * per group (v[g] = cell 2*lane + cell 2*lane+1 of group g), in the
 * reference's tree order. Instead of a full butterfly per group (every lane
 * adding at every level), the warp halves its set of groups at each of the
 * first three levels (lane pairs exchange the halves they do not keep), then
 * finishes with two butterfly levels: the same pairs are added at every
 * level, but each level costs 4, 2, 1, 1, 1 additions per lane instead of 8.
 * Returns the total of group ((lane&1)<<2 | (lane&2) | (lane>>2&1)); lanes
 * with equal low three bits hold the same group. */
__device__ __forceinline__ double warp_sum8_groups(const double v[8], int lane) {
  const bool h1 = lane & 1, h2 = lane & 2, h4 = lane & 4;
  double a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double send = h1 ? v[k] : v[4 + k];
    const double recv = __shfl_xor_sync(TL_FULL_MASK, send, 1);
    a[k] = (h1 ? v[4 + k] : v[k]) + recv;
  }
  double b[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double send = h2 ? a[k] : a[2 + k];
    const double recv = __shfl_xor_sync(TL_FULL_MASK, send, 2);
    b[k] = (h2 ? a[2 + k] : a[k]) + recv;
  }
  const double send = h4 ? b[0] : b[1];
  const double recv = __shfl_xor_sync(TL_FULL_MASK, send, 4);
  double c = (h4 ? b[1] : b[0]) + recv;
  c = c + __shfl_xor_sync(TL_FULL_MASK, c, 8);
  c = c + __shfl_xor_sync(TL_FULL_MASK, c, 16);
  return c;
}

__device__ __forceinline__ int warp_sum8_group_of_lane(int lane) {
  return ((lane & 1) << 2) | (lane & 2) | ((lane >> 2) & 1);
}

/* ----------------------------------------------------- reducing kernels */

/* Op must provide `static constexpr int N` (number of sums) and
 * `operator()(i, kk, jj, double* c)` that, for an interior cell, performs
 * the cell's update and stores its N contributions into c. */
template <class Op>
__global__ void __launch_bounds__(kRedThreads)
reduce_kernel(Op op, int x, int y, int hd, double* part, size_t part_stride,
              int ntiles, unsigned* ticket, double* result) {
  constexpr int N = Op::N;
  __shared__ double s_group[N][TL_GROUP];
  __shared__ double s_scratch[TL_RED_SCRATCH];
  __shared__ int s_last;
  const unsigned len = (unsigned)x * (unsigned)y;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned base = (unsigned)tile * TL_TILE;
    /* each warp: groups g0 .. g0+7 of the tile, the first tree level in the
     * lane (cells 2*lane, 2*lane+1), the other five shared by the warp */
    for (int g0 = 8 * warp; g0 < TL_GROUP; g0 += 8 * nwarps) {
      double v[N][8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const unsigned i0 = base + (unsigned)(g0 + k) * TL_GROUP + 2u * lane;
        double c0[N], c1[N];
#pragma unroll
        for (int s = 0; s < N; ++s) { c0[s] = 0.0; c1[s] = 0.0; }
        if (i0 < len) {
          const int jj = (int)(i0 / (unsigned)x);
          const int kk = (int)(i0 - (unsigned)jj * (unsigned)x);
          if (interior(kk, jj, x, y, hd)) op(i0, kk, jj, c0);
        }
        if (i0 + 1 < len) {
          const unsigned i1 = i0 + 1;
          const int jj = (int)(i1 / (unsigned)x);
          const int kk = (int)(i1 - (unsigned)jj * (unsigned)x);
          if (interior(kk, jj, x, y, hd)) op(i1, kk, jj, c1);
        }
#pragma unroll
        for (int s = 0; s < N; ++s) v[s][k] = c0[s] + c1[s];
      }
#pragma unroll
      for (int s = 0; s < N; ++s) {
        const double t = warp_sum8_groups(v[s], lane);
        if (lane < 8) s_group[s][g0 + warp_sum8_group_of_lane(lane)] = t;
      }
    }
    __syncthreads();
    if (warp < N) {
      const double v = tl_tree64(s_group[warp][2 * lane], s_group[warp][2 * lane + 1]);
      if (lane == 0) part[warp * part_stride + tile] = v;
    }
    __syncthreads();
  }

  /* Last block to finish reduces the tile partials. */
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int s = 0; s < N; ++s) {
    const double total = tl_reduce_partials(part + s * part_stride, ntiles, s_scratch);
    if (threadIdx.x == 0) result[s] = total;
  }
  if (threadIdx.x == 0) {
    __threadfence_system();
    *ticket = 0u;
  }
}

/* Launches a reducing kernel and returns its N sums in out[0..N). */
template <class Op>
int launch_reduce(tl_context* ctx, const Op& op, int x, int y, int hd,
                  double* out) {
  const size_t ntiles = tl_num_tiles(x, y);
  int rc = tl_ensure_partials(ctx, ntiles);
  if (rc != TL_OK) return rc;
  const int blocks = (int)ntiles;
  reduce_kernel<Op><<<blocks, kRedThreads, 0, ctx->stream>>>(
      op, x, y, hd, ctx->d_part, ctx->part_cap, (int)ntiles,
      ctx->d_sync + TL_SYNC_TICKET, ctx->d_result);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int s = 0; s < Op::N; ++s) out[s] = ((volatile double*)ctx->h_result)[s];
  return TL_OK;
}

/* ------------------------------------------------------------ kernels */

struct CgInitUOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:7-37 */
  int coefficient;
  double *p, *r, *u, *w;
  const double *density, *energy;
  int x, y;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    p[i] = 0.0;
    r[i] = 0.0;
    u[i] = energy[i] * density[i];
    if (jj > 0 && jj < y - 1 && kk > 0 && kk < x - 1) {
      w[i] = (coefficient == TL_CONDUCTIVITY) ? density[i] : 1.0 / density[i];
    }
  }
};

struct CgInitKOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:40-69 */
  int x, y, hd;
  const double* w;
  double *kx, *ky;
  double rx, ry;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (jj >= hd && jj < y - 1 && kk >= hd && kk < x - 1) {
      kx[i] = rx * (w[i - 1] + w[i]) / (2.0 * w[i - 1] * w[i]);
      ky[i] = ry * (w[i - x] + w[i]) / (2.0 * w[i - x] * w[i]);
    }
  }
};

struct CgInitOthersOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:72-134 */
  static constexpr int N = 1;
  int x;
  const double *kx, *ky, *u;
  double *p, *r, *w;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    const double s = smvp(PlainLoad{u}, kx, ky, i, x);
    w[i] = s;
    const double rv = u[i] - s;
    r[i] = rv;
    p[i] = rv;
    c[0] = rv * rv;
  }
};

struct CgCalcWOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:137-195 */
  static constexpr int N = 1;
  int x;
  const double *p, *kx, *ky;
  double* w;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    const double s = smvp(PlainLoad{p}, kx, ky, i, x);
    w[i] = s;
    c[0] = s * p[i];
  }
};

struct CgCalcUrOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:198-254 */
  static constexpr int N = 1;
  double *u, *r;
  const double *p, *w;
  double alpha;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    u[i] = u[i] + alpha * p[i];
    const double rv = r[i] - alpha * w[i];
    r[i] = rv;
    c[0] = rv * rv;
  }
};

struct CgCalcPOp {  /* TeaLeaf/c_kernels/sycl/cg.cpp:257-281 */
  int x, y, hd;
  double beta;
  double* p;
  const double* r;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) p[i] = beta * p[i] + r[i];
  }
};

struct CopyUOp {  /* TeaLeaf/c_kernels/sycl/solver_methods.cpp:7-31 */
  int x, y, hd;
  const double* u;
  double* u0;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) u0[i] = u[i];
  }
};

struct ResidualOp {  /* TeaLeaf/c_kernels/sycl/solver_methods.cpp:34-65 */
  int x, y, hd;
  const double *u, *u0, *kx, *ky;
  double* r;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) {
      const double s = smvp(PlainLoad{u}, kx, ky, i, x);
      r[i] = u0[i] - s;
    }
  }
};

/* calc_residual and calc_2norm of its result in one pass: the same r and
 * the same sum (same cells, same tree) as ResidualOp then Norm2Op. */
struct ResidualNormOp {
  static constexpr int N = 1;
  int x;
  const double *u, *u0, *kx, *ky;
  double* r;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    const double rv = u0[i] - smvp(PlainLoad{u}, kx, ky, i, x);
    r[i] = rv;
    c[0] = rv * rv;
  }
};

struct Norm2Op {  /* TeaLeaf/c_kernels/sycl/solver_methods.cpp:68-117 */
  static constexpr int N = 1;
  const double* b;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    c[0] = b[i] * b[i];
  }
};

struct FinaliseOp {  /* TeaLeaf/c_kernels/sycl/solver_methods.cpp:120-145 */
  int x, y, hd;
  const double *u, *density;
  double* energy;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) energy[i] = u[i] / density[i];
  }
};

struct SummaryOp {  /* TeaLeaf/c_kernels/sycl/field_summary.cpp:6-151 */
  static constexpr int N = 4;
  const double *u, *density, *energy0, *volume;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    const double cell_vol = volume[i];
    const double cell_mass = cell_vol * density[i];
    c[0] = cell_vol;
    c[1] = cell_mass;
    c[2] = cell_mass * energy0[i];
    c[3] = cell_mass * u[i];
  }
};

struct InitialStateOp {  /* TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:8-27 */
  double e, d;
  double *energy0, *density;
  __device__ void operator()(unsigned i, int, int) const {
    energy0[i] = e;
    density[i] = d;
  }
};

struct StateOp {  /* TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:30-92 */
  int x, y;
  tl_state s;
  double *energy0, *density, *u;
  const double *cell_x, *cell_y, *vertex_x, *vertex_y;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    bool apply = false;
    if (s.geometry == TL_RECTANGULAR) {
      apply = vertex_x[kk + 1] >= s.x_min && vertex_x[kk] < s.x_max &&
              vertex_y[jj + 1] >= s.y_min && vertex_y[jj] < s.y_max;
    } else if (s.geometry == TL_CIRCULAR) {
      const double radius = sqrt((cell_x[kk] - s.x_min) * (cell_x[kk] - s.x_min) +
                                 (cell_y[jj] - s.y_min) * (cell_y[jj] - s.y_min));
      apply = radius <= s.radius;
    } else if (s.geometry == TL_POINT) {
      apply = vertex_x[kk] == s.x_min && vertex_y[jj] == s.y_min;
    }
    if (apply) {
      energy0[i] = s.energy;
      density[i] = s.density;
    }
    if (kk > 0 && kk < x - 1 && jj > 0 && jj < y - 1) u[i] = energy0[i] * density[i];
  }
};

struct CopyAllOp {  /* store_energy / jacobi_copy_u: dst = src everywhere */
  double* dst;
  const double* src;
  __device__ void operator()(unsigned i, int, int) const { dst[i] = src[i]; }
};

struct ChunkDataOp {  /* TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:31-64 */
  int x, y;
  const double *vertex_x, *vertex_y;
  double *cell_x, *cell_y, *volume, *x_area, *y_area;
  double dx, dy;
  __device__ void operator()(unsigned i, int, int) const {
    if (i < (unsigned)x) cell_x[i] = 0.5 * (vertex_x[i] + vertex_x[i + 1]);
    if (i < (unsigned)y) cell_y[i] = 0.5 * (vertex_y[i] + vertex_y[i + 1]);
    volume[i] = dx * dy;
    x_area[i] = dy;
    y_area[i] = dx;
  }
};

__global__ void vertices_kernel(int x, int y, int hd, double* vertex_x,
                                double* vertex_y, double x_min, double y_min,
                                double dx, double dy) {
  /* TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:8-28 */
  const int n = (x > y ? x : y) + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i < x + 1) vertex_x[i] = x_min + dx * (i - (double)hd);
    if (i < y + 1) vertex_y[i] = y_min + dy * (i - (double)hd);
  }
}

struct JacobiInitOp {  /* TeaLeaf/c_kernels/sycl/jacobi.cpp:7-56 */
  int x, y, hd, coefficient;
  double rx, ry;
  double *u, *u0, *kx, *ky;
  const double *density, *energy;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (kk > 0 && kk < x - 1 && jj > 0 && jj < y - 1) {
      const double v = energy[i] * density[i];
      u0[i] = v;
      u[i] = v;
    }
    if (jj >= hd && jj < y - 1 && kk >= hd && kk < x - 1) {
      const bool cond = coefficient == TL_CONDUCTIVITY;
      const double dc = cond ? density[i] : 1.0 / density[i];
      const double dl = cond ? density[i - 1] : 1.0 / density[i - 1];
      const double dd = cond ? density[i - x] : 1.0 / density[i - x];
      kx[i] = rx * (dl + dc) / (2.0 * dl * dc);
      ky[i] = ry * (dd + dc) / (2.0 * dd * dc);
    }
  }
};

struct JacobiIterateOp {  /* TeaLeaf/c_kernels/sycl/jacobi.cpp:59-119 */
  static constexpr int N = 1;
  int x;
  double* u;
  const double *u0, *r, *kx, *ky;
  __device__ void operator()(unsigned i, int, int, double* c) const {
    const double v = (u0[i] + (kx[i + 1] * r[i + 1] + kx[i] * r[i - 1]) +
                      (ky[i + x] * r[i + x] + ky[i] * r[i - x])) /
                     (1.0 + (kx[i] + kx[i + 1]) + (ky[i] + ky[i + x]));
    u[i] = v;
    c[0] = fabs(v - r[i]);
  }
};

struct ChebyInitOp {  /* TeaLeaf/c_kernels/sycl/cheby.cpp:7-38 */
  int x, y, hd;
  double theta;
  double *p, *r, *w;
  const double *u, *u0, *kx, *ky;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) {
      const double s = smvp(PlainLoad{u}, kx, ky, i, x);
      w[i] = s;
      const double rv = u0[i] - s;
      r[i] = rv;
      p[i] = rv / theta;
    }
  }
};

struct ChebyIterateOp {  /* TeaLeaf/c_kernels/sycl/cheby.cpp:67-110 */
  int x, y, hd;
  double alpha, beta;
  double *p, *r, *w;
  const double *u, *u0, *kx, *ky;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) {
      const double s = smvp(PlainLoad{u}, kx, ky, i, x);
      w[i] = s;
      const double rv = u0[i] - s;
      r[i] = rv;
      p[i] = alpha * p[i] + beta * rv;
    }
  }
};

struct AddInteriorOp {  /* cheby_calc_u: u += p (cheby.cpp:41-64) */
  int x, y, hd;
  const double* p;
  double* u;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) u[i] = u[i] + p[i];
  }
};

struct PpcgInitOp {  /* TeaLeaf/c_kernels/sycl/ppcg.cpp:7-30 */
  int x, y, hd;
  double theta;
  double* sd;
  const double* r;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) sd[i] = r[i] / theta;
  }
};

struct PpcgCalcUrOp {  /* TeaLeaf/c_kernels/sycl/ppcg.cpp:33-63 */
  int x, y, hd;
  const double *sd, *kx, *ky;
  double *r, *u;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) {
      const double s = smvp(PlainLoad{sd}, kx, ky, i, x);
      r[i] = r[i] - s;
      u[i] = u[i] + sd[i];
    }
  }
};

struct PpcgCalcSdOp {  /* TeaLeaf/c_kernels/sycl/ppcg.cpp:66-94 */
  int x, y, hd;
  double alpha, beta;
  double* sd;
  const double* r;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd)) sd[i] = alpha * sd[i] + beta * r[i];
  }
};

/* --------------------------------------------------------------- halos */

constexpr int kMaxHaloFields = 8;
struct HaloFields {
  double* f[kMaxHaloFields];
  int n;
};

/* Left and right faces (TeaLeaf/c_kernels/sycl/local_halos.cpp:7-54) for
 * all fields: one thread per (field, row, layer, side). */
__global__ void halo_lr_kernel(HaloFields hf, int x, int y, int hd, int depth,
                               int do_left, int do_right) {
  const long total = (long)hf.n * y * depth * 2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const int side = (int)(t & 1);
    long rest = t >> 1;
    const int flip = (int)(rest % depth);
    rest /= depth;
    const int jj = (int)(rest % y);
    const int fi = (int)(rest / y);
    double* f = hf.f[fi];
    if (side == 0 && do_left) {
      f[(long)jj * x + hd - depth + flip] = f[(long)jj * x + hd + depth - flip - 1];
    } else if (side == 1 && do_right) {
      f[(long)jj * x + x - hd + flip] = f[(long)jj * x + x - hd - 1 - flip];
    }
  }
}

/* Top and bottom faces, full rows (local_halos.cpp:57-102). */
__global__ void halo_tb_kernel(HaloFields hf, int x, int y, int hd, int depth,
                               int do_bottom, int do_top) {
  const long total = (long)hf.n * x * depth * 2;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const int kk = (int)(t % x);
    long rest = t / x;
    const int side = (int)(rest & 1);
    rest >>= 1;
    const int line = (int)(rest % depth);
    const int fi = (int)(rest / depth);
    double* f = hf.f[fi];
    if (side == 1 && do_top) {
      f[(long)(y - hd + line) * x + kk] = f[(long)(y - hd - 1 - line) * x + kk];
    } else if (side == 0 && do_bottom) {
      f[(long)(hd - 1 - line) * x + kk] = f[(long)(hd + line) * x + kk];
    }
  }
}

int launch_halos(tl_context* ctx, int x, int y, int hd, int depth,
                 int face_mask, double* const* fields, int nfields) {
  if (nfields <= 0 || face_mask == 0) return TL_OK;
  TL_REQUIRE(depth >= 1 && depth <= hd, "halo depth must be in [1, halo_depth]");
  TL_REQUIRE(x - 2 * hd >= 1 && y - 2 * hd >= 1, "empty interior");
  const bool L = face_mask & (1 << TL_CHUNK_LEFT), R = face_mask & (1 << TL_CHUNK_RIGHT);
  const bool B = face_mask & (1 << TL_CHUNK_BOTTOM), T = face_mask & (1 << TL_CHUNK_TOP);
  for (int f0 = 0; f0 < nfields; f0 += kMaxHaloFields) {
    HaloFields hf;
    hf.n = std::min(kMaxHaloFields, nfields - f0);
    for (int k = 0; k < hf.n; ++k) {
      TL_REQUIRE(fields[f0 + k] != nullptr, "null halo field");
      hf.f[k] = fields[f0 + k];
    }
    /* Left and right may share a launch only when neither reads a layer
     * that the other writes (interior at least `depth` wide). */
    const bool lr_together = (x - 2 * hd) >= depth;
    const bool tb_together = (y - 2 * hd) >= depth;
    const long lr_threads = (long)hf.n * y * depth * 2;
    const long tb_threads = (long)hf.n * x * depth * 2;
    const int lr_blocks = (int)std::min<long>((lr_threads + 255) / 256, 4096);
    const int tb_blocks = (int)std::min<long>((tb_threads + 255) / 256, 4096);
    if (L || R) {
      if (lr_together || !(L && R)) {
        halo_lr_kernel<<<lr_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, L, R);
        TL_CHECK_LAUNCH(ctx);
      } else {
        halo_lr_kernel<<<lr_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, 1, 0);
        TL_CHECK_LAUNCH(ctx);
        halo_lr_kernel<<<lr_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, 0, 1);
        TL_CHECK_LAUNCH(ctx);
      }
    }
    if (T || B) {
      /* Reference order is T then B; they commute when disjoint. */
      if (tb_together || !(T && B)) {
        halo_tb_kernel<<<tb_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, B, T);
        TL_CHECK_LAUNCH(ctx);
      } else {
        halo_tb_kernel<<<tb_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, 0, 1);
        TL_CHECK_LAUNCH(ctx);
        halo_tb_kernel<<<tb_blocks, 256, 0, ctx->stream>>>(hf, x, y, hd, depth, 1, 0);
        TL_CHECK_LAUNCH(ctx);
      }
    }
  }
  return TL_OK;
}

__global__ void pack_kernel(int x, int y, int hd, int depth, int face, int pack,
                            double* field, double* buffer) {
  /* TeaLeaf/c_kernels/sycl/pack_halos.cpp:7-184 */
  const bool lr = (face == TL_CHUNK_LEFT || face == TL_CHUNK_RIGHT);
  const long n = lr ? (long)y * depth : (long)x * depth;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    long fi;
    if (lr) {
      const int jj = (int)(t / depth), d = (int)(t % depth);
      int col;
      if (face == TL_CHUNK_LEFT) col = pack ? hd : hd - depth;
      else col = pack ? x - hd - depth : x - hd;
      fi = (long)jj * x + col + d;
    } else {
      int row;
      if (face == TL_CHUNK_BOTTOM) row = pack ? hd : hd - depth;
      else row = pack ? y - hd - depth : y - hd;
      fi = (long)row * x + t;
    }
    if (pack) buffer[t] = field[fi];
    else field[fi] = buffer[t];
  }
}

/* -------------------------------------------------- persistent CG solve */

struct CgPersistParams {
  int x, y, hd, ntiles, max_iters;
  double eps, rro;
  double *u, *p, *r, *w;
  const double *kx, *ky, *diag;
  double *part_w, *part_r;
  double *pw_hist, *rrn_hist;
  unsigned* sync;
  int* status;
  int* steps_out;
};

/* Diagonal of the operator, (1 + (kx[i+1]+kx[i])) + (ky[i+x]+ky[i]), computed
 * once per solve with exactly the grouping of TeaLeaf/shared.h:60-61 so that
 * diag*a equals the first term of the operator bit for bit. */
struct DiagOp {
  int x, y, hd;
  const double *kx, *ky;
  double* diag;
  __device__ void operator()(unsigned i, int kk, int jj) const {
    if (interior(kk, jj, x, y, hd))
      diag[i] = 1.0 + (kx[i + 1] + kx[i]) + (ky[i + x] + ky[i]);
  }
};

constexpr int kWarpsPerTile = TL_GROUP / 8;  /* 8 warps x 8 groups = one tile */

/* The fused contract (kFused): w = diag p with the four neighbour terms
 * subtracted by fused multiply-adds in the order right, left, up, down. */
__device__ __forceinline__ double smvp_fused(double dg, double a, double kr, double ar,
                                             double kl, double al, double ku, double au,
                                             double kd, double ad) {
  double t = xmul<3>(dg, a);
  t = __fma_rn(-kr, ar, t);
  t = __fma_rn(-kl, al, t);
  t = __fma_rn(-ku, au, t);
  return __fma_rn(-kd, ad, t);
}

/* w = A p for the two cells i0, i0+1 of a lane (i0 even). Returns the
 * lane's first-level tree value of p.w: w0 p0 + w1 p1 (a cell outside the
 * interior contributes 0), or, fused, fma(w0, p0, w1 p1). kVec: the row
 * length x is even, so the pair lies in one row and every pair load is
 * 16-byte aligned; the left and right neighbours come from the adjacent
 * lanes. Otherwise scalar loads. */
template <bool kVec, bool kFused>
__device__ __forceinline__ double w_pair(const CgPersistParams& P, unsigned i0, unsigned len,
                                         int lane) {
  const int x = P.x, y = P.y, hd = P.hd;
  double w0 = 0.0, w1 = 0.0, a0 = 0.0, a1 = 0.0;
  if constexpr (kVec) {
    const int jj = (int)(i0 / (unsigned)x);
    const int kk0 = (int)(i0 - (unsigned)jj * (unsigned)x);
    const bool row = i0 < len && jj >= hd && jj < y - hd;
    double2 pc = make_double2(0.0, 0.0), pu = pc, pd = pc, kxp = pc, kyp = pc, kyu = pc,
            dg = pc;
    if (row) {
      pc = __ldcg(reinterpret_cast<const double2*>(P.p + i0));
      pu = __ldcg(reinterpret_cast<const double2*>(P.p + i0 + x));
      pd = __ldcg(reinterpret_cast<const double2*>(P.p + i0 - x));
      kxp = __ldg(reinterpret_cast<const double2*>(P.kx + i0));
      kyp = __ldg(reinterpret_cast<const double2*>(P.ky + i0));
      kyu = __ldg(reinterpret_cast<const double2*>(P.ky + i0 + x));
      dg = __ldg(reinterpret_cast<const double2*>(P.diag + i0));
    }
    double pl = __shfl_up_sync(TL_FULL_MASK, pc.y, 1);
    double pr = __shfl_down_sync(TL_FULL_MASK, pc.x, 1);
    double kx2 = __shfl_down_sync(TL_FULL_MASK, kxp.x, 1);
    const bool in0 = row && kk0 >= hd && kk0 < x - hd;
    const bool in1 = row && kk0 + 1 >= hd && kk0 + 1 < x - hd;
    if (lane == 0 && in0) pl = __ldcg(P.p + i0 - 1);
    if (lane == 31 && in1) {
      pr = __ldcg(P.p + i0 + 2);
      kx2 = __ldg(P.kx + i0 + 2);
    }
    if (in0) {
      const double s0 =
          kFused ? smvp_fused(dg.x, pc.x, kxp.y, pc.y, kxp.x, pl, kyu.x, pu.x, kyp.x, pd.x)
                 : xmul<1>(dg.x, pc.x) - (xmul<1>(kxp.y, pc.y) + xmul<1>(kxp.x, pl)) -
                       (xmul<1>(kyu.x, pu.x) + xmul<1>(kyp.x, pd.x));
      P.w[i0] = s0;
      w0 = s0;
      a0 = pc.x;
    }
    if (in1) {
      const double s1 =
          kFused ? smvp_fused(dg.y, pc.y, kx2, pr, kxp.y, pc.x, kyu.y, pu.y, kyp.y, pd.y)
                 : xmul<1>(dg.y, pc.y) - (xmul<1>(kx2, pr) + xmul<1>(kxp.y, pc.x)) -
                       (xmul<1>(kyu.y, pu.y) + xmul<1>(kyp.y, pd.y));
      P.w[i0 + 1] = s1;
      w1 = s1;
      a1 = pc.y;
    }
  } else {
    const double* __restrict__ kx = P.kx;
    const double* __restrict__ ky = P.ky;
    double wv[2] = {0.0, 0.0}, av[2] = {0.0, 0.0};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const unsigned i = i0 + h;
      if (i < len) {
        const int jj = (int)(i / (unsigned)x);
        const int kk = (int)(i - (unsigned)jj * (unsigned)x);
        if (interior(kk, jj, x, y, hd)) {
          const double pc = __ldcg(P.p + i);
          const double s =
              kFused ? smvp_fused(P.diag[i], pc, kx[i + 1], __ldcg(P.p + i + 1), kx[i],
                                  __ldcg(P.p + i - 1), ky[i + x], __ldcg(P.p + i + x), ky[i],
                                  __ldcg(P.p + i - x))
                     : xmul<1>(P.diag[i], pc) -
                           (xmul<1>(kx[i + 1], __ldcg(P.p + i + 1)) +
                            xmul<1>(kx[i], __ldcg(P.p + i - 1))) -
                           (xmul<1>(ky[i + x], __ldcg(P.p + i + x)) +
                            xmul<1>(ky[i], __ldcg(P.p + i - x)));
          P.w[i] = s;
          wv[h] = s;
          av[h] = pc;
        }
      }
    }
    w0 = wv[0]; w1 = wv[1]; a0 = av[0]; a1 = av[1];
  }
  if (kFused) return __fma_rn(w0, a0, xmul<3>(w1, a1));
  return xmul<2>(w0, a0) + xmul<2>(w1, a1);
}

/* u += alpha p, r -= alpha w for the two cells of a lane (fused: one
 * rounding each); returns the lane's first-level tree value of r.r,
 * r0 r0 + r1 r1 or, fused, fma(r0, r0, r1 r1). */
template <bool kVec, bool kFused>
__device__ __forceinline__ double ur_pair(const CgPersistParams& P, unsigned i0, unsigned len,
                                          double alpha) {
  const int x = P.x, y = P.y, hd = P.hd;
  auto upd_u = [alpha](double u, double p) {
    return kFused ? __fma_rn(alpha, p, u) : u + xmul<2>(alpha, p);
  };
  auto upd_r = [alpha](double r, double w) {
    return kFused ? __fma_rn(-alpha, w, r) : r - xmul<2>(alpha, w);
  };
  double r0 = 0.0, r1 = 0.0;
  if constexpr (kVec) {
    const int jj = (int)(i0 / (unsigned)x);
    const int kk0 = (int)(i0 - (unsigned)jj * (unsigned)x);
    const bool row = i0 < len && jj >= hd && jj < y - hd;
    const bool in0 = row && kk0 >= hd && kk0 < x - hd;
    const bool in1 = row && kk0 + 1 >= hd && kk0 + 1 < x - hd;
    if (in0 || in1) {
      const double2 uu = __ldcg(reinterpret_cast<const double2*>(P.u + i0));
      const double2 pp = __ldcg(reinterpret_cast<const double2*>(P.p + i0));
      const double2 rr = __ldcg(reinterpret_cast<const double2*>(P.r + i0));
      const double2 ww = __ldcg(reinterpret_cast<const double2*>(P.w + i0));
      if (in0 && in1) {
        const double2 un = make_double2(upd_u(uu.x, pp.x), upd_u(uu.y, pp.y));
        const double2 rn = make_double2(upd_r(rr.x, ww.x), upd_r(rr.y, ww.y));
        *reinterpret_cast<double2*>(P.u + i0) = un;
        *reinterpret_cast<double2*>(P.r + i0) = rn;
        r0 = rn.x;
        r1 = rn.y;
      } else if (in0) {
        P.u[i0] = upd_u(uu.x, pp.x);
        r0 = upd_r(rr.x, ww.x);
        P.r[i0] = r0;
      } else {
        P.u[i0 + 1] = upd_u(uu.y, pp.y);
        r1 = upd_r(rr.y, ww.y);
        P.r[i0 + 1] = r1;
      }
    }
  } else {
    double rv[2] = {0.0, 0.0};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const unsigned i = i0 + h;
      if (i < len) {
        const int jj = (int)(i / (unsigned)x);
        const int kk = (int)(i - (unsigned)jj * (unsigned)x);
        if (interior(kk, jj, x, y, hd)) {
          P.u[i] = upd_u(__ldcg(P.u + i), __ldcg(P.p + i));
          rv[h] = upd_r(__ldcg(P.r + i), __ldcg(P.w + i));
          P.r[i] = rv[h];
        }
      }
    }
    r0 = rv[0];
    r1 = rv[1];
  }
  if (kFused) return __fma_rn(r0, r0, xmul<3>(r1, r1));
  return xmul<2>(r0, r0) + xmul<2>(r1, r1);
}

/* One CG step loop of TeaLeaf/drivers/cg_driver.c:18-25 with the kernels of
 * TeaLeaf/c_kernels/sycl/cg.cpp:137-281, all on the device. A block of 1024
 * threads works on 4 tiles at a time (8 warps per tile, 8 groups of 64
 * cells per warp); blocks own tiles blockIdx.x*4 + k*gridDim.x*4 in every
 * phase. The p halo cells that the stencil reads (depth 1 on each face) are
 * written by the owner of the adjacent interior cell in the p update, which
 * yields the same values as the reference's halo update; corner and outer
 * halo cells are brought up to date by the exact halo update launched after
 * the loop. */
template <bool kVec, bool kFused>
__global__ void __launch_bounds__(kPersistThreads, 1)
cg_persistent_kernel(CgPersistParams P) {
  constexpr int kSub = kPersistThreads / 32 / kWarpsPerTile;  /* tiles per pass */
  __shared__ double s_group[kSub][TL_GROUP];
  __shared__ double s_scratch[TL_RED_SCRATCH];
  const int x = P.x, y = P.y, hd = P.hd;
  const unsigned len = (unsigned)x * (unsigned)y;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int sub = warp / kWarpsPerTile;       /* which tile of the pass */
  const int wt = warp % kWarpsPerTile;        /* warp within the tile */
  const int my_group = warp_sum8_group_of_lane(lane);
  double rro = P.rro;
  int steps = 0;
  const int stride = gridDim.x * kSub;

  for (int k = 0; k < P.max_iters; ++k) {
    /* ---- w = A p, pw partials (cg_calc_w) */
    for (int t0 = blockIdx.x * kSub; t0 < P.ntiles; t0 += stride) {
      const int tile = t0 + sub;
      if (tile < P.ntiles) {
        const unsigned base = (unsigned)tile * TL_TILE + (unsigned)wt * 8 * TL_GROUP;
        double v[8];
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          const unsigned i0 = base + (unsigned)g * TL_GROUP + 2u * lane;
          v[g] = w_pair<kVec, kFused>(P, i0, len, lane);
        }
        const double gs = warp_sum8_groups(v, lane);
        if (lane < 8) s_group[sub][wt * 8 + my_group] = gs;
      }
      __syncthreads();
      if (wt == 0 && tile < P.ntiles) {
        const double t = tl_tree64(s_group[sub][2 * lane], s_group[sub][2 * lane + 1]);
        if (lane == 0) P.part_w[tile] = t;
      }
      __syncthreads();
    }
    if (!tl_grid_barrier(P.sync, P.status)) break;
    const double pw = tl_reduce_partials(P.part_w, P.ntiles, s_scratch);
    const double alpha = rro / pw;

    /* ---- u += alpha p, r -= alpha w, rrn partials (cg_calc_ur) */
    for (int t0 = blockIdx.x * kSub; t0 < P.ntiles; t0 += stride) {
      const int tile = t0 + sub;
      if (tile < P.ntiles) {
        const unsigned base = (unsigned)tile * TL_TILE + (unsigned)wt * 8 * TL_GROUP;
        double v[8];
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          const unsigned i0 = base + (unsigned)g * TL_GROUP + 2u * lane;
          v[g] = ur_pair<kVec, kFused>(P, i0, len, alpha);
        }
        const double gs = warp_sum8_groups(v, lane);
        if (lane < 8) s_group[sub][wt * 8 + my_group] = gs;
      }
      __syncthreads();
      if (wt == 0 && tile < P.ntiles) {
        const double t = tl_tree64(s_group[sub][2 * lane], s_group[sub][2 * lane + 1]);
        if (lane == 0) P.part_r[tile] = t;
      }
      __syncthreads();
    }
    if (!tl_grid_barrier(P.sync, P.status)) break;
    const double rrn = tl_reduce_partials(P.part_r, P.ntiles, s_scratch);
    const double beta = rrn / rro;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      P.pw_hist[k] = pw;
      P.rrn_hist[k] = rrn;
    }

    /* ---- p = beta p + r (cg_calc_p), plus the depth-1 face halos of p */
    for (int t0 = blockIdx.x * kSub; t0 < P.ntiles; t0 += stride) {
      const unsigned base = (unsigned)t0 * TL_TILE;
      for (unsigned t = threadIdx.x; t < (unsigned)kSub * TL_TILE; t += blockDim.x) {
        const unsigned i = base + t;
        if (i >= len) break;
        const int jj = (int)(i / (unsigned)x);
        const int kk = (int)(i - (unsigned)jj * (unsigned)x);
        if (!interior(kk, jj, x, y, hd)) continue;
        const double pv = kFused ? __fma_rn(beta, __ldcg(P.p + i), __ldcg(P.r + i))
                                 : xmul<2>(beta, __ldcg(P.p + i)) + __ldcg(P.r + i);
        P.p[i] = pv;
        if (kk == hd) P.p[i - 1] = pv;
        if (kk == x - hd - 1) P.p[i + 1] = pv;
        if (jj == hd) P.p[i - x] = pv;
        if (jj == y - hd - 1) P.p[i + x] = pv;
      }
    }
    rro = rrn;
    steps = k + 1;
    if (sqrt(fabs(rrn)) < P.eps) break;
    if (!tl_grid_barrier(P.sync, P.status)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.steps_out = steps;
}

}  // namespace

/* ================================================================ ABI */

#define CTX_OK(ctx) TL_REQUIRE((ctx) != nullptr, "null context")
#define CELLS_OK(x, y)                                                                 \
  TL_REQUIRE((x) > 0 && (y) > 0 && (size_t)(x) * (size_t)(y) <= (size_t)TL_MAX_CELLS,  \
             "invalid grid dimensions (at most TL_MAX_CELLS cells)")
#define DIMS_OK(x, y, hd)                                                              \
  do {                                                                                 \
    TL_REQUIRE((x) > 2 * (hd) && (y) > 2 * (hd) && (hd) >= 1, "invalid grid dimensions"); \
    TL_REQUIRE((size_t)(x) * (size_t)(y) <= (size_t)TL_MAX_CELLS,                      \
               "grid larger than TL_MAX_CELLS (536,870,912 cells)");                   \
  } while (0)

extern "C" int tl_set_chunk_data_vertices(tl_context* ctx, int x, int y, int hd,
                                          double* vertex_x, double* vertex_y,
                                          double x_min, double y_min, double dx,
                                          double dy) {
  CTX_OK(ctx);
  TL_REQUIRE(vertex_x && vertex_y, "null vertex array");
  const int n = (x > y ? x : y) + 1;
  vertices_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(x, y, hd, vertex_x, vertex_y,
                                                             x_min, y_min, dx, dy);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

extern "C" int tl_set_chunk_data(tl_context* ctx, int x, int y, int hd,
                                 const double* vertex_x, const double* vertex_y,
                                 double* cell_x, double* cell_y, double* volume,
                                 double* x_area, double* y_area, double x_min,
                                 double y_min, double dx, double dy) {
  CTX_OK(ctx);
  (void)hd; (void)x_min; (void)y_min;
  return launch_map(ctx, ChunkDataOp{x, y, vertex_x, vertex_y, cell_x, cell_y, volume,
                                     x_area, y_area, dx, dy},
                    x, y);
}

extern "C" int tl_set_chunk_initial_state(tl_context* ctx, int x, int y,
                                          double default_energy,
                                          double default_density, double* energy0,
                                          double* density) {
  CTX_OK(ctx);
  CELLS_OK(x, y);
  return launch_map(ctx, InitialStateOp{default_energy, default_density, energy0, density},
                    x, y);
}

extern "C" int tl_set_chunk_state(tl_context* ctx, int x, int y, int hd,
                                  const tl_state* state, double* energy0,
                                  double* density, double* u, const double* cell_x,
                                  const double* cell_y, const double* vertex_x,
                                  const double* vertex_y) {
  CTX_OK(ctx);
  (void)hd;
  TL_REQUIRE(state != nullptr, "null state");
  return launch_map(ctx, StateOp{x, y, *state, energy0, density, u, cell_x, cell_y,
                                 vertex_x, vertex_y},
                    x, y);
}

extern "C" int tl_store_energy(tl_context* ctx, int x, int y, double* energy,
                               const double* energy0) {
  CTX_OK(ctx);
  CELLS_OK(x, y);
  return launch_map(ctx, CopyAllOp{energy, energy0}, x, y);
}

extern "C" int tl_update_face(tl_context* ctx, int x, int y, int hd,
                              double* field, int face, int depth) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(face >= 0 && face < 4, "invalid face");
  double* fields[1] = {field};
  return launch_halos(ctx, x, y, hd, depth, 1 << face, fields, 1);
}

extern "C" int tl_local_halos(tl_context* ctx, int x, int y, int hd, int depth,
                              int face_mask, double* const* fields, int nfields) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(nfields == 0 || fields != nullptr, "null field list");
  return launch_halos(ctx, x, y, hd, depth, face_mask, fields, nfields);
}

extern "C" int tl_pack_or_unpack(tl_context* ctx, int x, int y, int hd, int depth,
                                 int face, int pack, double* field, double* buffer) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(field && buffer, "null field or buffer");
  TL_REQUIRE(face >= 0 && face < 4 && depth >= 1 && depth <= hd, "invalid face or depth");
  const size_t n = (face == TL_CHUNK_LEFT || face == TL_CHUNK_RIGHT) ? (size_t)y * depth
                                                                      : (size_t)x * depth;
  int rc = tl_ensure_stage(ctx, n);
  if (rc != TL_OK) return rc;
  if (!pack) {
    TL_CUDA(cudaMemcpyAsync(ctx->d_stage, buffer, n * sizeof(double),
                            cudaMemcpyHostToDevice, ctx->stream));
  }
  pack_kernel<<<(int)std::min<size_t>((n + 255) / 256, 1024), 256, 0, ctx->stream>>>(
      x, y, hd, depth, face, pack, field, ctx->d_stage);
  TL_CHECK_LAUNCH(ctx);
  if (pack) {
    TL_CUDA(cudaMemcpyAsync(buffer, ctx->d_stage, n * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->stream));
  }
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_field_summary(tl_context* ctx, int x, int y, int hd,
                                const double* u, const double* density,
                                const double* energy0, const double* volume,
                                double* vol, double* mass, double* ie, double* temp) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(vol && mass && ie && temp, "null summary output");
  double out[4];
  int rc = launch_reduce(ctx, SummaryOp{u, density, energy0, volume}, x, y, hd, out);
  if (rc != TL_OK) return rc;
  *vol = out[0];
  *mass = out[1];
  *ie = out[2];
  *temp = out[3];
  return TL_OK;
}

static int cg_init_impl(tl_context* ctx, int x, int y, int hd, int coefficient,
                        double rx, double ry, double* p, double* r, double* u,
                        double* w, double* kx, double* ky, const double* density,
                        const double* energy, double* rro_sum) {
  int rc = launch_map(ctx, CgInitUOp{coefficient, p, r, u, w, density, energy, x, y}, x, y);
  if (rc != TL_OK) return rc;
  rc = launch_map(ctx, CgInitKOp{x, y, hd, w, kx, ky, rx, ry}, x, y);
  if (rc != TL_OK) return rc;
  return launch_reduce(ctx, CgInitOthersOp{x, kx, ky, u, p, r, w}, x, y, hd, rro_sum);
}

extern "C" int tl_cg_init(tl_context* ctx, int x, int y, int hd, int coefficient,
                          double rx, double ry, double* p, double* r, double* u,
                          double* w, double* kx, double* ky, const double* density,
                          const double* energy, double* rro) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(rro != nullptr, "null rro");
  double s = 0.0;
  int rc = cg_init_impl(ctx, x, y, hd, coefficient, rx, ry, p, r, u, w, kx, ky, density,
                        energy, &s);
  if (rc != TL_OK) return rc;
  *rro += s;
  return TL_OK;
}

extern "C" int tl_cg_calc_w(tl_context* ctx, int x, int y, int hd, double* w,
                            const double* p, const double* kx, const double* ky,
                            double* pw) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(pw != nullptr, "null pw");
  double s = 0.0;
  int rc = launch_reduce(ctx, CgCalcWOp{x, p, kx, ky, w}, x, y, hd, &s);
  if (rc != TL_OK) return rc;
  *pw += s;
  return TL_OK;
}

extern "C" int tl_cg_calc_ur(tl_context* ctx, int x, int y, int hd, double* u,
                             double* r, const double* p, const double* w,
                             double alpha, double* rrn) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(rrn != nullptr, "null rrn");
  double s = 0.0;
  int rc = launch_reduce(ctx, CgCalcUrOp{u, r, p, w, alpha}, x, y, hd, &s);
  if (rc != TL_OK) return rc;
  *rrn = s;
  return TL_OK;
}

extern "C" int tl_cg_calc_p(tl_context* ctx, int x, int y, int hd, double beta,
                            double* p, const double* r) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, CgCalcPOp{x, y, hd, beta, p, r}, x, y);
}

extern "C" int tl_copy_u(tl_context* ctx, int x, int y, int hd, const double* u,
                         double* u0) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, CopyUOp{x, y, hd, u, u0}, x, y);
}

int tl_internal_residual_norm(tl_context* ctx, int x, int y, int hd, const double* u,
                              const double* u0, double* r, const double* kx, const double* ky,
                              double* rr) {
  *rr = 0.0;
  return launch_reduce(ctx, ResidualNormOp{x, u, u0, kx, ky, r}, x, y, hd, rr);
}

extern "C" int tl_calculate_residual(tl_context* ctx, int x, int y, int hd,
                                     const double* u, const double* u0, double* r,
                                     const double* kx, const double* ky) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, ResidualOp{x, y, hd, u, u0, kx, ky, r}, x, y);
}

extern "C" int tl_calculate_2norm(tl_context* ctx, int x, int y, int hd,
                                  const double* buffer, double* norm) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(norm != nullptr, "null norm");
  double s = 0.0;
  int rc = launch_reduce(ctx, Norm2Op{buffer}, x, y, hd, &s);
  if (rc != TL_OK) return rc;
  *norm = s;
  return TL_OK;
}

extern "C" int tl_finalise(tl_context* ctx, int x, int y, int hd, const double* u,
                           const double* density, double* energy) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, FinaliseOp{x, y, hd, u, density, energy}, x, y);
}

extern "C" int tl_jacobi_init(tl_context* ctx, int x, int y, int hd, int coefficient,
                              double rx, double ry, double* u, double* u0,
                              const double* density, const double* energy, double* kx,
                              double* ky) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, JacobiInitOp{x, y, hd, coefficient, rx, ry, u, u0, kx, ky,
                                      density, energy},
                    x, y);
}

extern "C" int tl_jacobi_iterate(tl_context* ctx, int x, int y, int hd, double* u,
                                 const double* u0, double* r, const double* kx,
                                 const double* ky, double* error) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(error != nullptr, "null error");
  int rc = launch_map(ctx, CopyAllOp{r, u}, x, y);
  if (rc != TL_OK) return rc;
  double s = 0.0;
  rc = launch_reduce(ctx, JacobiIterateOp{x, u, u0, r, kx, ky}, x, y, hd, &s);
  if (rc != TL_OK) return rc;
  *error = s;
  return TL_OK;
}

extern "C" int tl_cheby_init(tl_context* ctx, int x, int y, int hd, double theta,
                             double* p, double* r, const double* u, const double* u0,
                             double* w, const double* kx, const double* ky) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, ChebyInitOp{x, y, hd, theta, p, r, w, u, u0, kx, ky}, x, y);
}

extern "C" int tl_cheby_iterate(tl_context* ctx, int x, int y, int hd, double alpha,
                                double beta, double* p, double* r, double* u,
                                const double* u0, double* w, const double* kx,
                                const double* ky) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  int rc = launch_map(ctx, ChebyIterateOp{x, y, hd, alpha, beta, p, r, w, u, u0, kx, ky},
                      x, y);
  if (rc != TL_OK) return rc;
  return launch_map(ctx, AddInteriorOp{x, y, hd, p, u}, x, y);
}

extern "C" int tl_ppcg_init(tl_context* ctx, int x, int y, int hd, double theta,
                            double* sd, const double* r) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  return launch_map(ctx, PpcgInitOp{x, y, hd, theta, sd, r}, x, y);
}

extern "C" int tl_ppcg_inner_iteration(tl_context* ctx, int x, int y, int hd,
                                       double theta, double alpha, double beta,
                                       double* sd, double* r, double* u,
                                       const double* kx, const double* ky) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  (void)theta;
  int rc = launch_map(ctx, PpcgCalcUrOp{x, y, hd, sd, kx, ky, r, u}, x, y);
  if (rc != TL_OK) return rc;
  return launch_map(ctx, PpcgCalcSdOp{x, y, hd, alpha, beta, sd, r}, x, y);
}

/* The persistent CG loop from a prepared state (r, p with its face halos,
 * rro = r.r), as in tl_cg_solve after its initialisation; also used by the
 * mixed-precision solver to finish in FP64. Leaves u and p with their final
 * depth-1 halos. pw_hist/rrn_hist (host) may be null. */
int tl_internal_cg64_loop(tl_context* ctx, int x, int y, int hd, double eps, int max_iters,
                          double* p, double* r, double* u, double* w, const double* kx,
                          const double* ky, double rro, double* pw_hist, double* rrn_hist,
                          int* steps) {
  *steps = 0;
  double* up[2] = {u, p};
  if (max_iters <= 0) return TL_OK;
  const size_t ntiles = tl_num_tiles(x, y);
  int rc = tl_ensure_partials(ctx, ntiles);
  if (rc != TL_OK) return rc;
  rc = tl_ensure_history(ctx, (size_t)max_iters);
  if (rc != TL_OK) return rc;
  rc = tl_ensure_diag(ctx, (size_t)x * y);
  if (rc != TL_OK) return rc;
  rc = launch_map(ctx, DiagOp{x, y, hd, kx, ky, ctx->d_diag}, x, y);
  if (rc != TL_OK) return rc;

  int per_sm = 0;
  /* Pair loads need an even row length (16-byte aligned pairs in one row). */
  const void* kernel =
      ctx->fp64_fused ? ((x % 2 == 0) ? (const void*)cg_persistent_kernel<true, true>
                                      : (const void*)cg_persistent_kernel<false, true>)
                      : ((x % 2 == 0) ? (const void*)cg_persistent_kernel<true, false>
                                      : (const void*)cg_persistent_kernel<false, false>);
  TL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistThreads, 0));
  TL_REQUIRE(per_sm >= 1, "persistent CG kernel cannot be resident");
  const int tiles_per_block = kPersistThreads / 32 / kWarpsPerTile;
  int grid = ctx->num_sms * std::min(per_sm, 1);
  const int needed = (int)((ntiles + tiles_per_block - 1) / tiles_per_block);
  if (grid > needed) grid = needed;

  CgPersistParams P;
  P.x = x; P.y = y; P.hd = hd; P.ntiles = (int)ntiles; P.max_iters = max_iters;
  P.eps = eps; P.rro = rro;
  P.u = u; P.p = p; P.r = r; P.w = w; P.kx = kx; P.ky = ky; P.diag = ctx->d_diag;
  P.part_w = ctx->d_part; P.part_r = ctx->d_part + ctx->part_cap;
  P.pw_hist = ctx->d_hist; P.rrn_hist = ctx->d_hist + ctx->hist_cap;
  P.sync = ctx->d_sync; P.status = ctx->d_status; P.steps_out = ctx->d_steps;
  TL_CUDA(cudaMemsetAsync(ctx->d_sync + TL_SYNC_BAR_COUNT, 0, 2 * sizeof(unsigned),
                          ctx->stream));
  TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  ctx->h_steps[0] = -1;
  void* args[] = {&P};
  TL_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
  TL_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(kPersistThreads), args, 0,
                                      ctx->stream));
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
  /* Final state of the u and p halos, as after the reference's last halo
   * update of the loop. */
  rc = launch_halos(ctx, x, y, hd, 1, 0xF, up, 2);
  if (rc != TL_OK) return rc;
  int status = 0;
  TL_CUDA(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                          ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  if (status != 0) {
    return tl_set_error(status, "persistent CG kernel reported a grid-barrier timeout");
  }
  const int n = ((volatile int*)ctx->h_steps)[0];
  TL_REQUIRE(n >= 0 && n <= max_iters, "persistent CG kernel did not report its steps");
  if (n > 0 && pw_hist && rrn_hist) {
    TL_CUDA(cudaMemcpyAsync(pw_hist, ctx->d_hist, (size_t)n * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->stream));
    TL_CUDA(cudaMemcpyAsync(rrn_hist, ctx->d_hist + ctx->hist_cap, (size_t)n * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  *steps = n;
  float ms = 0.0f;
  TL_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  ctx->last_solve.kernel_ms = ms;
  ctx->last_solve.steps = n;
  ctx->last_solve.kernel_launches = 1;
  return TL_OK;
}

/* CG from the current iterate u towards A u = u0: r = u0 - A u, p = r,
 * rro = r.r, then the persistent loop. */
int tl_internal_cg64_from_iterate(tl_context* ctx, int x, int y, int hd, double eps,
                                  int max_iters, double* p, double* r, double* u,
                                  const double* u0, double* w, const double* kx,
                                  const double* ky, int* steps) {
  double* up[2] = {u, p};
  int rc = launch_halos(ctx, x, y, hd, 1, 0xF, up, 1);
  if (rc != TL_OK) return rc;
  rc = launch_map(ctx, ResidualOp{x, y, hd, u, u0, kx, ky, r}, x, y);
  if (rc != TL_OK) return rc;
  rc = launch_map(ctx, CopyUOp{x, y, hd, r, p}, x, y);
  if (rc != TL_OK) return rc;
  rc = launch_halos(ctx, x, y, hd, 1, 0xF, up + 1, 1);
  if (rc != TL_OK) return rc;
  double rro = 0.0;
  rc = launch_reduce(ctx, Norm2Op{r}, x, y, hd, &rro);
  if (rc != TL_OK) return rc;
  return tl_internal_cg64_loop(ctx, x, y, hd, eps, max_iters, p, r, u, w, kx, ky, rro, nullptr,
                               nullptr, steps);
}

/* cg_init_driver of TeaLeaf/drivers/cg_driver.c:31-66 on the device:
 * initialisation kernels, halos of u and p, u0 = u; returns r.p. */
int tl_internal_cg_setup(tl_context* ctx, int x, int y, int hd, int coefficient, double rx,
                         double ry, double* p, double* r, double* u, double* u0, double* w,
                         double* kx, double* ky, const double* density, const double* energy,
                         double* rro) {
  *rro = 0.0;
  int rc = cg_init_impl(ctx, x, y, hd, coefficient, rx, ry, p, r, u, w, kx, ky, density,
                        energy, rro);
  if (rc != TL_OK) return rc;
  double* up[2] = {u, p};
  rc = launch_halos(ctx, x, y, hd, 1, 0xF, up, 2);
  if (rc != TL_OK) return rc;
  return launch_map(ctx, CopyUOp{x, y, hd, u, u0}, x, y);
}

/* The set-up of the solver-replacement path: cg_init_driver without
 * cg_init_others (that path computes its own true residual): u =
 * energy*density, kx, ky (skipped when the caller knows that they already
 * hold this density's values), halos of u and p, u0 = u. */
int tl_internal_cg_setup_lean(tl_context* ctx, int x, int y, int hd, int coefficient, double rx,
                              double ry, double* p, double* r, double* u, double* u0, double* w,
                              double* kx, double* ky, const double* density,
                              const double* energy, bool couplings_current) {
  int rc = launch_map(ctx, CgInitUOp{coefficient, p, r, u, w, density, energy, x, y}, x, y);
  if (rc != TL_OK) return rc;
  if (!couplings_current) {
    rc = launch_map(ctx, CgInitKOp{x, y, hd, w, kx, ky, rx, ry}, x, y);
    if (rc != TL_OK) return rc;
  }
  double* up[2] = {u, p};
  rc = launch_halos(ctx, x, y, hd, 1, 0xF, up, 2);
  if (rc != TL_OK) return rc;
  return launch_map(ctx, CopyUOp{x, y, hd, u, u0}, x, y);
}

extern "C" int tl_cg_solve(tl_context* ctx, int x, int y, int hd, int coefficient,
                           double rx, double ry, double eps, int max_iters, double* p,
                           double* r, double* u, double* u0, double* w, double* kx,
                           double* ky, const double* density, const double* energy,
                           double* rro0, double* pw_hist, double* rrn_hist, int* steps) {
  CTX_OK(ctx);
  DIMS_OK(x, y, hd);
  TL_REQUIRE(rro0 && steps && (max_iters == 0 || (pw_hist && rrn_hist)),
             "null output of tl_cg_solve");
  TL_REQUIRE(max_iters >= 0, "negative max_iters");
  *steps = 0;
  double rro = 0.0;
  int rc = tl_internal_cg_setup(ctx, x, y, hd, coefficient, rx, ry, p, r, u, u0, w, kx, ky,
                                density, energy, &rro);
  if (rc != TL_OK) return rc;
  *rro0 += rro;
  return tl_internal_cg64_loop(ctx, x, y, hd, eps, max_iters, p, r, u, w, kx, ky, rro,
                               pw_hist, rrn_hist, steps);
}

/* ====================================== allocation-free cg_calc_w variant
 *
 * tl_cg_calc_w_noalloc computes exactly what tl_cg_calc_w computes (same
 * kernel, same summation order, same bits) without a context and without
 * allocating anything: its reduction scratch (one partial per 4096-cell
 * tile, the final sum and the last-block ticket) lives in the fixed array
 * below, which every GPU that loads this library holds until the process
 * exits. Host code may not use the array's name as a device address, so the
 * address is looked up with cudaGetSymbolAddress, once per device, on the
 * first call made while that device is current. */
#define TL_NOALLOC_MAX_TILES 32768 /* 32768 tiles = 134,217,728 cells */

static __device__ __align__(256) double g_noalloc_scratch[TL_NOALLOC_MAX_TILES + 2];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_address[kNoallocMaxDevices] = {};
}  // namespace

extern "C" int tl_cg_calc_w_noalloc(void* stream, int x, int y, int hd, double* w,
                                    const double* p, const double* kx, const double* ky,
                                    double* pw) {
  TL_REQUIRE(x > 2 * hd && y > 2 * hd && hd >= 1, "invalid grid dimensions");
  const size_t ntiles = tl_num_tiles(x, y);
  if (ntiles > TL_NOALLOC_MAX_TILES) {
    return tl_set_error(TL_ERR_ARG,
                        "tl_cg_calc_w_noalloc: grid of " + std::to_string((size_t)x * y) +
                            " cells exceeds the fixed scratch limit of 134217728 cells "
                            "(32768 tiles of 4096)");
  }
  TL_REQUIRE(w && p && kx && ky && pw, "tl_cg_calc_w_noalloc: null argument");
  int dev = 0;
  TL_CUDA(cudaGetDevice(&dev));
  TL_REQUIRE(dev >= 0 && dev < kNoallocMaxDevices, "tl_cg_calc_w_noalloc: device ordinal");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_address[dev]) {
      void* addr = nullptr;
      TL_CUDA(cudaGetSymbolAddress(&addr, g_noalloc_scratch));
      g_noalloc_address[dev] = (double*)addr;
    }
    scratch = g_noalloc_address[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* result = scratch + TL_NOALLOC_MAX_TILES;
  unsigned* ticket = (unsigned*)(scratch + TL_NOALLOC_MAX_TILES + 1);
  TL_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
  reduce_kernel<CgCalcWOp><<<(unsigned)ntiles, kRedThreads, 0, s>>>(
      CgCalcWOp{x, p, kx, ky, w}, x, y, hd, scratch, (size_t)TL_NOALLOC_MAX_TILES,
      (int)ntiles, ticket, result);
  TL_CUDA(cudaGetLastError());
  double sum = 0.0;
  TL_CUDA(cudaMemcpyAsync(&sum, result, sizeof(double), cudaMemcpyDeviceToHost, s));
  TL_CUDA(cudaStreamSynchronize(s));
  *pw += sum;
  return TL_OK;
}
