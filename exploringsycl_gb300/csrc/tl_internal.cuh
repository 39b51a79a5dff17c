/*
 * tl_internal.cuh -- shared internals of the GB300 TeaLeaf backend:
 * the context, error reporting, the deterministic reduction primitives and
 * the bounded grid barrier of the persistent kernels.
 *
 * Reduction order. Every dot product is summed exactly as the reference
 * sums it: values of 64 consecutive linear cells (halo cells contribute 0)
 * are combined by a pairwise tree whose stride doubles from 1 to 32
 * (TeaLeaf/c_kernels/sycl/cg.cpp:113-126), and the resulting partial sums
 * are reduced level by level by the same 64-wide tree, padded with zeros
 * (TeaLeaf/c_kernels/sycl/sycl_shared.hpp:35-79).
 *
 * On the GPU a warp holds one 64-cell group, two consecutive cells per lane:
 * the in-lane add is the stride-1 level, and a butterfly of shuffles with
 * lane masks 1, 2, 4, 8, 16 performs the stride-2..32 levels (IEEE addition
 * is commutative, so both partners of each butterfly step compute the same
 * bits). A thread block processes "tiles" of 64 groups = 4096 consecutive
 * cells and folds the 64 group sums of a tile with the same warp tree, giving
 * one second-level partial per tile. Whatever reduces those tile partials
 * (the last block of a step-wise kernel, or every block of a persistent
 * kernel after its grid barrier) continues the tree level by level.
 */
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "tealeaf_gb300.h"

#define TL_GROUP 64                       /* cells per first-level group */
#define TL_TILE (TL_GROUP * TL_GROUP)     /* cells per tile (4096) */
#define TL_MAX_TILES (1 << 17)            /* grids up to 5.4e8 cells */
static_assert((long long)TL_MAX_TILES * TL_TILE == TL_MAX_CELLS,
              "the public grid limit is the reduction scratch's");
/* Shared scratch of a block-wide reduction of up to TL_MAX_TILES partials:
 * the first level (TL_MAX_TILES/64 values), then the smaller levels. */
#define TL_RED_SCRATCH (TL_MAX_TILES / TL_GROUP + TL_MAX_TILES / TL_TILE + 64)
#define TL_FULL_MASK 0xffffffffu

/* Result slots in the pinned result page. */
#define TL_SLOT_A 0
#define TL_SLOT_B 1
#define TL_SLOT_C 2
#define TL_SLOT_D 3
#define TL_NUM_SLOTS 8

/* Sync words in device scratch. */
#define TL_SYNC_TICKET 0     /* last-block tickets, one per slot group */
#define TL_SYNC_BAR_COUNT 8  /* grid barrier arrival counter */
#define TL_SYNC_BAR_GEN 9    /* grid barrier generation */
#define TL_SYNC_WORDS 16

/* How long a block waits at a grid barrier before it gives up and reports
 * TL_ERR_TIMEOUT (nanoseconds of %globaltimer). */
#define TL_BARRIER_BUDGET_NS 2000000000ull

struct tl_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;

  double* d_part = nullptr;       /* 4 tile-partial arrays of part_cap doubles */
  size_t part_cap = 0;
  unsigned* d_sync = nullptr;     /* TL_SYNC_WORDS words */
  int* d_status = nullptr;        /* kernel-reported error code */
  double* h_result = nullptr;     /* pinned, mapped: TL_NUM_SLOTS doubles */
  double* d_result = nullptr;     /* device alias of h_result */
  int* h_steps = nullptr;         /* pinned, mapped: persistent-solve counters */
  int* d_steps = nullptr;
  double* d_hist = nullptr;       /* 2 x hist_cap doubles of per-step scalars */
  size_t hist_cap = 0;
  double* d_stage = nullptr;      /* halo pack staging */
  double* d_diag = nullptr;       /* operator diagonal of the current solve */
  float* d_f32 = nullptr;         /* mixed-precision solver fields (8 x f32_cap) */
  size_t f32_cap = 0;
  size_t diag_cap = 0;
  size_t stage_cap = 0;
  long long launches = 0;
  cudaEvent_t ev_start = nullptr;  /* around the persistent kernel of a solve */
  cudaEvent_t ev_stop = nullptr;
  tl_solve_stats last_solve = {0.0f, 0, 0};
  int fp64_fused = 0;             /* TL_FP64_FUSED: the persistent FP64 CG uses FMAs */
  /* coarse level of the two-level learned PCG (tl_coarse.cu): the FP32
   * inverse of the coarse operator of the couplings last seen and the FP16
   * copy the kernel reads, kept while they do not change, and its per-step
   * vectors */
  float* d_ainv = nullptr;        /* nc x nc, row-major */
  size_t ainv_cap = 0;
  __half* d_ainv16 = nullptr;     /* the same times 2^coarse_exp, FP16 */
  size_t ainv16_cap = 0;
  int coarse_exp = 0;
  double* d_coarse_work = nullptr; /* the inverse's FP64 columns, then the bands */
  size_t coarse_work_cap = 0;
  float* d_coarse_vec = nullptr;  /* tile restriction partials, then e_c */
  size_t coarse_vec_cap = 0;
  unsigned long long* d_hash = nullptr;
  int coarse_H = 0, coarse_W = 0, coarse_blk = 0;
  unsigned long long coarse_hash = 0;
  /* starting guesses of tl_solve (tl_project.cu): the newest solution X of
   * the operator last seen (slot proj_xslot) and the differences of
   * consecutive solutions before it (slots proj_order, oldest first), in
   * proj_slots fields of proj_field_cap doubles, proj_count vectors held;
   * proj_gram[i][j] = v_i . A v_j by slot; the operator they belong to */
  double* d_proj = nullptr;
  size_t proj_field_cap = 0;
  int proj_slots = 0, proj_count = 0, proj_xslot = 0;
  int proj_order[TL_PROJ_MAX] = {0};
  double proj_gram[TL_PROJ_MAX][TL_PROJ_MAX] = {{0.0}};
  double* d_proj_part = nullptr;  /* block partials of the dot products */
  int proj_x = 0, proj_y = 0, proj_hd = 0;
  int proj_last_n = 0;            /* the last guess: its basis slots and coefficients */
  int proj_last_slot[TL_PROJ_MAX] = {0};
  double proj_last_coef[TL_PROJ_MAX] = {0.0};
  /* the operator tl_solve's replacement path saw last: x, y, hd, the hash of
   * density with rx, ry and the coefficient kind, and the hash of the kx,
   * ky it computed from them (cg_init's couplings are recomputed only when
   * one of them changed); the FP32 coefficients packed from that operator
   * (packed_kind 1: the learned solvers' packed layout, 2: the halo layout) */
  int op_x = 0, op_y = 0, op_hd = 0;
  unsigned long long op_dens_hash = 0, op_k_hash = 0;
  int packed_kind = 0;
  unsigned long long packed_hash = 0;
  unsigned long long* d_hash64 = nullptr;
  /* the diagonal of that operator (FP64, x*y), for the replacement path */
  double* d_diag64 = nullptr;
  size_t diag64_cap = 0;
  unsigned long long diag64_id = 0;
  unsigned long long proj_hash = 0;
};

/* The coarse level of a packed [H][W] field: blk x blk aggregates
 * (blk = 1 << blk_shift), an ncx x ncy coarse grid of nc unknowns, the
 * inverse of its operator P^T A P (FP32, row-major nc x nc) and its FP16
 * copy (entries times 2^exp16, so that the largest lies in [2^14, 2^15)),
 * the per-tile restriction partials (8 per 128 x 64 tile) and the coarse
 * correction e_c. */
struct tl_coarse_level {
  int blk_shift, ncx, ncy, nc;
  const float* ainv;
  const __half* ainv16;
  int exp16;
  float* rc_part;
  float* ec;
};

/* Set-up of tl_solve's replacement path (tl_fp64.cu): cg_init_driver
 * without cg_init_others; kx, ky are left as they are when
 * couplings_current. */
int tl_internal_cg_setup_lean(tl_context* ctx, int x, int y, int hd, int coefficient, double rx,
                              double ry, double* p, double* r, double* u, double* u0, double* w,
                              double* kx, double* ky, const double* density,
                              const double* energy, bool couplings_current);

/* 64-bit content hashes of n doubles in one pass (tl_project.cu): *out_a
 * of a (mixed with salt_a; a may be NULL), *out_bc of b and c together (c
 * may be NULL; b NULL leaves *out_bc alone). */
int tl_internal_hash64(tl_context* ctx, const double* a, const double* b, const double* c,
                       size_t n, unsigned long long salt_a, unsigned long long* out_a,
                       unsigned long long* out_bc);

/* r = u0 - A u over the interior (calc_residual) and r.r (calc_2norm of r)
 * in one pass, both bit-identical to the two kernels (tl_fp64.cu). */
int tl_internal_residual_norm(tl_context* ctx, int x, int y, int hd, const double* u,
                              const double* u0, double* r, const double* kx, const double* ky,
                              double* rr);

/* Starting guess of tl_solve from the solutions of earlier solves with the
 * same operator (tl_project.cu): writes the guess into u's interior and the
 * number of basis directions kept into *basis (0: none, u untouched); *bb
 * receives b.b when solutions were held (the pass that sums them), and is
 * left alone otherwise. After
 * the solve, push records the solution u with its true residual
 * r = b - A u. */
int tl_internal_project_guess(tl_context* ctx, int slots, int x, int y, int hd,
                              unsigned long long op_hash, const double* b, double* u,
                              int* basis, double* bb);
/* Writes the last guess into u again (after u was overwritten). */
int tl_internal_project_recombine(tl_context* ctx, int x, int y, int hd, double* u);
int tl_internal_project_push(tl_context* ctx, int x, int y, int hd, const double* b,
                             const double* u, const double* r, const double* kx,
                             const double* ky, const double* diag);

/* Thread-local error message and helpers (tl_context.cu). */
int tl_set_error(int code, const std::string& msg);
int tl_cuda_error(cudaError_t e, const char* what, const char* file, int line);
int tl_ensure_partials(tl_context* ctx, size_t ntiles);
int tl_ensure_history(tl_context* ctx, size_t n);
int tl_ensure_stage(tl_context* ctx, size_t n);
int tl_ensure_diag(tl_context* ctx, size_t n);

/* Internal entry points of tl_fp64.cu shared with the other solvers. */
int tl_internal_cg_setup(tl_context* ctx, int x, int y, int hd, int coefficient, double rx,
                         double ry, double* p, double* r, double* u, double* u0, double* w,
                         double* kx, double* ky, const double* density, const double* energy,
                         double* rro);
int tl_internal_cg64_loop(tl_context* ctx, int x, int y, int hd, double eps, int max_iters,
                          double* p, double* r, double* u, double* w, const double* kx,
                          const double* ky, double rro, double* pw_hist, double* rrn_hist,
                          int* steps);
struct tl_net;
int tl_internal_unpack_add(tl_context* ctx, int x, int y, int hd, const float* e,
                           double inv_scale, double* u);
int tl_internal_fpcg_learned(tl_context* ctx, tl_net* net, int H, int W, const float* kx,
                             const float* ky, const float* s, float* r, float* e, float* p,
                             float* w, float* z, double tol, int max_iters, int* iters);
/* The learned preconditioner collapsed to one stencil (tl_precond.cu). */
int tl_internal_net_stencil(tl_net* net, const void** umma, const float** kscale);
int tl_internal_apply_collapsed(tl_context* ctx, const void* umma, const float* kscale, int H,
                                int W, const float* r, const float* s, float* z);
int tl_internal_fpcg_collapsed(tl_context* ctx, const void* umma, const float* kscale, int H,
                               int W, const float* kx, const float* ky, const float* s,
                               float* r, float* r_alt, float* e, float* w, float* z, float* pa,
                               float* pb, double tol, int max_iters, int* iters,
                               double* rr_final, const tl_coarse_level* coarse = nullptr);
/* The coarse level for the couplings kx, ky of a packed [H][W] field
 * (tl_coarse.cu): rebuilt only when H, W or the couplings change. A caller
 * that knows a content hash of the couplings passes it in known_hash (the
 * coarse level then skips its own). */
int tl_internal_coarse_prepare(tl_context* ctx, int H, int W, const float* kx, const float* ky,
                               tl_coarse_level* out, const unsigned long long* known_hash = nullptr);
int tl_internal_cg64_from_iterate(tl_context* ctx, int x, int y, int hd, double eps,
                                  int max_iters, double* p, double* r, double* u,
                                  const double* u0, double* w, const double* kx,
                                  const double* ky, int* steps);

#define TL_CUDA(call)                                                      \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) return tl_cuda_error(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define TL_CHECK_LAUNCH(ctx)                                               \
  do {                                                                     \
    (ctx)->launches++;                                                     \
    cudaError_t e_ = cudaGetLastError();                                   \
    if (e_ != cudaSuccess) return tl_cuda_error(e_, "kernel launch", __FILE__, __LINE__); \
  } while (0)

#define TL_REQUIRE(cond, msg)                                              \
  do {                                                                     \
    if (!(cond)) return tl_set_error(TL_ERR_ARG, msg);                     \
  } while (0)

static inline size_t tl_num_tiles(int x, int y) {
  return ((size_t)x * (size_t)y + TL_TILE - 1) / TL_TILE;
}

/* ----------------------------------------------------------- device side */

/* Pairwise 64-wide tree over two values per lane (cells 2*lane, 2*lane+1
 * of the group); every lane returns the group sum. */
__device__ __forceinline__ double tl_tree64(double a, double b) {
  double v = a + b;
  v = v + __shfl_xor_sync(TL_FULL_MASK, v, 1);
  v = v + __shfl_xor_sync(TL_FULL_MASK, v, 2);
  v = v + __shfl_xor_sync(TL_FULL_MASK, v, 4);
  v = v + __shfl_xor_sync(TL_FULL_MASK, v, 8);
  v = v + __shfl_xor_sync(TL_FULL_MASK, v, 16);
  return v;
}

/* Reduces n tile partials (global memory, written by other blocks before a
 * grid-wide synchronisation) to one value in the reference order, using the
 * whole block. `scratch` is shared memory of TL_RED_SCRATCH doubles; the
 * first level goes to scratch[0, ceil(n/64)) and later levels alternate
 * with the region after it, which each smaller level fits. Every thread
 * returns the same value. */
__device__ __forceinline__ double tl_reduce_partials(const double* part, int n,
                                                     double* scratch) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  int ng = (n + TL_GROUP - 1) / TL_GROUP;
  double* src = scratch;
  double* dst = scratch + ng;
  for (int g = warp; g < ng; g += nwarps) {
    const int i0 = g * TL_GROUP + 2 * lane;
    const double a = (i0 < n) ? __ldcg(part + i0) : 0.0;
    const double b = (i0 + 1 < n) ? __ldcg(part + i0 + 1) : 0.0;
    const double s = tl_tree64(a, b);
    if (lane == 0) src[g] = s;
  }
  __syncthreads();
  n = ng;
  while (n > 1) {
    ng = (n + TL_GROUP - 1) / TL_GROUP;
    for (int g = warp; g < ng; g += nwarps) {
      const int i0 = g * TL_GROUP + 2 * lane;
      const double a = (i0 < n) ? src[i0] : 0.0;
      const double b = (i0 + 1 < n) ? src[i0 + 1] : 0.0;
      const double s = tl_tree64(a, b);
      if (lane == 0) dst[g] = s;
    }
    __syncthreads();
    double* t = src;
    src = dst;
    dst = t;
    n = ng;
  }
  const double total = src[0];
  __syncthreads();
  return total;
}

__device__ __forceinline__ unsigned long long tl_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* Grid-wide barrier for co-resident blocks (cooperative launch): waits until
 * `expected` blocks have arrived. Spins for at most `budget_ns` of
 * %globaltimer; on expiry it records TL_ERR_TIMEOUT in *status and returns
 * false instead of waiting further. Returns false as well when any block has
 * recorded an error, so that all blocks leave their loops together. */
__device__ __forceinline__ bool tl_grid_barrier_n(unsigned* sync, int* status,
                                                  unsigned expected,
                                                  unsigned long long budget_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* gen = sync + TL_SYNC_BAR_GEN;
    const unsigned my_gen = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(sync + TL_SYNC_BAR_COUNT, 1u);
    if (arrived == expected - 1) {
      atomicExch(sync + TL_SYNC_BAR_COUNT, 0u);
      __threadfence();
      atomicAdd(sync + TL_SYNC_BAR_GEN, 1u);
    } else {
      const unsigned long long t0 = tl_globaltimer();
      while (*gen == my_gen) {
        if (tl_globaltimer() - t0 > budget_ns) {
          atomicCAS(status, 0, TL_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __threadfence();
    if (*(volatile int*)status != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool tl_grid_barrier(unsigned* sync, int* status) {
  return tl_grid_barrier_n(sync, status, gridDim.x, TL_BARRIER_BUDGET_NS);
}
