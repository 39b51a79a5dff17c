/*
 * tl_precond.cu -- the learned preconditioner collapsed to one stencil, and
 * the persistent PCG kernel of the mixed-precision solver that
 * applies it on the tensor cores.
 *
 * Collapse. The network of tl_learned.cu has no bias and no activation, so
 * between its two diagonal scalings it is a linear, translation-invariant
 * operator: the four 3x3 layers compose to C r = sum_u G(u) r(. + u) with a
 * 16-channel 9x9 kernel G, and the adjoint stack C^T C is the 17x17 stencil
 *   K(d) = sum_u G(u) . G(u + d),      z = D^-1 r + S (K * (S r)),
 * where (K * y)(j) = sum_d K(d) y(j + d). K is the autocorrelation of G:
 * symmetric, with a non-negative Fourier transform. More than 8 cells from
 * the domain edge the stencil and the layer-by-layer network are the same
 * operator (tests check this to rounding); at the edge the stencil acts on
 * the zero-extended field once instead of truncating every layer, so S K S
 * is a principal submatrix of a positive semi-definite Toeplitz operator and
 * M^-1 stays symmetric positive definite. Cost: 289 multiply-adds per cell
 * against ~28 k for the eight 16-channel layers. K and its tensor-core
 * operands are built on the device from the FP32 master weights whenever the
 * weights change (tl_learned.cu, collapse_kernel).
 *
 * Tensor cores (tcgen05). For one row offset dy, correlating a row with
 * K(dy, .) is a product with a banded Toeplitz matrix. A 16-column input
 * window reaches 32 output columns, so one MMA of M = 128 tile rows, N = 32,
 * K = 16 (FP16 inputs, FP32 accumulation in tensor memory, lane = tile row)
 * per window and dy: 85 per 128 x 64 tile, issued by one thread. The A
 * operand is the staged y = sigma S r in the canonical K-major layout
 * (tl_tc05.cuh): chunks of 8 staged columns, each 144 rows x 16 bytes, so a
 * window is two consecutive chunks and the row offset dy a shift of the
 * start address by 16 (dy + 8) bytes. sigma = 1 / RMS(r) keeps y in FP16's
 * normal range whatever the residual's size (the operator is linear; the
 * factor is removed in the epilogue), and K is scaled by a power of two for
 * the same reason. The output ranges of neighbouring windows overlap, so
 * even and odd windows accumulate into separate tensor-memory columns, and
 * the epilogue adds the two.
 *
 * PCG (beta = z_new.r_new / z_old.r_old: M^-1 is a fixed linear SPD operator,
 * and the Polak-Ribiere form of flexible PCG measured the same step counts),
 * on the packed interior [H][W] with zero-flux edges, one cooperative
 * persistent kernel of one 1024-thread block per SM, two phases and two grid
 * barriers per step:
 *   P: (all warps) p_new = z + beta p_old at the cell and its four
 *      neighbours, w = A p_new, p.w partial sums, and the previous step's
 *      e += alpha p_old;
 *   Z: warp 0 issues each tile's MMAs and commits them to an mbarrier;
 *      warps 1..31 stage the next tile: r_new = r_old - alpha w, written to
 *      memory for the tile's own cells, and with its 8-cell halo as y (FP16)
 *      into one of two staging buffers; then they finish the previous tile:
 *      eight of them move its accumulators from tensor memory into a
 *      row-major shared tile, and all of them read r_new back (from L2) and
 *      write z = S K y / sigma + D^-1 r_new with coalesced stores and sum
 *      r.r and r.z. Staged tiles and accumulators are double-buffered, so
 *      the tensor core works while the block streams memory.
 * The residual is double-buffered because a tile reads its neighbours' old
 * residual while they write the new one. Memory per cell and step: P reads z,
 * p_old, kx, ky, e and writes p_new, w, e (32 B); Z reads r, w, s and writes r,
 * z (20 B): 52 B, against 56 B for the Jacobi-PCG kernel of tl_mixed.cu. The
 * last step's e update is one extra pass at the end. Tiles of phase Z are
 * visited in reverse order so that the cells phase P wrote last are still in
 * L2. Every mbarrier wait is bounded; tensor memory is freed after a final
 * commit on every exit path.
 */
#include <cuda_fp16.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tl_internal.cuh"
#include "tl_tc05.cuh"

namespace {

constexpr int kThreads = 1024;          /* 32 warps, one block per SM */
constexpr int kIssuers = 1;             /* phase Z: warp 0 issues the MMAs */
constexpr int kWorkers = kThreads - 32 * kIssuers;  /* warps 1..31 stage and finish tiles */
constexpr int kChunk = 4 * kThreads;    /* phase P: cells per block iteration */
constexpr int kHalo = 8;
constexpr int kTH = 128;                /* tile rows = MMA M = tensor-memory lanes */
constexpr int kTW = 64;                 /* tile columns */
constexpr int kRows = kTH + 2 * kHalo;  /* 144 staged rows */
constexpr int kGroups = (kTW + 2 * kHalo) / 4;  /* float4 groups per staged row */
constexpr int kWindows = kTW / 16 + 1;          /* 16-column input windows per tile */
/* A operand: ten K-major chunks of 8 staged columns, each 144 rows x 16 B,
 * +16 B so that the 8-byte stores of one staged row spread over the banks */
constexpr int kChunkBytes = kRows * 16 + 16;
constexpr int kABytes = (kTW + 2 * kHalo) / 8 * kChunkBytes;
constexpr int kABuf = (kABytes + 127) / 128 * 128;
constexpr int kBBytes = 17 * 1024;      /* 17 B operands (one per dy) of 32 x 16 FP16 */
constexpr int kZStride = kTW + 4;       /* floats per row of the accumulator hand-over */
/* accumulators per buffer: even windows into columns 0..95 (tile column c at
 * 16 + c), odd windows into 96..159 (tile column c at 96 + c); two buffers */
constexpr uint32_t kDCols = 160;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kIdesc = tc05::idesc_f16_f32<kTH, 32>();
constexpr unsigned long long kWaitNs = 1000000000ull;  /* bound of every mbarrier wait */
constexpr int kReaders = 8;             /* warps 4..11 move accumulators to shared memory */
constexpr int kBarWorkers = 1;          /* named barrier of the worker warps */

/* dynamic shared memory */
constexpr int kOffA0 = 0;
constexpr int kOffA1 = kABuf;
constexpr int kOffB = 2 * kABuf;
constexpr int kOffZ = kOffB + kBBytes;
/* mbarriers: a_full[2], mma_done[2][kIssuers], d_free[2], drain */
constexpr int kOffBar = kOffZ + kTH * kZStride * 4;
constexpr int kOffTmem = kOffBar + (5 + 2 * kIssuers) * 8;
constexpr int kLpcgSmem = (kOffTmem + 8 + 127) / 128 * 128;
/* two-level kernel: the epilogue's restriction sums of the tile row pairs
 * (two tiles in flight x 64 pairs x 2 aggregate columns), then r_c and e_c */
constexpr int kMaxCoarse = 4096;
static_assert(kMaxCoarse % kThreads == 0, "coarse vectors are split evenly over a block");
constexpr int kRestSlots = 8;           /* restriction partials per tile */
constexpr int kOffRest = kLpcgSmem;
constexpr int kOffCoarse = kOffRest + 2 * (kTH / 2) * 2 * 4;
constexpr int kLpcgSmemCoarse = kOffCoarse + 2 * kMaxCoarse * 4;
static_assert(kOffB % 128 == 0 && kOffZ % 16 == 0 && kOffBar % 8 == 0,
              "alignment");
static_assert(kLpcgSmemCoarse <= 227 * 1024, "shared memory");
static_assert(2 * kDCols <= kTmemCols, "tensor memory");

struct LpcgParams {
  int H, W, chunks, tiles_x, tiles, max_iters;
  double tol2;
  const float *kx, *ky, *s;
  float *r0, *r1;  /* residual, double-buffered (r0 holds the incoming one) */
  float *e, *w, *z, *p0, *p1;
  const __half* umma;  /* window B operands, 17 x 32 x 16 FP16 */
  const float* kscale;
  double* part;  /* 3 arrays of gridDim.x partial sums: p.w, r.r, r.z */
  /* coarse level (two-level kernel only): blk = 1 << cshift aggregates on an
   * ncx-wide coarse grid of nc unknowns, Ac^-1 as FP16 (nc x nc, entries
   * times 2^e; ainv_unscale = 2^-e), the tiles' restriction partials (8 per
   * tile) and the correction e_c */
  int cshift, ncx, nc;
  const __half* ainv;
  float ainv_unscale;
  float* rc_part;
  float* ec;
  unsigned* sync;
  int* status;
  int* iters_out;
  double* rr_out;
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TL_FULL_MASK, v, o);
  return v;
}

/* Block-wide sum in a fixed order; every thread returns it. */
__device__ __forceinline__ float block_sum(float v, float* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  float t = lane < (int)(blockDim.x >> 5) ? s_red[lane] : 0.0f;
  t = warp_sum(t);
  __syncthreads();
  return t;
}

/* Sum of n doubles written by other blocks before a grid barrier, in one
 * fixed order (lane-strided sequential sums, then a butterfly), so that
 * every block obtains the same bits. */
__device__ __forceinline__ double sum_partials(const double* part, int n, double* s_one) {
  if (threadIdx.x < 32) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(part + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TL_FULL_MASK, v, o);
    if (threadIdx.x == 0) *s_one = v;
  }
  __syncthreads();
  const double t = *s_one;
  __syncthreads();
  return t;
}

__device__ __forceinline__ float4 ld4(const float* p) {
  return __ldcg(reinterpret_cast<const float4*>(p));
}

__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;\n" :: "r"(id), "r"(n) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n"
               :: "r"(tc05::smem_addr(mbar)) : "memory");
}

/* ------------------------------------------------------------ phase P */

/* p_new = z + beta p_old, w = A p_new, p.w; and the previous step's
 * e += alpha_prev p_old (p_old is loaded here anyway). Two-level kernel
 * (kCoarse): z is the learned part in memory plus the coarse correction of
 * the cell's aggregate, e_c[(y >> cshift) * ncx + (x >> cshift)] from s_ec
 * (aggregates are at least 32 wide, so the four cells of a thread share
 * one). */
template <bool kCoarse>
__device__ __forceinline__ float phase_p(const LpcgParams& P, const float* __restrict__ pold,
                                         float* __restrict__ pnew, float bf, float a_prev,
                                         const float* __restrict__ s_ec) {
  const int H = P.H, W = P.W;
  const size_t n = (size_t)H * W;
  const int lane = threadIdx.x & 31;
  const float* __restrict__ z = P.z;
  float pw = 0.0f;
  for (int c = blockIdx.x; c < P.chunks; c += gridDim.x) {
    const size_t i0 = (size_t)c * kChunk + 4u * threadIdx.x;
    const bool act = i0 < n;
    const int yy = act ? (int)(i0 / (unsigned)W) : 0;
    const int xx0 = act ? (int)(i0 - (size_t)yy * W) : 0;
    float4 pc = make_float4(0.f, 0.f, 0.f, 0.f), pu = pc, pd = pc, kxc = pc, kyc = pc,
           kyu = pc;
    auto coarse_at = [&](int y, int x) -> float {
      if constexpr (kCoarse) return s_ec[(y >> P.cshift) * P.ncx + (x >> P.cshift)];
      return 0.0f;
    };
    if (act) {
      float4 zc = ld4(z + i0);
      const float4 oc = ld4(pold + i0);
      if constexpr (kCoarse) {
        const float c = coarse_at(yy, xx0);
        zc.x += c; zc.y += c; zc.z += c; zc.w += c;
      }
      float4 ev = ld4(P.e + i0);
      pc = make_float4(zc.x + bf * oc.x, zc.y + bf * oc.y, zc.z + bf * oc.z, zc.w + bf * oc.w);
      ev.x += a_prev * oc.x; ev.y += a_prev * oc.y; ev.z += a_prev * oc.z; ev.w += a_prev * oc.w;
      *reinterpret_cast<float4*>(P.e + i0) = ev;
      if (yy + 1 < H) {
        float4 zu = ld4(z + i0 + W);
        const float4 ou = ld4(pold + i0 + W);
        if constexpr (kCoarse) {
          const float c = coarse_at(yy + 1, xx0);
          zu.x += c; zu.y += c; zu.z += c; zu.w += c;
        }
        pu = make_float4(zu.x + bf * ou.x, zu.y + bf * ou.y, zu.z + bf * ou.z, zu.w + bf * ou.w);
        kyu = __ldg(reinterpret_cast<const float4*>(P.ky + i0 + W));
      }
      if (yy > 0) {
        float4 zd = ld4(z + i0 - W);
        const float4 od = ld4(pold + i0 - W);
        if constexpr (kCoarse) {
          const float c = coarse_at(yy - 1, xx0);
          zd.x += c; zd.y += c; zd.z += c; zd.w += c;
        }
        pd = make_float4(zd.x + bf * od.x, zd.y + bf * od.y, zd.z + bf * od.z, zd.w + bf * od.w);
      }
      kxc = __ldg(reinterpret_cast<const float4*>(P.kx + i0));
      kyc = __ldg(reinterpret_cast<const float4*>(P.ky + i0));
    }
    float pl = __shfl_up_sync(TL_FULL_MASK, pc.w, 1);
    float pr = __shfl_down_sync(TL_FULL_MASK, pc.x, 1);
    float kx4 = __shfl_down_sync(TL_FULL_MASK, kxc.x, 1);
    if (lane == 0 && act && xx0 > 0) {
      float zl = __ldcg(z + i0 - 1);
      if constexpr (kCoarse) zl += coarse_at(yy, xx0 - 1);
      pl = zl + bf * __ldcg(pold + i0 - 1);
    }
    if (lane == 31 && act && xx0 + 4 < W) {
      float zr = __ldcg(z + i0 + 4);
      if constexpr (kCoarse) zr += coarse_at(yy, xx0 + 4);
      pr = zr + bf * __ldcg(pold + i0 + 4);
      kx4 = __ldg(P.kx + i0 + 4);
    }
    if (!act) continue;
    const float pv[4] = {pc.x, pc.y, pc.z, pc.w};
    const float pvu[4] = {pu.x, pu.y, pu.z, pu.w};
    const float pvd[4] = {pd.x, pd.y, pd.z, pd.w};
    const float kxv[5] = {kxc.x, kxc.y, kxc.z, kxc.w, kx4};
    const float kyv[4] = {kyc.x, kyc.y, kyc.z, kyc.w};
    const float kyuv[4] = {kyu.x, kyu.y, kyu.z, kyu.w};
    float wv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int xx = xx0 + q;
      const float a = pv[q];
      const float al = (xx == 0) ? a : (q == 0 ? pl : pv[q - 1]);
      const float ar = (xx == W - 1) ? a : (q == 3 ? pr : pv[q + 1]);
      const float ad = (yy == 0) ? a : pvd[q];
      const float au = (yy == H - 1) ? a : pvu[q];
      wv[q] = a + kxv[q + 1] * (a - ar) + kxv[q] * (a - al) + kyuv[q] * (a - au) +
              kyv[q] * (a - ad);
      pw += wv[q] * a;
    }
    *reinterpret_cast<float4*>(pnew + i0) = pc;
    *reinterpret_cast<float4*>(P.w + i0) = make_float4(wv[0], wv[1], wv[2], wv[3]);
  }
  return pw;
}

/* ------------------------------------------------------------ phase Z */

struct ZSums {
  float rr, rz;
};

struct ZArgs {
  int H, W, tiles_x, tiles;
  const float* rold;
  float* rnew;
  const float* w;
  const float* s;
  float* z;
  float alpha, sigma, zscale;
  /* two-level kernel: the row-pair sums of the tiles in flight
   * (rest[parity][pair][aggregate column]) and the tiles' partials */
  float* rest;
  float* rc_part;
  int cshift;
};

/* Per-block tcgen05 state. The phase parities are kept by the threads that
 * wait on each mbarrier, so that every wait names the phase it needs. */
struct TileState {
  unsigned char* smem;
  uint64_t* a_full;    /* [2] staged tile b is in shared memory (1 arrival) */
  uint64_t* mma_done;  /* [2][kIssuers] issuer i's MMAs of buffer b completed */
  uint64_t* d_free;    /* [2] accumulators of buffer b moved out (8 arrivals) */
  uint64_t* drain;     /* every MMA issued so far completed (teardown) */
  uint32_t tmem;
  /* mbarrier phase parities, bit b for buffer b (a runtime-indexed array
   * would live in local memory): the next a_full / d_free / mma_done phase
   * to wait for, and whether buffer b has received MMAs before */
  uint32_t a_par, d_par, issued;  /* issuer */
  uint32_t done_par;              /* readers */
};

/* Stages y = sigma * s * r_new, r_new = r_old - alpha w, for tile rows
 * y0-8 .. y0+135 and columns x0-8 .. x0+71 as FP16 into the A buffer (zero
 * outside the domain; W % 4 == 0, so a group of four columns is entirely
 * inside or outside), and writes r_new of the tile's own cells to memory.
 * Each thread issues the loads of two groups before it converts them. */
__device__ __forceinline__ void stage_a(const ZArgs& A, int y0, int x0, unsigned char* abuf,
                                        int tid, int nthr) {
  constexpr int kTotal = kRows * kGroups;
  for (int q0 = tid; q0 < kTotal; q0 += 2 * nthr) {
    float4 r[2], ww[2], ss[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int q = q0 + u * nthr;
      const int row = q / kGroups, grp = q - row * kGroups;
      const int gy = y0 - kHalo + row, gx = x0 - kHalo + 4 * grp;
      r[u] = ww[u] = ss[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (q < kTotal && gy >= 0 && gy < A.H && gx >= 0 && gx < A.W) {
        const size_t i = (size_t)gy * A.W + gx;
        r[u] = ld4(A.rold + i);
        if (A.w) ww[u] = ld4(A.w + i);
        ss[u] = __ldg(reinterpret_cast<const float4*>(A.s + i));
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int q = q0 + u * nthr;
      if (q >= kTotal) break;
      const int row = q / kGroups, grp = q - row * kGroups;
      const float a = A.alpha, sg = A.sigma;
      const float4 rv = make_float4(r[u].x - a * ww[u].x, r[u].y - a * ww[u].y,
                                    r[u].z - a * ww[u].z, r[u].w - a * ww[u].w);
      const __half2 lo = __floats2half2_rn(sg * ss[u].x * rv.x, sg * ss[u].y * rv.y);
      const __half2 hi = __floats2half2_rn(sg * ss[u].z * rv.z, sg * ss[u].w * rv.w);
      uint2 packed;
      packed.x = *reinterpret_cast<const uint32_t*>(&lo);
      packed.y = *reinterpret_cast<const uint32_t*>(&hi);
      *reinterpret_cast<uint2*>(abuf + (grp >> 1) * kChunkBytes + row * 16 + (grp & 1) * 8) =
          packed;
      const int trow = row - kHalo, tcol = 4 * grp - kHalo;
      if (trow >= 0 && trow < kTH && tcol >= 0 && tcol < kTW) {
        const int gy = y0 + trow, gx = x0 + tcol;
        if (gy < A.H && gx < A.W)
          *reinterpret_cast<float4*>(A.rnew + (size_t)gy * A.W + gx) = rv;
      }
    }
  }
}

/* The MMAs of one tile that issuer kW0 owns (one thread): input window w
 * (staged columns 16 w .. 16 w + 15, K-major chunks 2 w and 2 w + 1) at row
 * offset dy = dyi - 8 reaches the 32 output columns 16 w - 16 .. 16 w + 15;
 * even and odd windows accumulate into separate column ranges of the buffer,
 * so every window's first MMA (dyi = 0) initialises its own columns. The
 * loop runs over dy outside and the windows inside: consecutive MMAs then
 * accumulate into different columns and need not wait for one another. */
template <int kW0>
__device__ __forceinline__ void issue_tile(uint32_t a_addr, uint32_t b_addr, uint32_t d_tmem) {
  const uint64_t a_desc = tc05::smem_desc(a_addr, kChunkBytes, 128);
  const uint64_t b_desc = tc05::smem_desc(b_addr, 512, 128);
#pragma unroll 1
  for (int dyi = 0; dyi < 17; ++dyi) {
    const uint32_t boff = (uint32_t)(dyi * 1024) >> 4;
#pragma unroll
    for (int w = kW0; w < kWindows; w += kIssuers) {
      const uint32_t d = d_tmem + ((w & 1) ? 96u + 16u * (uint32_t)(w - 1) : 16u * (uint32_t)w);
      const uint32_t aoff = (uint32_t)(2 * w * kChunkBytes + dyi * 16) >> 4;
      tc05::mma_f16(d, a_desc + aoff, b_desc + boff, kIdesc, dyi != 0);
    }
  }
}

template <int kW0>
__device__ __forceinline__ void issue_tile_of(int issuer, uint32_t a_addr, uint32_t b_addr,
                                              uint32_t d_tmem) {
  if constexpr (kW0 < kIssuers) {
    if (issuer == kW0) {
      issue_tile<kW0>(a_addr, b_addr, d_tmem);
    } else {
      issue_tile_of<kW0 + 1>(issuer, a_addr, b_addr, d_tmem);
    }
  }
}

/* Phase Z, warps 0 .. kIssuers-1: for each tile, wait until it is staged and
 * its accumulator buffer has been read out, then issue the MMAs of windows
 * w = issuer, issuer + kIssuers, ... (lane 0) and commit them to this
 * issuer's mma_done barrier. With several issuers the tile's MMA stream is
 * shared; one issuer with the windows interleaved measured faster than two
 * or three (by ~2 % of the step time at 4096^2).
 * Each whole warp runs the loop so that it reaches the block-wide barriers
 * after the phase converged. */
__device__ __forceinline__ void z_issuer_warp(const ZArgs& A, TileState& T, int* status,
                                              int issuer) {
  const int lane = threadIdx.x & 31;
  int j = 0;
  for (int c = blockIdx.x; c < A.tiles; c += gridDim.x, ++j) {
    const int b = j & 1;
    bool ok = tc05::mbar_wait(&T.a_full[b], (T.a_par >> b) & 1u, kWaitNs);
    T.a_par ^= 1u << b;
    if (ok && ((T.issued >> b) & 1u)) {
      ok = tc05::mbar_wait(&T.d_free[b], (T.d_par >> b) & 1u, kWaitNs);
      T.d_par ^= 1u << b;
    }
    if (!ok && lane == 0) atomicCAS(status, 0, TL_ERR_TIMEOUT);
    __syncwarp();
    if (lane == 0) {
      tc05::fence_after_sync();
      if (ok) {
        issue_tile_of<0>(issuer, tc05::smem_addr(T.smem + (b ? kOffA1 : kOffA0)),
                         tc05::smem_addr(T.smem + kOffB), T.tmem + (uint32_t)b * kDCols);
      }
      tc05::mma_commit(&T.mma_done[b * kIssuers + issuer]);
    }
    T.issued |= 1u << b;
    __syncwarp();
  }
}

/* Finishes one tile of phase Z (worker warps): warps 4..11 wait for its MMAs
 * and move the accumulators (even + odd windows) to the row-major hand-over
 * tile zt, then every worker forms z = s K y / sigma + s^2 r_new for its cells
 * from zt, r_new (written by the staging, read back from L2) and s, with
 * coalesced accesses, and sums r.r and r.z. */
template <bool kCoarse>
__device__ __forceinline__ void z_finish_tile(const ZArgs& A, TileState& T, ZSums& sums,
                                              int* status, int tile, int bb) {
  const int tid = threadIdx.x - 32 * kIssuers;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool reader = warp >= 4 && warp < 4 + kReaders;
  float* zt = reinterpret_cast<float*>(T.smem + kOffZ);
  if (reader) {
    bool ok = true;
    for (int i = 0; i < kIssuers; ++i)
      ok = tc05::mbar_wait(&T.mma_done[bb * kIssuers + i], (T.done_par >> bb) & 1u, kWaitNs) &&
           ok;
    T.done_par ^= 1u << bb;
    /* The lanes leave their polling loops at different times; tcgen05.ld
     * is warp-collective (.sync.aligned) and needs the warp converged. */
    ok = __all_sync(0xffffffffu, ok);
    if (!ok && lane == 0) atomicCAS(status, 0, TL_ERR_TIMEOUT);
    __syncwarp();
    tc05::fence_after_sync();
    const int sp = warp & 3, half = (warp - 4) >> 2;
    const uint32_t base = T.tmem + ((uint32_t)(32 * sp) << 16) + (uint32_t)bb * kDCols +
                          (uint32_t)(32 * half);
    float* zr = zt + (32 * sp + lane) * kZStride + 32 * half;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      float ev[16], od[16];
      tc05::tmem_ld16x2(base + 16 + 16 * q, base + 96 + 16 * q, ev, od);
#pragma unroll
      for (int i = 0; i < 16; ++i) zr[16 * q + i] = ev[i] + od[i];
    }
    tc05::fence_before_sync();
    __syncwarp();
    if (lane == 0) mbar_arrive(&T.d_free[bb]);
  }
  named_sync(kBarWorkers, kWorkers);
  const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
  const int y0 = ty * kTH, x0 = tx * kTW;
  constexpr int kQuads = kTH * kTW / 4;
  for (int q = tid; q < kQuads; q += kWorkers) {
    const int row = q / (kTW / 4), c4 = 4 * (q % (kTW / 4));
    const int gy = y0 + row, gx = x0 + c4;
    float rsum = 0.0f;
    if (gy < A.H && gx < A.W) {
      const size_t i = (size_t)gy * A.W + gx;
      const float4 rn = ld4(A.rnew + i);
      const float4 ss = __ldg(reinterpret_cast<const float4*>(A.s + i));
      const float4 acc = *reinterpret_cast<const float4*>(zt + row * kZStride + c4);
      float4 zv;
      zv.x = ss.x * (acc.x * A.zscale) + ss.x * ss.x * rn.x;
      zv.y = ss.y * (acc.y * A.zscale) + ss.y * ss.y * rn.y;
      zv.z = ss.z * (acc.z * A.zscale) + ss.z * ss.z * rn.z;
      zv.w = ss.w * (acc.w * A.zscale) + ss.w * ss.w * rn.w;
      *reinterpret_cast<float4*>(A.z + i) = zv;
      sums.rr += rn.x * rn.x + rn.y * rn.y + rn.z * rn.z + rn.w * rn.w;
      sums.rz += rn.x * zv.x + rn.y * zv.y + rn.z * zv.z + rn.w * zv.w;
      if constexpr (kCoarse) rsum = (rn.x + rn.y) + (rn.z + rn.w);
    }
    if constexpr (kCoarse) {
      /* The restriction: a warp holds the 32 quads of tile rows 2m and 2m+1
       * (16 per row); sum them per aggregate column (8-lane groups for
       * 32-wide aggregates, whole rows otherwise), then the two rows. */
      rsum += __shfl_xor_sync(TL_FULL_MASK, rsum, 1);
      rsum += __shfl_xor_sync(TL_FULL_MASK, rsum, 2);
      rsum += __shfl_xor_sync(TL_FULL_MASK, rsum, 4);
      if (A.cshift > 5) rsum += __shfl_xor_sync(TL_FULL_MASK, rsum, 8);
      rsum += __shfl_xor_sync(TL_FULL_MASK, rsum, 16);
      float* rest = A.rest + bb * kTH + (q >> 5) * 2;  /* [parity][pair][column] */
      if (lane == 0) rest[0] = rsum;
      if (lane == 8 && A.cshift == 5) rest[1] = rsum;
    }
  }
}

/* One worker warp, after a worker barrier that follows z_finish_tile of
 * `tile` (processing parity bb): the tile's restriction partials, the sums
 * of its row-pair sums over each aggregate in a fixed order, into
 * rc_part[tile * kRestSlots + local aggregate] (aggregate rows of the tile
 * first, then columns). */
__device__ __forceinline__ void z_restrict_tile(const ZArgs& A, int tile, int bb) {
  const int lane = threadIdx.x & 31;
  const int b = 1 << A.cshift;
  const int arows = b < kTH ? b : kTH, acols = b < kTW ? b : kTW;
  const int ncol = kTW / acols, nloc = (kTH / arows) * ncol;
  if (lane < nloc) {
    const int ar = lane / ncol, ac = lane - ar * ncol;
    const float* rest = A.rest + bb * kTH;
    float t = 0.0f;
    for (int m = ar * arows / 2; m < (ar + 1) * arows / 2; ++m) t += rest[m * 2 + ac];
    A.rc_part[(size_t)tile * kRestSlots + lane] = t;
  }
}

/* Phase Z, warps kIssuers..31: stage tile j (writing r_new = r_old - alpha w
 * for its own cells), then finish tile j - 1. The hand-over tile is
 * single-buffered: a worker barrier separates the last reads of one tile's
 * rows from the readers' writes of the next. */
template <bool kCoarse>
__device__ __forceinline__ void z_worker_warps(const ZArgs& A, TileState& T, ZSums& sums,
                                               int* status) {
  const int tid = threadIdx.x - 32 * kIssuers;
  int prev = -1, prev_b = 0, j = 0;
  int pend = -1, pend_b = 0;  /* a finished tile whose restriction is still to be summed */
  for (int c = blockIdx.x; c < A.tiles; c += gridDim.x, ++j) {
    const int tile = A.tiles - 1 - c;
    const int b = j & 1;
    const int ty = tile / A.tiles_x, tx = tile - ty * A.tiles_x;
    stage_a(A, ty * kTH, tx * kTW, T.smem + (b ? kOffA1 : kOffA0), tid, kWorkers);
    tc05::fence_proxy_async_smem();
    named_sync(kBarWorkers, kWorkers);
    if (tid == 0) mbar_arrive(&T.a_full[b]);
    if constexpr (kCoarse) {
      if (pend >= 0 && tid < 32) z_restrict_tile(A, pend, pend_b);
      pend = -1;
    }
    if (prev >= 0) {
      z_finish_tile<kCoarse>(A, T, sums, status, prev, prev_b);
      pend = prev;
      pend_b = prev_b;
    }
    prev = tile;
    prev_b = b;
  }
  /* The last tile: its readers overwrite the hand-over tile, so every worker
   * must have finished reading the previous tile's rows first (inside the
   * loop the barrier after staging does this). */
  if (prev >= 0) {
    named_sync(kBarWorkers, kWorkers);
    if constexpr (kCoarse) {
      if (pend >= 0 && tid < 32) z_restrict_tile(A, pend, pend_b);
    }
    z_finish_tile<kCoarse>(A, T, sums, status, prev, prev_b);
    if constexpr (kCoarse) {
      named_sync(kBarWorkers, kWorkers);
      if (tid < 32) z_restrict_tile(A, prev, prev_b);
    }
  }
}

/* ------------------------------------------------------ persistent PCG */

/* ------------------------------------------------------------ phase C */

/* Two-level kernel, after phase Z's grid barrier: r_c = P^T r_new from the
 * tiles' restriction partials into s_rc (every block assembles the whole
 * vector, in the same order), then this block's share of the rows of
 * e_c = Ac^-1 r_c into P.ec, one warp per row: the FP16 entries widened to
 * FP32, FP32 sums in a fixed order, times 2^-e at the end (exact).
 * Returns (in every thread) the block's part of r_c . e_c over its rows,
 * summed in a fixed order. */
__device__ __forceinline__ float phase_c_gemv(const LpcgParams& P, float* s_rc, float* s_red) {
  const int b = 1 << P.cshift;
  const int arows = b < kTH ? b : kTH, acols = b < kTW ? b : kTW;
  const int ncol = kTW / acols;
  /* kMaxCoarse / kThreads entries per thread, all loads issued before the
   * first store (one L2 round trip instead of one per entry) */
  constexpr int kPer = kMaxCoarse / kThreads;
  float v[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int I = threadIdx.x + k * kThreads;
    v[k] = 0.0f;
    if (I < P.nc) {
      const int Jc = I / P.ncx, Ic = I - Jc * P.ncx;
      const int gy = Jc << P.cshift, gx = Ic << P.cshift;
      const int tile = (gy / kTH) * P.tiles_x + gx / kTW;
      const int loc = ((gy % kTH) / arows) * ncol + (gx % kTW) / acols;
      v[k] = __ldcg(P.rc_part + (size_t)tile * kRestSlots + loc);
      if (b > kTW) v[k] += __ldcg(P.rc_part + (size_t)(tile + 1) * kRestSlots);
    }
  }
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int I = threadIdx.x + k * kThreads;
    if (I < P.nc) s_rc[I] = v[k];
  }
  __syncthreads();
  const int rows = (P.nc + (int)gridDim.x - 1) / (int)gridDim.x;
  const int r0 = blockIdx.x * rows, r1 = min(P.nc, r0 + rows);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float dot = 0.0f;
  for (int I = r0 + warp; I < r1; I += (int)(blockDim.x >> 5)) {
    const __half* row = P.ainv + (size_t)I * P.nc;
    float acc = 0.0f;
    if ((P.nc & 7) == 0) {  /* 16-byte rows: eight entries per load */
      const uint4* row8 = reinterpret_cast<const uint4*>(row);
      const float4* rc4 = reinterpret_cast<const float4*>(s_rc);
#pragma unroll 4
      for (int q = lane; q < (P.nc >> 3); q += 32) {
        const uint4 a = __ldg(row8 + q);
        const __half2* h = reinterpret_cast<const __half2*>(&a);
        const float2 a0 = __half22float2(h[0]), a1 = __half22float2(h[1]);
        const float2 a2 = __half22float2(h[2]), a3 = __half22float2(h[3]);
        const float4 ra = rc4[2 * q], rb = rc4[2 * q + 1];
        acc += a0.x * ra.x + a0.y * ra.y + a1.x * ra.z + a1.y * ra.w + a2.x * rb.x +
               a2.y * rb.y + a3.x * rb.z + a3.y * rb.w;
      }
    } else {
      for (int q = lane; q < P.nc; q += 32) acc += __half2float(row[q]) * s_rc[q];
    }
    acc = warp_sum(acc) * P.ainv_unscale;
    if (lane == 0) P.ec[I] = acc;
    dot += acc * s_rc[I];
  }
  return block_sum(lane == 0 ? dot : 0.0f, s_red);
}

/* The solve; returns when done or when a wait ran out (status set). */
template <bool kCoarse>
__device__ __forceinline__ void lpcg_body(const LpcgParams& P, TileState& T, float* s_red,
                                          double* s_one) {
  const int G = gridDim.x;
  const int H = P.H, W = P.W;
  const double n = (double)H * (double)W;
  const float zscale_k = 1.0f / __ldg(P.kscale);
  /* two-level kernel only (the one-level kernel's shared memory ends
   * before these regions and never touches them) */
  float* s_rest = reinterpret_cast<float*>(T.smem + kOffRest);
  float* s_rc = reinterpret_cast<float*>(T.smem + kOffCoarse);
  float* s_ec = s_rc + kMaxCoarse;
  double* part_pw = P.part;
  double* part_rr = P.part + G;
  double* part_rz = P.part + 2 * G;
  double* part_ce = P.part + 3 * G;  /* two-level kernel: the blocks' r_c . e_c */

  /* r.r of the incoming residual: its RMS sets the FP16 staging scale. */
  {
    float rr = 0.0f;
    const size_t total = (size_t)H * W;
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < total;
         i += (size_t)G * kThreads) {
      const float v = __ldcg(P.r0 + i);
      rr += v * v;
    }
    rr = block_sum(rr, s_red);
    if (threadIdx.x == 0) part_rr[blockIdx.x] = (double)rr;
  }
  if (!tl_grid_barrier(P.sync, P.status)) return;
  double rr = sum_partials(part_rr, G, s_one);
  const double rr0 = rr;
  double rz_old = 0.0, alpha = 0.0, beta = 0.0;
  int par_r = 0, par_p = 0, iters = 0;
  bool done = !(rr0 > 0.0) || P.max_iters <= 0;

  for (int k = 0; !done; ++k) {
    float* rcur = par_r ? P.r1 : P.r0;
    float* rnext = par_r ? P.r0 : P.r1;
    const float* pold = par_p ? P.p1 : P.p0;
    float* pnew = par_p ? P.p0 : P.p1;
    if (k > 0) {
      /* ---- phase P */
      float pw = phase_p<kCoarse>(P, pold, pnew, (float)beta, (float)alpha, s_ec);
      pw = block_sum(pw, s_red);
      if (threadIdx.x == 0) part_pw[blockIdx.x] = (double)pw;
      if (!tl_grid_barrier(P.sync, P.status)) return;
      const double pwsum = sum_partials(part_pw, G, s_one);
      alpha = rz_old / pwsum;
    }
    /* ---- phase Z (step 0: z0 = M^-1 r0, alpha = 0) */
    ZArgs A;
    A.H = H; A.W = W; A.tiles_x = P.tiles_x; A.tiles = P.tiles;
    A.rold = rcur; A.rnew = rnext; A.w = P.w; A.s = P.s; A.z = P.z;
    A.alpha = (float)alpha;
    A.sigma = (float)(1.0 / sqrt(rr / n));
    A.zscale = zscale_k / A.sigma;
    A.rest = s_rest;
    A.rc_part = P.rc_part;
    A.cshift = P.cshift;
    ZSums sums = {0.0f, 0.0f};
    if (threadIdx.x < 32 * kIssuers) z_issuer_warp(A, T, P.status, threadIdx.x >> 5);
    else z_worker_warps<kCoarse>(A, T, sums, P.status);
    const float t_rr = block_sum(sums.rr, s_red);
    const float t_rz = block_sum(sums.rz, s_red);
    if (threadIdx.x == 0) {
      part_rr[blockIdx.x] = (double)t_rr;
      part_rz[blockIdx.x] = (double)t_rz;
    }
    if (!tl_grid_barrier(P.sync, P.status)) return;
    rr = sum_partials(part_rr, G, s_one);
    double rz = sum_partials(part_rz, G, s_one);
    const bool converged = rr <= P.tol2 * rr0 || !(rr == rr) || k >= P.max_iters;
    if constexpr (kCoarse) {
      /* z = z_learned + P e_c: r.z gains r_c . e_c; phase P adds P e_c */
      if (!converged) {
        const float dot = phase_c_gemv(P, s_rc, s_red);
        if (threadIdx.x == 0) part_ce[blockIdx.x] = (double)dot;
        if (!tl_grid_barrier(P.sync, P.status)) return;
        {
          constexpr int kPer = kMaxCoarse / kThreads;
          float ev[kPer];
#pragma unroll
          for (int q = 0; q < kPer; ++q) {
            const int I = threadIdx.x + q * kThreads;
            ev[q] = I < P.nc ? __ldcg(P.ec + I) : 0.0f;
          }
#pragma unroll
          for (int q = 0; q < kPer; ++q) {
            const int I = threadIdx.x + q * kThreads;
            if (I < P.nc) s_ec[I] = ev[q];
          }
        }
        rz += sum_partials(part_ce, G, s_one);  /* its barrier also publishes s_ec */
      }
    }
    beta = (k == 0) ? 0.0 : rz / rz_old;
    rz_old = rz;
    par_r ^= 1;
    if (k > 0) par_p ^= 1;
    iters = k;
    if (converged) done = true;
  }
  /* The last step's e += alpha p (every earlier one was added in phase P). */
  if (iters > 0) {
    const float* plast = par_p ? P.p1 : P.p0;
    const float af = (float)alpha;
    const size_t n4 = (size_t)H * W / 4;
    for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < n4;
         q += (size_t)G * kThreads) {
      const float4 pp = ld4(plast + 4 * q);
      float4 ev = ld4(P.e + 4 * q);
      ev.x += af * pp.x; ev.y += af * pp.y; ev.z += af * pp.z; ev.w += af * pp.w;
      *reinterpret_cast<float4*>(P.e + 4 * q) = ev;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *P.iters_out = iters;
    *P.rr_out = rr;
  }
}

template <bool kCoarse>
__global__ void __launch_bounds__(kThreads, 1) lpcg_kernel(LpcgParams P) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ float s_red[kThreads / 32];
  __shared__ double s_one;
  TileState T;
  T.smem = smem;
  T.a_full = reinterpret_cast<uint64_t*>(smem + kOffBar);
  T.mma_done = T.a_full + 2;
  T.d_free = T.mma_done + 2 * kIssuers;
  T.drain = T.d_free + 2;
  T.a_par = T.d_par = T.issued = T.done_par = 0u;
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(smem + kOffTmem);
  if (threadIdx.x < 32) {
    tc05::tmem_alloc(s_tmem, kTmemCols);
    tc05::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b) {
      tc05::mbar_init(&T.a_full[b], 1);
      for (int i = 0; i < kIssuers; ++i) tc05::mbar_init(&T.mma_done[b * kIssuers + i], 1);
      tc05::mbar_init(&T.d_free[b], kReaders);
    }
    tc05::mbar_init(T.drain, kIssuers);
    tc05::mbar_fence_init();
  }
  for (int i = threadIdx.x; i < kBBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(smem + kOffB)[i] = reinterpret_cast<const uint4*>(P.umma)[i];
  tc05::fence_proxy_async_smem();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  T.tmem = *s_tmem;

  lpcg_body<kCoarse>(P, T, s_red, &s_one);

  /* Teardown: every MMA this block issued has completed (a commit tracks all
   * of the issuing thread's earlier MMAs), then the tensor memory is freed. */
  if (threadIdx.x < 32 * kIssuers && (threadIdx.x & 31) == 0) {
    tc05::mma_commit(T.drain);
    if (!tc05::mbar_wait(T.drain, 0, kWaitNs)) atomicCAS(P.status, 0, TL_ERR_TIMEOUT);
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    __syncwarp();
    tc05::fence_after_sync();
    tc05::tmem_dealloc(T.tmem, kTmemCols);
  }
}



/* ------------------------------------------- stand-alone application */

__global__ void rms_partial_kernel(const float* __restrict__ r, size_t n,
                                   double* __restrict__ part) {
  __shared__ float s_red[kThreads / 32];
  float rr = 0.0f;
  for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (size_t)gridDim.x * kThreads) {
    const float v = r[i];
    rr += v * v;
  }
  rr = block_sum(rr, s_red);
  if (threadIdx.x == 0) part[blockIdx.x] = (double)rr;
}

/* ------------------------------------ tcgen05 stencil (stand-alone)
 *
 * One 128 x 64 tile per block, 8 warps. The scaled residual y is staged in
 * FP16 as the MMA's A operand: ten K-major chunks of 8 staged columns, each
 * 144 rows x 16 bytes (+16 bytes of padding so that the stores of one row
 * spread over the banks). For output columns 16 nb .. 16 nb + 15 and row
 * offset dy, the two 16-column windows of the band are chunks 2 nb + 2 kb and
 * 2 nb + 2 kb + 1 (LBO = chunk size), shifted down by dy + 8 rows (16 bytes
 * per row, SBO = 128); the B operands are the 34 Toeplitz blocks T(dy, kb)
 * (16 x 16). 136 MMAs of M = 128, N = 16, K = 16 accumulate the tile in 64
 * tensor-memory columns (lane = tile row); the epilogue reads them back with
 * tcgen05.ld, one row per thread. */
constexpr int kUTH = 128;
constexpr int kUTW = 64;
constexpr int kUThreads = 256;
constexpr int kURows = kUTH + 2 * kHalo;
constexpr int kUChunks = (kUTW + 2 * kHalo) / 8;
constexpr int kUChunkBytes = kURows * 16 + 16;
constexpr int kUBBytes = 17 * 2 * 512;
constexpr uint32_t kUTmemCols = 64;
constexpr uint32_t kUIdesc = tc05::idesc_f16_f32<128, 16>();
constexpr unsigned long long kUWaitNs = 1000000000ull;

__global__ void __launch_bounds__(kUThreads) stencil_apply_tc05_kernel(
    int H, int W, int tiles_x, const float* __restrict__ r, const float* __restrict__ s,
    float* __restrict__ z, const __half* __restrict__ umma, const float* __restrict__ kscale,
    const double* __restrict__ part, int nparts, int* __restrict__ status) {
  __shared__ __align__(1024) unsigned char s_a[kUChunks * kUChunkBytes];
  __shared__ __align__(1024) unsigned char s_b[kUBBytes];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tmem;
  __shared__ double s_one;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    tc05::tmem_alloc(&s_tmem, kUTmemCols);
    tc05::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    tc05::mbar_init(&s_mbar, 1);
    tc05::mbar_fence_init();
  }
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = s_tmem;

  double rr = 0.0;
  if (threadIdx.x < 32) {
    for (int i = threadIdx.x; i < nparts; i += 32) rr += part[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rr += __shfl_xor_sync(TL_FULL_MASK, rr, o);
    if (threadIdx.x == 0) s_one = rr;
  }
  __syncthreads();
  rr = s_one;
  const double n = (double)H * (double)W;
  const float sigma = rr > 0.0 ? (float)(1.0 / sqrt(rr / n)) : 1.0f;
  const float zscale = 1.0f / (__ldg(kscale) * sigma);

  /* B operands */
  for (int i = threadIdx.x; i < kUBBytes / 16; i += kUThreads)
    reinterpret_cast<uint4*>(s_b)[i] = reinterpret_cast<const uint4*>(umma)[i];
  /* A operand: y = sigma s r, rows y0-8 .., columns x0-8 .., zero outside */
  const int ty = blockIdx.x / tiles_x, tx = blockIdx.x - ty * tiles_x;
  const int y0 = ty * kUTH, x0 = tx * kUTW;
  constexpr int kGroups = (kUTW + 2 * kHalo) / 4;
  for (int q = threadIdx.x; q < kURows * kGroups; q += kUThreads) {
    const int row = q / kGroups, grp = q - row * kGroups;
    const int gy = y0 - kHalo + row, gx = x0 - kHalo + 4 * grp;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      const size_t i = (size_t)gy * W + gx;
      const float4 rv = __ldg(reinterpret_cast<const float4*>(r + i));
      const float4 sv = __ldg(reinterpret_cast<const float4*>(s + i));
      v = make_float4(sigma * sv.x * rv.x, sigma * sv.y * rv.y, sigma * sv.z * rv.z,
                      sigma * sv.w * rv.w);
    }
    const __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, v.w);
    uint2 packed;
    packed.x = *reinterpret_cast<const uint32_t*>(&lo);
    packed.y = *reinterpret_cast<const uint32_t*>(&hi);
    *reinterpret_cast<uint2*>(s_a + (grp >> 1) * kUChunkBytes + row * 16 + (grp & 1) * 8) =
        packed;
  }
  tc05::fence_proxy_async_smem();
  __syncthreads();

  if (threadIdx.x == 0) {
    tc05::fence_after_sync();
    const uint32_t a0 = tc05::smem_addr(s_a), b0 = tc05::smem_addr(s_b);
    for (int nb = 0; nb < kUTW / 16; ++nb) {
      for (int dyi = 0; dyi < 17; ++dyi) {
#pragma unroll
        for (int kb = 0; kb < 2; ++kb) {
          const uint64_t ad = tc05::smem_desc(a0 + (2 * nb + 2 * kb) * kUChunkBytes + dyi * 16,
                                              kUChunkBytes, 128);
          const uint64_t bd = tc05::smem_desc(b0 + (2 * dyi + kb) * 512, 256, 128);
          tc05::mma_f16(tmem + 16 * nb, ad, bd, kUIdesc, (dyi | kb) != 0);
        }
      }
    }
    tc05::mma_commit(&s_mbar);
  }
  bool ok = tc05::mbar_wait(&s_mbar, 0, kUWaitNs);
  if (!ok) {
    atomicCAS(status, 0, TL_ERR_TIMEOUT);
    tc05::mbar_wait(&s_mbar, 0, kUWaitNs);  /* let the MMAs drain before freeing */
  }
  ok = __syncthreads_and(ok) != 0;  /* tcgen05.ld below is warp-collective */
  tc05::fence_after_sync();
  if (ok) {
    const int sp = warp & 3, ch = warp >> 2;
    const int row = 32 * sp + lane, gy = y0 + row;
    float acc[32];
    tc05::tmem_ld16x2(tmem + ((uint32_t)(32 * sp) << 16) + 32 * ch,
                      tmem + ((uint32_t)(32 * sp) << 16) + 32 * ch + 16, acc, acc + 16);
    if (gy < H) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int gx = x0 + 32 * ch + 4 * q;
        if (gx >= W) break;
        const size_t i = (size_t)gy * W + gx;
        const float4 rv = __ldg(reinterpret_cast<const float4*>(r + i));
        const float4 sv = __ldg(reinterpret_cast<const float4*>(s + i));
        float4 zv;
        zv.x = sv.x * (acc[4 * q] * zscale) + sv.x * sv.x * rv.x;
        zv.y = sv.y * (acc[4 * q + 1] * zscale) + sv.y * sv.y * rv.y;
        zv.z = sv.z * (acc[4 * q + 2] * zscale) + sv.z * sv.z * rv.z;
        zv.w = sv.w * (acc[4 * q + 3] * zscale) + sv.w * sv.w * rv.w;
        *reinterpret_cast<float4*>(z + i) = zv;
      }
    }
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc05::fence_after_sync();
    tc05::tmem_dealloc(tmem, kUTmemCols);
  }
}

}  // namespace

static int check_packed_shape(int H, int W) {
  TL_REQUIRE(H >= 2 && W >= 8 && W % 4 == 0,
             "the collapsed preconditioner needs a packed [H][W] field with W % 4 == 0");
  TL_REQUIRE((size_t)H * W < (1ull << 31), "field too large for the collapsed preconditioner");
  return TL_OK;
}

/* z = M^-1 r with the collapsed stencil on the tcgen05 tensor cores (umma:
 * the Toeplitz B operands built from the network, kscale their scale). */
int tl_internal_apply_collapsed(tl_context* ctx, const void* umma, const float* kscale, int H,
                                int W, const float* r, const float* s, float* z) {
  int rc = check_packed_shape(H, W);
  if (rc != TL_OK) return rc;
  const size_t n = (size_t)H * W;
  const int nparts = std::max(1, std::min<int>(2 * ctx->num_sms, (int)((n + kThreads - 1) / kThreads)));
  rc = tl_ensure_partials(ctx, (size_t)nparts);
  if (rc != TL_OK) return rc;
  rms_partial_kernel<<<nparts, kThreads, 0, ctx->stream>>>(r, n, ctx->d_part);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  const int tiles_x = (W + kUTW - 1) / kUTW, tiles_y = (H + kUTH - 1) / kUTH;
  stencil_apply_tc05_kernel<<<tiles_x * tiles_y, kUThreads, 0, ctx->stream>>>(
      H, W, tiles_x, r, s, z, reinterpret_cast<const __half*>(umma), kscale, ctx->d_part, nparts,
      ctx->d_status);
  TL_CHECK_LAUNCH(ctx);
  int status = 0;
  TL_CUDA(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                          ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  if (status != 0) return tl_set_error(status, "tcgen05 stencil: MMA completion wait timed out");
  return TL_OK;
}

/* Inner PCG with the collapsed learned preconditioner on packed
 * FP32 arrays: solves A32 e = r until r.r <= tol^2 r0.r0 or max_iters steps.
 * r is the incoming residual (the kernel leaves the final residual in r or
 * r_alt); e, w, z, pa, pb are scratch of H*W floats, all 16-byte aligned.
 * umma: the window B operands of the network's stencil. Returns the step
 * count and the final r.r. */
int tl_internal_fpcg_collapsed(tl_context* ctx, const void* umma, const float* kscale, int H,
                               int W, const float* kx, const float* ky, const float* s,
                               float* r, float* r_alt, float* e, float* w, float* z, float* pa,
                               float* pb, double tol, int max_iters, int* iters,
                               double* rr_final, const tl_coarse_level* coarse) {
  int rc = check_packed_shape(H, W);
  if (rc != TL_OK) return rc;
  TL_REQUIRE(max_iters >= 0 && tol > 0.0, "tl_internal_fpcg_collapsed: bad arguments");
  if (coarse) {
    const int b = 1 << coarse->blk_shift;
    TL_REQUIRE(coarse->nc >= 1 && coarse->nc <= kMaxCoarse && b >= 32 && b <= 128 &&
                   H % b == 0 && W % b == 0 && coarse->ncx == W / b,
               "tl_internal_fpcg_collapsed: coarse level does not fit the field");
  }
  const size_t n = (size_t)H * W;
  const void* kernel = coarse ? (const void*)lpcg_kernel<true> : (const void*)lpcg_kernel<false>;
  const int smem = coarse ? kLpcgSmemCoarse : kLpcgSmem;
  TL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  TL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem));
  TL_REQUIRE(per_sm >= 1, "the learned PCG kernel cannot be resident");
  /* one block per SM: each block holds all 512 tensor-memory columns */
  const int G = ctx->num_sms;
  rc = tl_ensure_partials(ctx, (size_t)G);
  if (rc != TL_OK) return rc;
  TL_CUDA(cudaMemsetAsync(e, 0, n * sizeof(float), ctx->stream));
  TL_CUDA(cudaMemsetAsync(w, 0, n * sizeof(float), ctx->stream));
  TL_CUDA(cudaMemsetAsync(pa, 0, n * sizeof(float), ctx->stream));
  TL_CUDA(cudaMemsetAsync(pb, 0, n * sizeof(float), ctx->stream));
  LpcgParams P;
  P.H = H;
  P.W = W;
  P.chunks = (int)((n + kChunk - 1) / kChunk);
  P.tiles_x = (W + kTW - 1) / kTW;
  P.tiles = P.tiles_x * ((H + kTH - 1) / kTH);
  P.max_iters = max_iters;
  P.tol2 = tol * tol;
  P.kx = kx;
  P.ky = ky;
  P.s = s;
  P.r0 = r;
  P.r1 = r_alt;
  P.e = e;
  P.w = w;
  P.z = z;
  P.p0 = pa;
  P.p1 = pb;
  P.umma = reinterpret_cast<const __half*>(umma);
  P.kscale = kscale;
  P.part = ctx->d_part;
  P.cshift = coarse ? coarse->blk_shift : 0;
  P.ncx = coarse ? coarse->ncx : 0;
  P.nc = coarse ? coarse->nc : 0;
  P.ainv = coarse ? coarse->ainv16 : nullptr;
  P.ainv_unscale = coarse ? ldexpf(1.0f, -coarse->exp16) : 0.0f;
  P.rc_part = coarse ? coarse->rc_part : nullptr;
  P.ec = coarse ? coarse->ec : nullptr;
  P.sync = ctx->d_sync;
  P.status = ctx->d_status;
  P.iters_out = ctx->d_steps;
  P.rr_out = ctx->d_result + 7;
  TL_CUDA(cudaMemsetAsync(ctx->d_sync + TL_SYNC_BAR_COUNT, 0, 2 * sizeof(unsigned),
                          ctx->stream));
  TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  ctx->h_steps[0] = -1;
  void* args[] = {&P};
  TL_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(G), dim3(kThreads), args, smem,
                                      ctx->stream));
  TL_CHECK_LAUNCH(ctx);
  int status = 0;
  TL_CUDA(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                          ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  if (status != 0)
    return tl_set_error(status, "learned PCG kernel: a grid-barrier or MMA wait timed out");
  *iters = ((volatile int*)ctx->h_steps)[0];
  *rr_final = ((volatile double*)ctx->h_result)[7];
  return TL_OK;
}
