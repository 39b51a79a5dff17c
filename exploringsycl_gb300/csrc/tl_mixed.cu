/*
 * tl_mixed.cu -- mixed-precision solve of one TeaLeaf timestep: an FP64
 * defect-correction (iterative refinement) loop around an FP32 conjugate-
 * gradient inner solve, with optional Jacobi preconditioning of the inner
 * solve, and an automatic fall-back to the exact FP64 CG when refinement
 * stalls.
 *
 * The system is the reference's: A u = u0 with A the 5-point operator of
 * TeaLeaf/shared.h:59-63 built from kx, ky (TeaLeaf/c_kernels/sycl/cg.cpp:
 * 40-69), reflective (zero-flux) boundaries, initial guess u = u0 (the
 * reference's x0 = b, TeaLeaf/drivers/cg_driver.c:56-65), or with
 * projection > 0 the A-norm best combination of u0 and the solutions of
 * earlier solves with the same operator (tl_project.cu). The stop rule is a
 * relative FP64 *true* residual, ||u0 - A u||_2 <= rel_tol ||u0||_2 over the
 * interior (FP64 CG from u0: the reference's residual kernel; the other
 * paths: the same operator with fused multiply-adds on its precomputed
 * diagonal, one pass with r.r).
 *
 * Outer step (FP64): r = u0 - A u; stop if small; r32 = r * s (s scales the
 * residual to unit RMS); solve A32 e = r32 in FP32 to a relative reduction
 * inner_tol (0: the method's default, 3e-6 with the learned preconditioner,
 * whose restarts cost more than its extra inner steps, 1e-5 otherwise);
 * u += e / s. The inner operator A32 uses kx, ky rounded to FP32
 * and the flux form a + sum k (a - a_nb), in which a neighbour across the
 * domain boundary equals the cell itself (the reflective halo), so boundary
 * fluxes vanish exactly.
 *
 * Inner kernel: one persistent cooperative kernel, 1024 threads per SM, each
 * thread four consecutive cells of a 4096-cell tile. Per CG step two phases:
 *  (1) p_new = z + beta p_old is formed on the fly at the cell and its four
 *      neighbours (z = r, or r * inv_diag with Jacobi), w = A32 p_new, p_new
 *      stored to the other p buffer, p.w partial sums;
 *  (2) e += alpha p_new, r -= alpha w, r.r (and r.z) partial sums, tiles
 *      visited in reverse order so that the most recently written tiles of
 *      phase 1 are still in L2.
 * Memory per cell and step: 24 B + 24 B (+ 8 B with Jacobi) in FP32, against
 * 104 B for the FP64 step. Each thread keeps its partial sums in FP32
 * registers across all of its block's tiles; one block reduction per phase
 * gives one FP64 partial per block, and the partials are reduced in a fixed
 * order by every block (deterministic, no per-tile synchronisation).
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "tl_internal.cuh"

namespace {

constexpr int kThreads = 1024;

struct InnerParams {
  int x, y, hd, ntiles, max_iters, jacobi;
  double tol2;  /* stop when r.r <= tol2 * (r.r at start) */
  const float *kx, *ky, *invd;
  float *r, *e, *w, *pa, *pb;
  double *part_pw, *part_rr, *part_rz;
  unsigned* sync;
  int* status;
  int* iters_out;
  double* rr_out;
};

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TL_FULL_MASK, v, o);
  return v;
}

/* Block-wide sum of one float per thread, in a fixed order; thread 0 gets it. */
__device__ __forceinline__ float block_sum_f(float v, float* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_f(v);
  if (lane == 0) s_warp[warp] = v;
  __syncthreads();
  float t = 0.0f;
  if (warp == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0.0f;
    t = warp_sum_f(t);
  }
  __syncthreads();
  return t;
}

/* Preconditioned residual z at cell i. */
__device__ __forceinline__ float zval(const InnerParams& P, float r, unsigned i) {
  return P.jacobi ? r * __ldg(P.invd + i) : r;
}

template <bool kVec>
__global__ void __launch_bounds__(kThreads, 1) inner_cg_kernel(InnerParams P, int parity0) {
  __shared__ float s_warp[3][32];
  __shared__ double s_scratch[TL_RED_SCRATCH];
  const int x = P.x, y = P.y, hd = P.hd;
  const unsigned len = (unsigned)x * (unsigned)y;
  const int lane = threadIdx.x & 31;
  const int G = gridDim.x;
  double rz_old = 0.0, beta = 0.0, rr0 = -1.0;
  int iters = 0;
  int parity = parity0;
  float* __restrict__ r = P.r;
  float* __restrict__ e = P.e;
  float* __restrict__ w = P.w;
  const float* __restrict__ kx = P.kx;
  const float* __restrict__ ky = P.ky;

  for (int k = 0; k <= P.max_iters; ++k) {
    const float* __restrict__ pold = parity ? P.pb : P.pa;
    float* __restrict__ pnew = parity ? P.pa : P.pb;
    const float bf = (float)beta;

    if (k > 0) {
      /* ---- phase 1: p_new = z + beta p_old, w = A p_new, p.w */
      float pw = 0.0f;
      for (int tile = blockIdx.x; tile < P.ntiles; tile += G) {
        const unsigned i0 = (unsigned)tile * TL_TILE + 4u * threadIdx.x;
        if (kVec) {
          const int jj = (int)(i0 / (unsigned)x);
          const int kk0 = (int)(i0 - (unsigned)jj * (unsigned)x);
          const bool row = i0 < len && jj >= hd && jj < y - hd;
          float4 pc = make_float4(0.f, 0.f, 0.f, 0.f), pu = pc, pd = pc;
          float4 kxc = pc, kyc = pc, kyu = pc;
          if (row) {
            const float4 rc = __ldcg(reinterpret_cast<const float4*>(r + i0));
            const float4 ru = __ldcg(reinterpret_cast<const float4*>(r + i0 + x));
            const float4 rd = __ldcg(reinterpret_cast<const float4*>(r + i0 - x));
            const float4 oc = __ldcg(reinterpret_cast<const float4*>(pold + i0));
            const float4 ou = __ldcg(reinterpret_cast<const float4*>(pold + i0 + x));
            const float4 od = __ldcg(reinterpret_cast<const float4*>(pold + i0 - x));
            if (P.jacobi) {
              const float4 dc = __ldg(reinterpret_cast<const float4*>(P.invd + i0));
              const float4 du = __ldg(reinterpret_cast<const float4*>(P.invd + i0 + x));
              const float4 dd = __ldg(reinterpret_cast<const float4*>(P.invd + i0 - x));
              pc = make_float4(rc.x * dc.x + bf * oc.x, rc.y * dc.y + bf * oc.y,
                               rc.z * dc.z + bf * oc.z, rc.w * dc.w + bf * oc.w);
              pu = make_float4(ru.x * du.x + bf * ou.x, ru.y * du.y + bf * ou.y,
                               ru.z * du.z + bf * ou.z, ru.w * du.w + bf * ou.w);
              pd = make_float4(rd.x * dd.x + bf * od.x, rd.y * dd.y + bf * od.y,
                               rd.z * dd.z + bf * od.z, rd.w * dd.w + bf * od.w);
            } else {
              pc = make_float4(rc.x + bf * oc.x, rc.y + bf * oc.y, rc.z + bf * oc.z,
                               rc.w + bf * oc.w);
              pu = make_float4(ru.x + bf * ou.x, ru.y + bf * ou.y, ru.z + bf * ou.z,
                               ru.w + bf * ou.w);
              pd = make_float4(rd.x + bf * od.x, rd.y + bf * od.y, rd.z + bf * od.z,
                               rd.w + bf * od.w);
            }
            kxc = __ldg(reinterpret_cast<const float4*>(kx + i0));
            kyc = __ldg(reinterpret_cast<const float4*>(ky + i0));
            kyu = __ldg(reinterpret_cast<const float4*>(ky + i0 + x));
          }
          float pl = __shfl_up_sync(TL_FULL_MASK, pc.w, 1);
          float pr = __shfl_down_sync(TL_FULL_MASK, pc.x, 1);
          float kx4 = __shfl_down_sync(TL_FULL_MASK, kxc.x, 1);
          const bool in0 = row && kk0 >= hd && kk0 < x - hd;
          const bool in3 = row && kk0 + 3 >= hd && kk0 + 3 < x - hd;
          if (lane == 0 && in0 && kk0 > hd) {
            pl = zval(P, __ldcg(r + i0 - 1), i0 - 1) + bf * __ldcg(pold + i0 - 1);
          }
          if (lane == 31 && in3) {
            if (kk0 + 3 < x - hd - 1) {
              pr = zval(P, __ldcg(r + i0 + 4), i0 + 4) + bf * __ldcg(pold + i0 + 4);
            }
            kx4 = __ldg(kx + i0 + 4);
          }
          float pv[4] = {pc.x, pc.y, pc.z, pc.w};
          const float pvu[4] = {pu.x, pu.y, pu.z, pu.w};
          const float pvd[4] = {pd.x, pd.y, pd.z, pd.w};
          const float kxv[5] = {kxc.x, kxc.y, kxc.z, kxc.w, kx4};
          const float kyv[4] = {kyc.x, kyc.y, kyc.z, kyc.w};
          const float kyuv[4] = {kyu.x, kyu.y, kyu.z, kyu.w};
          float wv[4] = {0.f, 0.f, 0.f, 0.f};
          float outp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int kk = kk0 + q;
            if (!(row && kk >= hd && kk < x - hd)) continue;
            const float a = pv[q];
            const float al = (kk == hd) ? a : (q == 0 ? pl : pv[q - 1]);
            const float ar = (kk == x - hd - 1) ? a : (q == 3 ? pr : pv[q + 1]);
            const float ad = (jj == hd) ? a : pvd[q];
            const float au = (jj == y - hd - 1) ? a : pvu[q];
            const float wq = a + kxv[q + 1] * (a - ar) + kxv[q] * (a - al) +
                             kyuv[q] * (a - au) + kyv[q] * (a - ad);
            wv[q] = wq;
            outp[q] = a;
            pw += wq * a;
          }
          if (i0 < len) {
            *reinterpret_cast<float4*>(pnew + i0) = make_float4(outp[0], outp[1], outp[2], outp[3]);
            *reinterpret_cast<float4*>(w + i0) = make_float4(wv[0], wv[1], wv[2], wv[3]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const unsigned i = i0 + q;
            if (i >= len) continue;
            const int jj = (int)(i / (unsigned)x);
            const int kk = (int)(i - (unsigned)jj * (unsigned)x);
            float a = 0.f, wq = 0.f;
            if (jj >= hd && jj < y - hd && kk >= hd && kk < x - hd) {
              auto pn = [&](unsigned j) { return zval(P, __ldcg(r + j), j) + bf * __ldcg(pold + j); };
              a = pn(i);
              const float al = (kk == hd) ? a : pn(i - 1);
              const float ar = (kk == x - hd - 1) ? a : pn(i + 1);
              const float ad = (jj == hd) ? a : pn(i - x);
              const float au = (jj == y - hd - 1) ? a : pn(i + x);
              wq = a + kx[i + 1] * (a - ar) + kx[i] * (a - al) + ky[i + x] * (a - au) +
                   ky[i] * (a - ad);
              pw += wq * a;
            }
            pnew[i] = a;
            w[i] = wq;
          }
        }
      }
      {
        const float t = block_sum_f(pw, s_warp[0]);
        if (threadIdx.x == 0) P.part_pw[blockIdx.x] = (double)t;
      }
      if (!tl_grid_barrier(P.sync, P.status)) break;
      const double pwsum = tl_reduce_partials(P.part_pw, G, s_scratch);
      const double alpha = rz_old / pwsum;
      const float af = (float)alpha;

      /* ---- phase 2: e += alpha p, r -= alpha w, r.r and r.z (reverse order) */
      const int count = (P.ntiles - 1 - blockIdx.x) / G + 1;
      float rr = 0.0f, rz = 0.0f;
#pragma unroll 2
      for (int c = count - 1; c >= 0; --c) {
        const int tile = blockIdx.x + c * G;
        const unsigned i0 = (unsigned)tile * TL_TILE + 4u * threadIdx.x;
        if (i0 < len) {
          if (kVec) {
            const float4 pp = __ldcg(reinterpret_cast<const float4*>(pnew + i0));
            const float4 ww = __ldcg(reinterpret_cast<const float4*>(w + i0));
            float4 ee = __ldcg(reinterpret_cast<const float4*>(e + i0));
            float4 rv = __ldcg(reinterpret_cast<const float4*>(r + i0));
            ee.x += af * pp.x; ee.y += af * pp.y; ee.z += af * pp.z; ee.w += af * pp.w;
            rv.x -= af * ww.x; rv.y -= af * ww.y; rv.z -= af * ww.z; rv.w -= af * ww.w;
            *reinterpret_cast<float4*>(e + i0) = ee;
            *reinterpret_cast<float4*>(r + i0) = rv;
            rr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
            if (P.jacobi) {
              const float4 d = __ldg(reinterpret_cast<const float4*>(P.invd + i0));
              rz += rv.x * rv.x * d.x + rv.y * rv.y * d.y + rv.z * rv.z * d.z + rv.w * rv.w * d.w;
            }
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const unsigned i = i0 + q;
              if (i >= len) continue;
              const float ev = e[i] + af * pnew[i];
              const float rv = r[i] - af * w[i];
              e[i] = ev;
              r[i] = rv;
              rr += rv * rv;
              if (P.jacobi) rz += rv * rv * __ldg(P.invd + i);
            }
          }
        }
      }
      /* Cells outside the interior hold r = 0 and contribute nothing. */
      const float t1 = block_sum_f(rr, s_warp[1]);
      const float t2 = P.jacobi ? block_sum_f(rz, s_warp[2]) : t1;
      if (threadIdx.x == 0) {
        P.part_rr[blockIdx.x] = (double)t1;
        P.part_rz[blockIdx.x] = (double)t2;
      }
    } else {
      /* ---- step 0: r.r and r.z of the incoming residual */
      float rr = 0.0f, rz = 0.0f;
      for (int tile = blockIdx.x; tile < P.ntiles; tile += G) {
        const unsigned i0 = (unsigned)tile * TL_TILE + 4u * threadIdx.x;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const unsigned i = i0 + q;
          if (i >= len) continue;
          const float rv = __ldcg(r + i);
          rr += rv * rv;
          if (P.jacobi) rz += rv * rv * __ldg(P.invd + i);
        }
      }
      const float t1 = block_sum_f(rr, s_warp[1]);
      const float t2 = P.jacobi ? block_sum_f(rz, s_warp[2]) : t1;
      if (threadIdx.x == 0) {
        P.part_rr[blockIdx.x] = (double)t1;
        P.part_rz[blockIdx.x] = (double)t2;
      }
    }
    if (!tl_grid_barrier(P.sync, P.status)) break;
    const double rr = tl_reduce_partials(P.part_rr, G, s_scratch);
    const double rz = P.jacobi ? tl_reduce_partials(P.part_rz, G, s_scratch) : rr;
    if (k == 0) {
      rr0 = rr;
      beta = 0.0;
    } else {
      beta = rz / rz_old;
      parity ^= 1;
    }
    rz_old = rz;
    iters = k;
    if (rr <= P.tol2 * rr0 || !(rr == rr) || k == P.max_iters) {
      if (blockIdx.x == 0 && threadIdx.x == 0) *P.rr_out = rr;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.iters_out = iters;
}

/* r32 = r64 * scale on the interior (0 elsewhere); e32 = 0; p buffers = 0. */
__global__ void demote_kernel(int x, int y, int hd, const double* r64, double scale,
                              float* r32, float* e32, float* pa, float* pb) {
  const unsigned len = (unsigned)x * (unsigned)y;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    const bool in = kk >= hd && kk < x - hd && jj >= hd && jj < y - hd;
    r32[i] = in ? (float)(r64[i] * scale) : 0.0f;
    e32[i] = 0.0f;
    pa[i] = 0.0f;
    pb[i] = 0.0f;
  }
}

/* FP32 coefficients and the inverse diagonal of A32 (for Jacobi). */
__global__ void coeff_kernel(int x, int y, int hd, const double* kx, const double* ky,
                             float* kx32, float* ky32, float* invd) {
  const unsigned len = (unsigned)x * (unsigned)y;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    kx32[i] = (float)kx[i];
    ky32[i] = (float)ky[i];
    float d = 1.0f;
    if (kk >= hd && kk < x - hd && jj >= hd && jj < y - hd) {
      /* zero-flux boundary: a boundary coefficient multiplies (a - a) = 0 */
      const float kr = (kk == x - hd - 1) ? 0.0f : (float)kx[i + 1];
      const float kl = (kk == hd) ? 0.0f : (float)kx[i];
      const float ku = (jj == y - hd - 1) ? 0.0f : (float)ky[i + x];
      const float kd = (jj == hd) ? 0.0f : (float)ky[i];
      d = 1.0f + kr + kl + ku + kd;
    }
    invd[i] = 1.0f / d;
  }
}

/* u += e32 / scale on the interior (FP64 accumulation). */
__global__ void promote_add_kernel(int x, int y, int hd, const float* e32, double inv_scale,
                                   double* u) {
  const unsigned len = (unsigned)x * (unsigned)y;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    if (kk >= hd && kk < x - hd && jj >= hd && jj < y - hd)
      u[i] = u[i] + (double)e32[i] * inv_scale;
  }
}

/* The diagonal of the 5-point operator on the interior, 1 + (kx[i+1] +
 * kx[i]) + (ky[i+x] + ky[i]), kept per operator for the true residuals of
 * the replacement path. */
__global__ void diag64_kernel(int x, int y, int hd, const double* __restrict__ kx,
                              const double* __restrict__ ky, double* __restrict__ diag) {
  const unsigned len = (unsigned)x * (unsigned)y;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    if (kk >= hd && kk < x - hd && jj >= hd && jj < y - hd)
      diag[i] = 1.0 + (kx[i + 1] + kx[i]) + (ky[i + x] + ky[i]);
  }
}

/* The replacement path's true residual: r = u0 - A u over the interior with
 * fused multiply-adds on the precomputed diagonal (6 FP64 operations per
 * cell with r.r, against 14 in the reference's grouping; this is the solver's
 * own stop check, not a drop-in kernel), and r.r as one FP64 partial per
 * block in part (summed by the host in block order). */
constexpr int kResThreads = 256;
__global__ void __launch_bounds__(kResThreads)
residual64_kernel(int x, int y, int hd, const double* __restrict__ u,
                  const double* __restrict__ u0, const double* __restrict__ kx,
                  const double* __restrict__ ky, const double* __restrict__ diag,
                  double* __restrict__ r, double* part) {
  __shared__ double s_w[kResThreads / 32];
  const unsigned len = (unsigned)x * (unsigned)y;
  double acc = 0.0;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += gridDim.x * blockDim.x) {
    const int jj = (int)(i / (unsigned)x);
    const int kk = (int)(i - (unsigned)jj * (unsigned)x);
    if (kk >= hd && kk < x - hd && jj >= hd && jj < y - hd) {
      double v = fma(-diag[i], u[i], u0[i]);
      v = fma(ky[i], u[i - x], v);
      v = fma(ky[i + x], u[i + x], v);
      v = fma(kx[i], u[i - 1], v);
      v = fma(kx[i + 1], u[i + 1], v);
      r[i] = v;
      acc = fma(v, v, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(TL_FULL_MASK, acc, o);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kResThreads / 32; ++w) t += s_w[w];
    part[blockIdx.x] = t;
  }
}

int grid_for(tl_context* ctx, unsigned len) {
  unsigned b = (len + 255) / 256;
  const unsigned cap = (unsigned)ctx->num_sms * 16u;
  return (int)std::max(1u, std::min(b, cap));
}

}  // namespace

/* Scratch of the mixed solvers: kMixedFields float arrays of x*y cells,
 * each starting on a 256-byte boundary (slot k at d_f32 + k * f32_cap). */
constexpr int kMixedFields = 10;
static int ensure_mixed(tl_context* ctx, size_t n) {
  n = (n + 63) & ~(size_t)63;
  if (n <= ctx->f32_cap) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->packed_kind = 0;
  cudaFree(ctx->d_f32);
  ctx->d_f32 = nullptr;
  ctx->f32_cap = 0;
  TL_CUDA(cudaMalloc(&ctx->d_f32, kMixedFields * n * sizeof(float)));
  ctx->f32_cap = n;
  return TL_OK;
}

static int norm2(tl_context* ctx, int x, int y, int hd, const double* f, double* out) {
  *out = 0.0;
  return tl_calculate_2norm(ctx, x, y, hd, f, out);
}

extern "C" int tl_solve(tl_context* ctx, int x, int y, int hd, int coefficient, double rx,
                        double ry, const tl_solve_params* prm, double* p, double* r,
                        double* u, double* u0, double* w, double* kx, double* ky,
                        const double* density, const double* energy, tl_solve_report* rep) {
  TL_REQUIRE(ctx && prm && rep, "tl_solve: null argument");
  TL_REQUIRE(x > 2 * hd && y > 2 * hd && hd >= 1, "invalid grid dimensions");
  TL_REQUIRE((size_t)x * (size_t)y <= (size_t)TL_MAX_CELLS,
             "grid larger than TL_MAX_CELLS (536,870,912 cells)");
  TL_REQUIRE(prm->rel_tol > 0.0, "tl_solve: rel_tol must be positive");
  *rep = tl_solve_report{};
  const unsigned len = (unsigned)x * (unsigned)y;
  float ms_total = 0.0f;
  /* the whole solve's events, released on every return path */
  struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EventPair() {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
    }
  } ev;
  TL_CUDA(cudaEventCreate(&ev.a));
  TL_CUDA(cudaEventCreate(&ev.b));
  cudaEvent_t t0 = ev.a, t1 = ev.b;
  TL_CUDA(cudaEventRecord(t0, ctx->stream));

  /* Set-up as the reference's cg_init_driver: u = energy*density, kx, ky,
   * halos, u0 = u. FP64 CG from u0 takes it whole (r, p and rro as the
   * reference's CG loop starts from them); the other paths compute their own
   * true residual and take it without cg_init_others, and without
   * recomputing kx, ky when density, rx, ry, the coefficient kind and kx,
   * ky themselves are what they were after the last such set-up (content
   * hashes): the couplings are a function of those alone. */
  double rro = 0.0;
  const bool reference_cg = prm->method == TL_METHOD_CG64 && prm->projection <= 0;
  unsigned long long op_hash = 0;
  int rc;
  if (reference_cg) {
    rc = tl_internal_cg_setup(ctx, x, y, hd, coefficient, rx, ry, p, r, u, u0, w, kx, ky,
                              density, energy, &rro);
    if (rc != TL_OK) return rc;
  } else {
    uint64_t brx, bry;
    memcpy(&brx, &rx, sizeof(brx));
    memcpy(&bry, &ry, sizeof(bry));
    const unsigned long long salt =
        brx * 0x9E3779B97F4A7C15ull ^ bry * 0xC2B2AE3D27D4EB4Full ^ (unsigned)coefficient;
    unsigned long long hdens = 0, hk = 0;
    rc = tl_internal_hash64(ctx, density, kx, ky, len, salt, &hdens, &hk);
    if (rc != TL_OK) return rc;
    const bool current = ctx->op_x == x && ctx->op_y == y && ctx->op_hd == hd &&
                         ctx->op_dens_hash == hdens && ctx->op_k_hash == hk;
    rc = tl_internal_cg_setup_lean(ctx, x, y, hd, coefficient, rx, ry, p, r, u, u0, w, kx, ky,
                                   density, energy, current);
    if (rc != TL_OK) return rc;
    if (!current) {
      rc = tl_internal_hash64(ctx, nullptr, kx, ky, len, 0, nullptr, &hk);
      if (rc != TL_OK) return rc;
      ctx->op_x = x;
      ctx->op_y = y;
      ctx->op_hd = hd;
      ctx->op_dens_hash = hdens;
      ctx->op_k_hash = hk;
    }
    op_hash = hk;
  }
  /* Starting guess from the solutions of earlier solves with this operator
   * (its pass also sums u0.u0 when it runs; bb < 0 otherwise). */
  int basis = 0;
  double bb = -1.0;
  if (prm->projection > 0) {
    rc = tl_internal_project_guess(ctx, prm->projection, x, y, hd, op_hash, u0, u, &basis, &bb);
    if (rc != TL_OK) return rc;
  }
  if (!(bb >= 0.0)) {
    rc = norm2(ctx, x, y, hd, u0, &bb);
    if (rc != TL_OK) return rc;
  }
  const double bnorm = sqrt(bb);
  const double target = prm->rel_tol * bnorm;

  /* the operator's diagonal for the replacement path's residuals (kept in
   * the context while the operator does not change) */
  if (!reference_cg) {
    const unsigned long long diag_id =
        op_hash ^ ((unsigned long long)x << 40) ^ ((unsigned long long)y << 16) ^ (unsigned)hd;
    if (!ctx->d_diag64 || ctx->diag64_cap < (size_t)len || ctx->diag64_id != diag_id) {
      if (ctx->diag64_cap < (size_t)len) {
        TL_CUDA(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->d_diag64);
        ctx->d_diag64 = nullptr;
        ctx->diag64_cap = 0;
        TL_CUDA(cudaMalloc(&ctx->d_diag64, (size_t)len * sizeof(double)));
        ctx->diag64_cap = len;
      }
      diag64_kernel<<<grid_for(ctx, len), 256, 0, ctx->stream>>>(x, y, hd, kx, ky,
                                                                ctx->d_diag64);
      TL_CHECK_LAUNCH(ctx);
      ctx->diag64_id = diag_id;
    }
  }
  const int res_grid = 4 * ctx->num_sms;
  if (!reference_cg) {
    rc = tl_ensure_partials(ctx, (size_t)res_grid);
    if (rc != TL_OK) return rc;
  }
  std::vector<double> res_part(res_grid);
  auto true_residual = [&](double* out) -> int {
    double rrv = 0.0;
    if (reference_cg) {
      int e = tl_internal_residual_norm(ctx, x, y, hd, u, u0, r, kx, ky, &rrv);
      *out = sqrt(rrv);
      return e;
    }
    residual64_kernel<<<res_grid, kResThreads, 0, ctx->stream>>>(x, y, hd, u, u0, kx, ky,
                                                                 ctx->d_diag64, r, ctx->d_part);
    TL_CHECK_LAUNCH(ctx);
    TL_CUDA(cudaMemcpyAsync(res_part.data(), ctx->d_part, res_grid * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int g = 0; g < res_grid; ++g) rrv += res_part[g];
    *out = sqrt(rrv);
    return TL_OK;
  };

  /* FP64 CG from the current u until the true residual meets the target:
   * CG stops on its recursive residual, which can end a little below the
   * true one, so up to two restarts from the true residual follow. Returns
   * the final true residual norm in *rn. */
  auto cg64_to_target = [&](int max_steps, int* steps_total, float* kernel_ms,
                            double* rn) -> int {
    double* uu1[1] = {u};
    for (int round = 0; round < 3; ++round) {
      int steps = 0;
      int e = tl_internal_cg64_from_iterate(ctx, x, y, hd, target, max_steps - *steps_total, p,
                                            r, u, u0, w, kx, ky, &steps);
      if (e != TL_OK) return e;
      *steps_total += steps;
      *kernel_ms += ctx->last_solve.kernel_ms;
      e = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu1, 1);
      if (e != TL_OK) return e;
      e = true_residual(rn);
      if (e != TL_OK) return e;
      if (*rn <= target || *steps_total >= max_steps || steps == 0) break;
    }
    return TL_OK;
  };

  /* A starting guess is kept while it is good: with u's halos current, rn
   * holds its true residual norm on entry; a guess whose relative residual
   * exceeds kGuessCheck is compared with u = u0 and the better one is kept
   * (rn and r follow). */
  constexpr double kGuessCheck = 1e-4;
  double* uu0[1] = {u};
  auto settle_guess = [&](double* rn) -> int {
    if (basis == 0 || !(*rn > kGuessCheck * bnorm)) return TL_OK;
    const double rn_guess = *rn;
    TL_CUDA(cudaMemcpyAsync(u, u0, (size_t)len * sizeof(double), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    int e = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu0, 1);
    if (e != TL_OK) return e;
    e = true_residual(rn);
    if (e != TL_OK) return e;
    if (*rn <= rn_guess) {
      basis = 0;
      return TL_OK;
    }
    e = tl_internal_project_recombine(ctx, x, y, hd, u);
    if (e != TL_OK) return e;
    e = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu0, 1);
    if (e != TL_OK) return e;
    return true_residual(rn);
  };
  if (prm->method == TL_METHOD_CG64) {
    int steps = 0;
    double* uu[1] = {u};
    if (!reference_cg) {
      /* FP64 CG from the guess (or from u0), restarted until the true
       * residual meets the target */
      double rn0 = 0.0;
      rc = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu, 1);
      if (rc != TL_OK) return rc;
      rc = true_residual(&rn0);
      if (rc != TL_OK) return rc;
      rc = settle_guess(&rn0);
      if (rc != TL_OK) return rc;
      rep->initial_rel_residual = bnorm > 0 ? rn0 / bnorm : rn0;
      double rn1 = 0.0;
      rc = cg64_to_target(prm->max_inner, &steps, &rep->inner_kernel_ms, &rn1);
      if (rc != TL_OK) return rc;
    } else {
      rep->initial_rel_residual = bnorm > 0 ? sqrt(rro) / bnorm : sqrt(rro);
      /* r = 0 (a zero right-hand side) is solved already; CG would form 0/0. */
      if (rro > 0.0) {
        rc = tl_internal_cg64_loop(ctx, x, y, hd, target, prm->max_inner, p, r, u, w, kx, ky,
                                   rro, nullptr, nullptr, &steps);
        if (rc != TL_OK) return rc;
      }
      rep->inner_kernel_ms = rro > 0.0 ? ctx->last_solve.kernel_ms : 0.0f;
    }
    rep->inner_steps = steps;
    rep->outer_steps = 1;
    double rn = 0.0;
    rc = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu, 1);
    if (rc != TL_OK) return rc;
    rc = true_residual(&rn);
    if (rc != TL_OK) return rc;
    rep->final_rel_residual = bnorm > 0 ? rn / bnorm : rn;
  } else {
    TL_REQUIRE(prm->method == TL_METHOD_MIXED_CG || prm->method == TL_METHOD_MIXED_JACOBI ||
                   prm->method == TL_METHOD_MIXED_LEARNED ||
                   prm->method == TL_METHOD_MIXED_LEARNED_LAYERS ||
                   prm->method == TL_METHOD_MIXED_LEARNED_COARSE,
               "tl_solve: unknown method");
    const bool layers = prm->method == TL_METHOD_MIXED_LEARNED_LAYERS;
    const bool two_level = prm->method == TL_METHOD_MIXED_LEARNED_COARSE;
    const bool learned = layers || two_level || prm->method == TL_METHOD_MIXED_LEARNED;
    const double inner_tol = prm->inner_tol > 0.0 ? prm->inner_tol : (learned ? 3e-6 : 1e-5);
    TL_REQUIRE(!learned || prm->learned, "tl_solve: the learned method needs a network");
    const int H = y - 2 * hd, W = x - 2 * hd;
    TL_REQUIRE(!layers || (H % 4 == 0 && W % 64 == 0),
               "tl_solve: the layer-by-layer network needs interior sizes H % 4 == 0, W % 64 == 0");
    TL_REQUIRE(!learned || layers || W % 4 == 0,
               "tl_solve: the learned preconditioner needs an interior width W % 4 == 0");
    rc = ensure_mixed(ctx, len);
    if (rc != TL_OK) return rc;
    const size_t ntiles = tl_num_tiles(x, y);
    rc = tl_ensure_partials(ctx, ntiles);
    if (rc != TL_OK) return rc;
    float* f = ctx->d_f32;
    const size_t cap = ctx->f32_cap;
    float *kx32 = f, *ky32 = f + cap, *invd = f + 2 * cap, *r32 = f + 3 * cap,
          *e32 = f + 4 * cap, *w32 = f + 5 * cap, *pa = f + 6 * cap, *pb = f + 7 * cap,
          *z32 = f + 8 * cap, *r32b = f + 9 * cap;
    tl_coarse_level coarse;
    /* the FP32 coefficients, packed again only when the operator or the
     * layout changed (the scratch is tl_solve's alone) */
    const unsigned long long packed_id =
        op_hash ^ ((unsigned long long)x << 40) ^ ((unsigned long long)y << 16) ^ (unsigned)hd;
    const int kind = learned ? 1 : 2;
    const bool packed = ctx->packed_kind == kind && ctx->packed_hash == packed_id;
    ctx->packed_kind = 0;
    if (learned) {
      /* packed layout: kx32, ky32, invd hold the packed kx, ky, s */
      if (!packed) {
        rc = tl_pack_coefficients(ctx, x, y, hd, kx, ky, kx32, ky32, invd);
        if (rc != TL_OK) return rc;
      }
      if (two_level) {
        /* the coarse level of this operator (rebuilt only when it changes) */
        const unsigned long long coarse_id = packed_id * 0xFF51AFD7ED558CCDull;
        rc = tl_internal_coarse_prepare(ctx, H, W, kx32, ky32, &coarse, &coarse_id);
        if (rc != TL_OK) return rc;
      }
    } else if (!packed) {
      coeff_kernel<<<grid_for(ctx, len), 256, 0, ctx->stream>>>(x, y, hd, kx, ky, kx32, ky32,
                                                                invd);
      TL_CHECK_LAUNCH(ctx);
    }
    ctx->packed_kind = kind;
    ctx->packed_hash = packed_id;
    const bool vec = (x % 4) == 0;
    const void* kernel = vec ? (const void*)inner_cg_kernel<true> : (const void*)inner_cg_kernel<false>;
    int per_sm = 0;
    TL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0));
    TL_REQUIRE(per_sm >= 1, "inner CG kernel cannot be resident");
    int grid = std::min<int>(ctx->num_sms, (int)ntiles);

    double* uu[1] = {u};
    double prev = 0.0;
    for (int outer = 0; outer <= prm->max_outer; ++outer) {
      rc = tl_local_halos(ctx, x, y, hd, 1, 0xF, uu, 1);
      if (rc != TL_OK) return rc;
      double rn = 0.0;
      rc = true_residual(&rn);
      if (rc != TL_OK) return rc;
      if (outer == 0) {
        rc = settle_guess(&rn);
        if (rc != TL_OK) return rc;
      }
      if (outer == 0) rep->initial_rel_residual = bnorm > 0 ? rn / bnorm : rn;
      rep->final_rel_residual = bnorm > 0 ? rn / bnorm : rn;
      if (rn <= target) break;
      const bool stalled = outer > 0 && rn > prm->stall_factor * prev;
      const bool exhausted = outer == prm->max_outer;
      if (stalled || exhausted || !(rn == rn)) {
        /* Refinement no longer converges, or has used its max_outer steps
         * without reaching the target: finish with the exact FP64 CG from
         * the current iterate. */
        rep->fallback_events++;
        int steps = 0;
        rc = cg64_to_target(prm->max_fallback, &steps, &rep->inner_kernel_ms, &rn);
        if (rc != TL_OK) return rc;
        rep->fallback_steps += steps;
        rep->final_rel_residual = bnorm > 0 ? rn / bnorm : rn;
        break;
      }
      prev = rn;
      const double scale = sqrt((double)(x - 2 * hd) * (double)(y - 2 * hd)) / rn;
      if (learned) {
        const double need = 0.5 * target / rn;
        const double tol = std::max(inner_tol, std::min(need, 0.5));
        rc = tl_pack_interior(ctx, x, y, hd, r, scale, r32);
        if (rc != TL_OK) return rc;
        int it = 0;
        double rr_in = 0.0;
        TL_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
        if (layers) {
          rc = tl_internal_fpcg_learned(ctx, prm->learned, H, W, kx32, ky32, invd, r32, e32, pa,
                                        w32, pb, tol, prm->max_inner, &it);
        } else {
          const void* umma = nullptr;
          const float* kscale = nullptr;
          rc = tl_internal_net_stencil(prm->learned, &umma, &kscale);
          if (rc != TL_OK) return rc;
          rc = tl_internal_fpcg_collapsed(ctx, umma, kscale, H, W, kx32, ky32, invd, r32, r32b,
                                          e32, w32, z32, pa, pb, tol, prm->max_inner, &it,
                                          &rr_in, two_level ? &coarse : nullptr);
        }
        if (rc != TL_OK) return rc;
        TL_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
        TL_CUDA(cudaStreamSynchronize(ctx->stream));
        /* A broken-down inner solve (non-finite residual) contributes no
         * correction; the next outer step then sees no progress and falls
         * back to FP64 CG. */
        if (layers) rr_in = ((volatile double*)ctx->h_result)[7];
        if (rr_in == rr_in && rr_in < 1e300) {
          rc = tl_internal_unpack_add(ctx, x, y, hd, e32, 1.0 / scale, u);
          if (rc != TL_OK) return rc;
        }
        TL_CUDA(cudaStreamSynchronize(ctx->stream));
        float kms = 0.0f;
        TL_CUDA(cudaEventElapsedTime(&kms, ctx->ev_start, ctx->ev_stop));
        rep->inner_kernel_ms += kms;
        rep->inner_steps += it;
        rep->outer_steps = outer + 1;
        continue;
      }
      demote_kernel<<<grid_for(ctx, len), 256, 0, ctx->stream>>>(x, y, hd, r, scale, r32, e32,
                                                                  pa, pb);
      TL_CHECK_LAUNCH(ctx);
      InnerParams P;
      P.x = x; P.y = y; P.hd = hd; P.ntiles = (int)ntiles; P.max_iters = prm->max_inner;
      P.jacobi = prm->method == TL_METHOD_MIXED_JACOBI;
      /* Ask each inner solve for no more than the remaining reduction (with
       * a factor 0.5 of margin), so the last refinement step does not
       * overshoot the target. */
      const double need = 0.5 * target / rn;
      const double tol = std::max(inner_tol, std::min(need, 0.5));
      P.tol2 = tol * tol;
      P.kx = kx32; P.ky = ky32; P.invd = invd;
      P.r = r32; P.e = e32; P.w = w32; P.pa = pa; P.pb = pb;
      P.part_pw = ctx->d_part; P.part_rr = ctx->d_part + ctx->part_cap;
      P.part_rz = ctx->d_part + 2 * ctx->part_cap;
      P.sync = ctx->d_sync; P.status = ctx->d_status;
      P.iters_out = ctx->d_steps; P.rr_out = ctx->d_result;
      TL_CUDA(cudaMemsetAsync(ctx->d_sync + TL_SYNC_BAR_COUNT, 0, 2 * sizeof(unsigned),
                              ctx->stream));
      TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
      ctx->h_steps[0] = -1;
      int parity0 = 0;
      void* args[] = {&P, &parity0};
      TL_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
      TL_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(kThreads), args, 0,
                                          ctx->stream));
      TL_CHECK_LAUNCH(ctx);
      TL_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
      int status = 0;
      TL_CUDA(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                              ctx->stream));
      TL_CUDA(cudaStreamSynchronize(ctx->stream));
      if (status != 0) return tl_set_error(status, "inner CG kernel: grid-barrier timeout");
      const double rr_in = ((volatile double*)ctx->h_result)[0];
      if (rr_in == rr_in && rr_in < 1e300) {
        promote_add_kernel<<<grid_for(ctx, len), 256, 0, ctx->stream>>>(x, y, hd, e32,
                                                                         1.0 / scale, u);
        TL_CHECK_LAUNCH(ctx);
      }
      rep->inner_steps += ((volatile int*)ctx->h_steps)[0];
      float kms = 0.0f;
      TL_CUDA(cudaEventElapsedTime(&kms, ctx->ev_start, ctx->ev_stop));
      rep->inner_kernel_ms += kms;
      rep->outer_steps = outer + 1;
    }
    /* leave u, p with their depth-1 halos as the CG driver would */
    double* up[2] = {u, p};
    rc = tl_local_halos(ctx, x, y, hd, 1, 0xF, up, 2);
    if (rc != TL_OK) return rc;
  }
  /* r is the true residual of the final u in both branches */
  if (prm->projection > 0) {
    rc = tl_internal_project_push(ctx, x, y, hd, u0, u, r, kx, ky, ctx->d_diag64);
    if (rc != TL_OK) return rc;
  }
  rep->projection_basis = basis;
  TL_CUDA(cudaEventRecord(t1, ctx->stream));
  TL_CUDA(cudaEventSynchronize(t1));
  TL_CUDA(cudaEventElapsedTime(&ms_total, t0, t1));
  rep->device_ms = ms_total;
  ctx->last_solve.kernel_ms = ms_total;
  ctx->last_solve.steps = rep->inner_steps + rep->fallback_steps;
  return TL_OK;
}
