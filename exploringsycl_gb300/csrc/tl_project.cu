/*
 * tl_project.cu -- starting guesses for a sequence of solves with one
 * operator (tl_solve_params.projection > 0).
 *
 * TeaLeaf solves A u_t = u_{t-1} once per timestep with the same A (density
 * and dt do not change), and the reference starts each solve from x0 = b
 * (TeaLeaf/drivers/cg_driver.c:56-65). The solutions of consecutive
 * timesteps lie close to a low-dimensional space: the A-norm best
 * approximation of the new solution from b and the last few solutions
 * leaves an initial residual several orders of magnitude below that of
 * x0 = b. This is the projection method for successive right-hand sides of
 * P. F. Fischer, "Projection techniques for iterative solution of Ax = b
 * with successive right-hand sides", Comput. Methods Appl. Mech. Engrg. 163
 * (1998) 193-204, in the form that keeps the raw solutions and solves the
 * small Galerkin system each time:
 *
 *   V = [b, x_1 .. x_m] (x_j the held solutions), G = V^T A V, g = V^T b,
 *   x0 = V c with G c = g,
 *
 * which minimises ||x* - x0||_A over span(V). The solutions of consecutive
 * timesteps are nearly parallel (and b equals the newest one up to
 * rounding), so G is very ill-conditioned; the useful information sits in
 * directions whose eigenvalues are 1e-10 .. 1e-15 of the largest. G is
 * scaled to unit diagonal and solved by its eigen-decomposition (cyclic
 * Jacobi rotations, which resolve small eigenvalues of a scaled positive
 * definite matrix to high relative accuracy), dropping eigenvalues below
 * 1e-15 of the largest.
 *
 * No product with A is formed for the Gram matrix: A b = b - r0 with r0 the
 * residual of u = b that cg_init computes, and after the solve A u = b - r
 * with r the final true residual. Per solve this costs two passes of FP64
 * dot products (2m + 2 and 2m + 2 per cell, FP64-throughput bound on this
 * part) and one combination pass.
 *
 * The held solutions belong to one operator: a 64-bit content hash of kx
 * and ky (and the grid's shape) is compared before each solve, and a
 * different operator drops them. tl_projection_reset drops them on request.
 * The guess is kept only if its true residual is below that of x0 = b;
 * otherwise the solve starts from b as the reference does.
 */
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "tl_internal.cuh"

namespace {

constexpr int kDotThreads = 256;
constexpr int kMaxVec = TL_PROJ_MAX + 1;  /* b and the held solutions */
constexpr double kEigCut = 1e-15;

struct VecList {
  const double* v[kMaxVec];
};
struct CoefList {
  double c[kMaxVec];
};

/* Order-independent 64-bit hash of the operator's couplings (all x*y words
 * of kx and ky, halos included: cg_init writes them deterministically). */
__global__ void operator_hash_kernel(const double* __restrict__ kx, const double* __restrict__ ky,
                                     size_t n, unsigned long long* out) {
  __shared__ unsigned long long s[kDotThreads / 32];
  unsigned long long h = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long a = (unsigned long long)__double_as_longlong(kx[i]);
    unsigned long long b = (unsigned long long)__double_as_longlong(ky[i]);
    unsigned long long v = a ^ (b * 0xD6E8FEB86659FD93ull) ^ ((unsigned long long)i * 0x9E3779B97F4A7C15ull);
    v ^= v >> 32;
    v *= 0xBF58476D1CE4E5B9ull;
    v ^= v >> 29;
    h += v;
  }
  for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = h;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += s[w];
    atomicAdd(out, t);
  }
}

/* For each listed vector a_j (j < na): a_j . p and a_j . q over the
 * interior, into out[block][2 j + {0, 1}] (one FP64 partial per block,
 * summed in a fixed order inside the block; the host adds the blocks in
 * block order). */
__global__ void __launch_bounds__(kDotThreads) proj_dots_kernel(int x, int y, int hd, VecList a,
                                                                int na,
                                                                const double* __restrict__ p,
                                                                const double* __restrict__ q,
                                                                double* out) {
  __shared__ double s[kDotThreads / 32][2 * kMaxVec];
  double acc[2 * kMaxVec];
#pragma unroll
  for (int k = 0; k < 2 * kMaxVec; ++k) acc[k] = 0.0;
  const int W = x - 2 * hd, H = y - 2 * hd;
  const size_t n = (size_t)W * H;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)W, col = i - row * (size_t)W;
    const size_t f = (row + hd) * (size_t)x + col + hd;
    const double pv = p[f], qv = q[f];
#pragma unroll
    for (int j = 0; j < kMaxVec; ++j) {
      if (j < na) {
        const double av = a.v[j][f];
        acc[2 * j] += av * pv;
        acc[2 * j + 1] += av * qv;
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 2 * kMaxVec; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 * na) {
    double t = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += s[w][threadIdx.x];
    out[(size_t)blockIdx.x * 2 * na + threadIdx.x] = t;
  }
}

/* out = sum_j c_j a_j over the interior (halos untouched). */
__global__ void proj_combine_kernel(int x, int y, int hd, VecList a, CoefList c, int na,
                                    double* out) {
  const int W = x - 2 * hd, H = y - 2 * hd;
  const size_t n = (size_t)W * H;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)W, col = i - row * (size_t)W;
    const size_t f = (row + hd) * (size_t)x + col + hd;
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < kMaxVec; ++j)
      if (j < na) v += c.c[j] * a.v[j][f];
    out[f] = v;
  }
}

/* Eigen-decomposition of the symmetric n x n matrix A (row-major, destroyed)
 * by cyclic Jacobi rotations: lam[k] and column k of V (V[i * n + k]). */
void jacobi_eigen(int n, double* A, double* lam, double* V) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i * n + j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += A[i * n + i] * A[i * n + i];
      for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    }
    if (off <= 1e-40 * diag) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (apq == 0.0) continue;
        /* the rotation that zeroes A[p][q]: tan of its angle t, the smaller
         * root of t^2 + 2 theta t - 1 = 0 */
        const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  /* columns p, q */
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  /* rows p, q */
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  for (int k = 0; k < n; ++k) lam[k] = A[k * n + k];
}

int grid_dots(const tl_context* ctx) { return 4 * ctx->num_sms; }

/* Runs proj_dots_kernel and sums its block partials on the host in block
 * order: out[2 j + {0, 1}] = a_j . p, a_j . q. */
int dots(tl_context* ctx, int x, int y, int hd, const VecList& a, int na, const double* p,
         const double* q, double* out) {
  const int G = grid_dots(ctx);
  proj_dots_kernel<<<G, kDotThreads, 0, ctx->stream>>>(x, y, hd, a, na, p, q, ctx->d_proj_part);
  TL_CHECK_LAUNCH(ctx);
  std::vector<double> h((size_t)G * 2 * na);
  TL_CUDA(cudaMemcpyAsync(h.data(), ctx->d_proj_part, h.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 2 * na; ++k) {
    double t = 0.0;
    for (int g = 0; g < G; ++g) t += h[(size_t)g * 2 * na + k];
    out[k] = t;
  }
  return TL_OK;
}

}  // namespace

int tl_internal_project_guess(tl_context* ctx, int slots, int x, int y, int hd,
                              const double* kx, const double* ky, const double* b,
                              const double* r0, double* u, int* basis) {
  *basis = 0;
  TL_REQUIRE(slots >= 1 && slots <= TL_PROJ_MAX, "tl_solve: projection must be 0 .. 8");
  const size_t len = (size_t)x * (size_t)y;
  /* storage: slots fields of len doubles, block partials */
  if (ctx->proj_slots != slots || ctx->proj_field_cap < len) {
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_proj);
    ctx->d_proj = nullptr;
    ctx->proj_slots = 0;
    ctx->proj_count = 0;
    TL_CUDA(cudaMalloc(&ctx->d_proj, (size_t)slots * len * sizeof(double)));
    ctx->proj_slots = slots;
    ctx->proj_field_cap = len;
  }
  if (!ctx->d_proj_part) {
    TL_CUDA(cudaMalloc(&ctx->d_proj_part,
                       (size_t)grid_dots(ctx) * 2 * kMaxVec * sizeof(double) + 64));
  }
  /* the operator's identity */
  unsigned long long* d_hash = reinterpret_cast<unsigned long long*>(
      ctx->d_proj_part + (size_t)grid_dots(ctx) * 2 * kMaxVec);
  TL_CUDA(cudaMemsetAsync(d_hash, 0, sizeof(unsigned long long), ctx->stream));
  operator_hash_kernel<<<2 * ctx->num_sms, kDotThreads, 0, ctx->stream>>>(kx, ky, len, d_hash);
  TL_CHECK_LAUNCH(ctx);
  unsigned long long hash = 0;
  TL_CUDA(cudaMemcpyAsync(&hash, d_hash, sizeof(hash), cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hash != ctx->proj_hash || x != ctx->proj_x || y != ctx->proj_y || hd != ctx->proj_hd) {
    ctx->proj_count = 0;
    ctx->proj_hash = hash;
    ctx->proj_x = x;
    ctx->proj_y = y;
    ctx->proj_hd = hd;
  }
  const int m = ctx->proj_count;
  if (m == 0) return TL_OK;
  /* V = [b, held solutions from the oldest]; G[0][j] = v_j . A b =
   * v_j . b - v_j . r0, g_j = v_j . b */
  VecList V;
  V.v[0] = b;
  for (int j = 0; j < m; ++j) V.v[1 + j] = ctx->d_proj + (size_t)ctx->proj_order[j] * len;
  const int n = m + 1;
  double d[2 * kMaxVec];
  int rc = dots(ctx, x, y, hd, V, n, b, r0, d);
  if (rc != TL_OK) return rc;
  double G[kMaxVec * kMaxVec], g[kMaxVec];
  for (int j = 0; j < n; ++j) {
    g[j] = d[2 * j];
    G[j] = G[j * n] = d[2 * j] - d[2 * j + 1];
  }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      G[(1 + i) * n + 1 + j] = ctx->proj_gram[ctx->proj_order[i]][ctx->proj_order[j]];
  /* scale to unit diagonal, eigen-decompose, solve on the kept eigenvalues */
  double s[kMaxVec];
  for (int i = 0; i < n; ++i) {
    if (!(G[i * n + i] > 0.0)) return TL_OK;  /* not positive: keep x0 = b */
    s[i] = 1.0 / sqrt(G[i * n + i]);
  }
  double Gs[kMaxVec * kMaxVec], lam[kMaxVec], Q[kMaxVec * kMaxVec];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Gs[i * n + j] = G[i * n + j] * s[i] * s[j];
  jacobi_eigen(n, Gs, lam, Q);
  double lmax = 0.0;
  for (int k = 0; k < n; ++k) lmax = std::max(lmax, lam[k]);
  CoefList c;
  for (int i = 0; i < kMaxVec; ++i) c.c[i] = 0.0;
  int kept = 0;
  for (int k = 0; k < n; ++k) {
    if (!(lam[k] > kEigCut * lmax)) continue;
    ++kept;
    double t = 0.0;
    for (int i = 0; i < n; ++i) t += Q[i * n + k] * g[i] * s[i];
    t /= lam[k];
    for (int i = 0; i < n; ++i) c.c[i] += Q[i * n + k] * t;
  }
  for (int i = 0; i < n; ++i) {
    c.c[i] *= s[i];
    if (!(c.c[i] == c.c[i]) || fabs(c.c[i]) > 1e300) return TL_OK;
  }
  proj_combine_kernel<<<4 * ctx->num_sms, 256, 0, ctx->stream>>>(x, y, hd, V, c, n, u);
  TL_CHECK_LAUNCH(ctx);
  *basis = kept;
  return TL_OK;
}

int tl_internal_project_push(tl_context* ctx, int x, int y, int hd, const double* b,
                             const double* u, const double* r) {
  if (ctx->proj_slots < 1 || ctx->proj_x != x || ctx->proj_y != y || ctx->proj_hd != hd)
    return TL_OK;
  const size_t len = (size_t)x * (size_t)y;
  /* the slot of the new solution: a free one, else the oldest */
  const int full = ctx->proj_count == ctx->proj_slots;
  const int slot = full ? ctx->proj_order[0] : ctx->proj_count;
  const int keep = full ? ctx->proj_count - 1 : ctx->proj_count;
  int order[TL_PROJ_MAX];
  for (int j = 0; j < keep; ++j) order[j] = ctx->proj_order[j + (full ? 1 : 0)];
  /* x_j . A u = x_j . b - x_j . r for the kept solutions and u itself */
  VecList V;
  for (int j = 0; j < keep; ++j) V.v[j] = ctx->d_proj + (size_t)order[j] * len;
  V.v[keep] = u;
  double d[2 * kMaxVec];
  int rc = dots(ctx, x, y, hd, V, keep + 1, b, r, d);
  if (rc != TL_OK) return rc;
  for (int j = 0; j <= keep; ++j) {
    const double v = d[2 * j] - d[2 * j + 1];
    const int other = j < keep ? order[j] : slot;
    ctx->proj_gram[slot][other] = v;
    ctx->proj_gram[other][slot] = v;
  }
  TL_CUDA(cudaMemcpyAsync(ctx->d_proj + (size_t)slot * len, u, len * sizeof(double),
                          cudaMemcpyDeviceToDevice, ctx->stream));
  order[keep] = slot;
  for (int j = 0; j <= keep; ++j) ctx->proj_order[j] = order[j];
  ctx->proj_count = keep + 1;
  return TL_OK;
}

extern "C" int tl_projection_reset(tl_context* ctx) {
  TL_REQUIRE(ctx, "tl_projection_reset: null context");
  ctx->proj_count = 0;
  ctx->proj_hash = 0;
  ctx->proj_x = ctx->proj_y = ctx->proj_hd = 0;
  return TL_OK;
}
