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
 * (1998) 193-204, in the form that solves the small Galerkin system each
 * time:
 *
 *   V a basis of span(x_1 .. x_m) (the last m solutions), G = V^T A V,
 *   g = V^T b, x0 = V c with G c = g,
 *
 * which minimises ||x* - x0||_A over that span. In TeaLeaf b itself is the
 * newest solution (u0 = energy * density, energy = u / density after the
 * previous solve), so the span holds it up to rounding.
 *
 * Basis. The solutions of consecutive timesteps are nearly parallel; their
 * own Gram matrix holds the directions that matter (the changes between
 * timesteps, and the changes of those) only in its last digits, and in FP64
 * at most 5 or 6 of 7 directions survive. The basis kept here is the newest
 * solution X and the differences d_k = x_k - x_{k-1} of consecutive ones,
 * each formed in FP64 from the full vectors, with its Gram matrix computed
 * from them: the same span, with every direction resolved (7 of 7 in the
 * CPU study that chose it, and a 10x smaller starting residual once the
 * plain basis saturates). G is scaled to unit diagonal and solved by its
 * eigen-decomposition (cyclic Jacobi rotations, which resolve small
 * eigenvalues of a scaled positive definite matrix to high relative
 * accuracy), dropping eigenvalues below 1e-15 of the largest.
 *
 * Cost per solve. Before: g (one FP64 dot product per basis vector, one
 * pass that also sums b.b for the solve's stop rule) and x0 (one pass). After: one pass that forms d = u - X, applies A
 * to it (the 5-point stencil on the difference) and its dot products with
 * X, d and the kept differences; the new solution's Gram row follows from
 * u = X + d (exact up to the rounding of d) as G[X][.] + G[d][.]. These
 * passes are bound by GB300's FP64 rate, about 0.9 ms at 4096^2 in all.
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
constexpr int kMaxVec = TL_PROJ_MAX + 1;  /* dot products of one pass, at most */
constexpr double kEigCut = 1e-15;

struct VecList {
  const double* v[kMaxVec];
};
/* pairs (a_k, p_k) of the dot products of one pass */
struct PairList {
  const double* a[kMaxVec];
  const double* p[kMaxVec];
};
struct CoefList {
  double c[kMaxVec];
};

/* Order-independent 64-bit hashes of n doubles: out[0] of a, out[1] of b
 * and c together (a or c may be NULL; b NULL skips out[1]). Each 32-bit half of
 * each double is mixed with its position (multiply, xorshift) and the mixed
 * words are summed modulo 2^64: any change of a word changes the sum unless
 * another change cancels it exactly. */
__device__ __forceinline__ unsigned long long mix32(unsigned w, unsigned pos) {
  w ^= pos * 0x9E3779B9u;
  w *= 0x85EBCA6Bu;
  w ^= w >> 13;
  w *= 0xC2B2AE35u;
  return (unsigned long long)w << (pos & 31u);
}

__global__ void hash64_kernel(const double* __restrict__ a, const double* __restrict__ b,
                              const double* __restrict__ c, size_t n, unsigned long long* out) {
  __shared__ unsigned long long s[2][kDotThreads / 32];
  unsigned long long ha = 0, hb = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const unsigned p = 4u * (unsigned)i;
    if (a) {
      const unsigned long long va = (unsigned long long)__double_as_longlong(a[i]);
      ha += mix32((unsigned)va, p) + mix32((unsigned)(va >> 32), p + 1u);
    }
    if (b) {
      const unsigned long long vb = (unsigned long long)__double_as_longlong(b[i]);
      hb += mix32((unsigned)vb, p) + mix32((unsigned)(vb >> 32), p + 1u);
      if (c) {
        const unsigned long long vc = (unsigned long long)__double_as_longlong(c[i]);
        hb += mix32((unsigned)vc, p + 2u) + mix32((unsigned)(vc >> 32), p + 3u);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ha += __shfl_xor_sync(0xffffffffu, ha, o);
    hb += __shfl_xor_sync(0xffffffffu, hb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s[0][threadIdx.x >> 5] = ha;
    s[1][threadIdx.x >> 5] = hb;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    unsigned long long t = 0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += s[threadIdx.x][w];
    atomicAdd(out + threadIdx.x, t);
  }
}

/* The dot products a_k . p_k (k < np) over the interior, into
 * out[block][k] (one FP64 partial per block, summed in a fixed order inside
 * the block; the host adds the blocks in block order). */
__global__ void __launch_bounds__(kDotThreads) proj_dots_kernel(int x, int y, int hd, PairList L,
                                                                int np, double* out) {
  __shared__ double s[kDotThreads / 32][kMaxVec];
  double acc[kMaxVec];
#pragma unroll
  for (int k = 0; k < kMaxVec; ++k) acc[k] = 0.0;
  const int W = x - 2 * hd, H = y - 2 * hd;
  const size_t n = (size_t)W * H;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)W, col = i - row * (size_t)W;
    const size_t f = (row + hd) * (size_t)x + col + hd;
#pragma unroll
    for (int k = 0; k < kMaxVec; ++k)
      if (k < np) acc[k] += L.a[k][f] * L.p[k][f];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kMaxVec; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < np) {
    double t = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += s[w][threadIdx.x];
    out[(size_t)blockIdx.x * np + threadIdx.x] = t;
  }
}

/* The pass after a solve with the held newest solution X: d = u - X over the
 * interior into dnew; A d by the 5-point operator of TeaLeaf/shared.h:59-63
 * (its diagonal precomputed, fused multiply-adds) applied to the difference
 * (u and X carry the same reflective halos, so d's boundary fluxes vanish as
 * u's do); and d . A d, X . A d and e_k . A d for the kept differences e_k,
 * into out[block][0], [1] and [2 + k]. */
__global__ void __launch_bounds__(kDotThreads)
proj_push_kernel(int x, int y, int hd, const double* __restrict__ u, const double* __restrict__ X,
                 const double* __restrict__ kx, const double* __restrict__ ky,
                 const double* __restrict__ diag, VecList e, int ne, double* __restrict__ dnew,
                 double* out) {
  __shared__ double s[kDotThreads / 32][kMaxVec];
  double acc[kMaxVec];
#pragma unroll
  for (int k = 0; k < kMaxVec; ++k) acc[k] = 0.0;
  const int W = x - 2 * hd, H = y - 2 * hd;
  const size_t n = (size_t)W * H;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / (size_t)W, col = i - row * (size_t)W;
    const size_t f = (row + hd) * (size_t)x + col + hd;
    const double d0 = u[f] - X[f];
    double ad = diag[f] * d0;
    ad = fma(-ky[f], u[f - x] - X[f - x], ad);
    ad = fma(-ky[f + x], u[f + x] - X[f + x], ad);
    ad = fma(-kx[f], u[f - 1] - X[f - 1], ad);
    ad = fma(-kx[f + 1], u[f + 1] - X[f + 1], ad);
    dnew[f] = d0;
    acc[0] += d0 * ad;
    acc[1] += X[f] * ad;
#pragma unroll
    for (int k = 0; k + 2 < kMaxVec; ++k)
      if (k < ne) acc[2 + k] += e.v[k][f] * ad;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kMaxVec; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 + ne) {
    double t = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += s[w][threadIdx.x];
    out[(size_t)blockIdx.x * (2 + ne) + threadIdx.x] = t;
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

/* Sums the block partials of the last pass on the host in block order:
 * out[k], k < np. */
int sum_partials(tl_context* ctx, int np, double* out) {
  const int G = grid_dots(ctx);
  std::vector<double> h((size_t)G * np);
  TL_CUDA(cudaMemcpyAsync(h.data(), ctx->d_proj_part, h.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < np; ++k) {
    double t = 0.0;
    for (int g = 0; g < G; ++g) t += h[(size_t)g * np + k];
    out[k] = t;
  }
  return TL_OK;
}

int dots(tl_context* ctx, int x, int y, int hd, const PairList& L, int np, double* out) {
  proj_dots_kernel<<<grid_dots(ctx), kDotThreads, 0, ctx->stream>>>(x, y, hd, L, np,
                                                                    ctx->d_proj_part);
  TL_CHECK_LAUNCH(ctx);
  return sum_partials(ctx, np, out);
}

double* slot_ptr(tl_context* ctx, int slot) {
  return ctx->d_proj + (size_t)slot * ctx->proj_field_cap;
}

}  // namespace

int tl_internal_project_guess(tl_context* ctx, int slots, int x, int y, int hd,
                              unsigned long long op_hash, const double* b, double* u,
                              int* basis, double* bb) {
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
    TL_CUDA(cudaMalloc(&ctx->d_proj_part, (size_t)grid_dots(ctx) * kMaxVec * sizeof(double)));
  }
  /* the operator's identity */
  if (op_hash != ctx->proj_hash || x != ctx->proj_x || y != ctx->proj_y || hd != ctx->proj_hd) {
    ctx->proj_count = 0;
    ctx->proj_hash = op_hash;
    ctx->proj_x = x;
    ctx->proj_y = y;
    ctx->proj_hd = hd;
  }
  ctx->proj_last_n = 0;
  const int n = ctx->proj_count;
  if (n == 0) return TL_OK;
  /* V = [X, the differences from the oldest]; g_j = v_j . b */
  int vslot[kMaxVec];
  vslot[0] = ctx->proj_xslot;
  for (int j = 1; j < n; ++j) vslot[j] = ctx->proj_order[j - 1];
  VecList V;
  PairList L;
  for (int j = 0; j < n; ++j) {
    V.v[j] = L.a[j] = slot_ptr(ctx, vslot[j]);
    L.p[j] = b;
  }
  L.a[n] = L.p[n] = b;
  double g[kMaxVec];
  int rc = dots(ctx, x, y, hd, L, n + 1, g);
  if (rc != TL_OK) return rc;
  *bb = g[n];
  double G[kMaxVec * kMaxVec];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      G[i * n + j] = ctx->proj_gram[vslot[i]][vslot[j]];
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
  ctx->proj_last_n = n;
  for (int i = 0; i < n; ++i) {
    ctx->proj_last_slot[i] = vslot[i];
    ctx->proj_last_coef[i] = c.c[i];
  }
  *basis = kept;
  return TL_OK;
}

int tl_internal_project_recombine(tl_context* ctx, int x, int y, int hd, double* u) {
  const int n = ctx->proj_last_n;
  TL_REQUIRE(n > 0, "tl_solve: no projected guess to restore");
  VecList V;
  CoefList c;
  for (int i = 0; i < kMaxVec; ++i) c.c[i] = 0.0;
  for (int i = 0; i < n; ++i) {
    V.v[i] = slot_ptr(ctx, ctx->proj_last_slot[i]);
    c.c[i] = ctx->proj_last_coef[i];
  }
  proj_combine_kernel<<<4 * ctx->num_sms, 256, 0, ctx->stream>>>(x, y, hd, V, c, n, u);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

int tl_internal_hash64(tl_context* ctx, const double* a, const double* b, const double* c,
                       size_t n, unsigned long long salt_a, unsigned long long* out_a,
                       unsigned long long* out_bc) {
  if (!ctx->d_hash64) TL_CUDA(cudaMalloc(&ctx->d_hash64, 2 * sizeof(unsigned long long)));
  TL_CUDA(cudaMemsetAsync(ctx->d_hash64, 0, 2 * sizeof(unsigned long long), ctx->stream));
  hash64_kernel<<<8 * ctx->num_sms, kDotThreads, 0, ctx->stream>>>(a, b, c, n, ctx->d_hash64);
  TL_CHECK_LAUNCH(ctx);
  unsigned long long h[2] = {0, 0};
  TL_CUDA(cudaMemcpyAsync(h, ctx->d_hash64, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  auto fin = [](unsigned long long v, unsigned long long salt) {
    v ^= salt;
    v *= 0x94D049BB133111EBull;
    v ^= v >> 31;
    return v;
  };
  if (out_a) *out_a = fin(h[0], salt_a);
  if (out_bc) *out_bc = fin(h[1], 0);
  return TL_OK;
}

int tl_internal_project_push(tl_context* ctx, int x, int y, int hd, const double* b,
                             const double* u, const double* r, const double* kx,
                             const double* ky, const double* diag) {
  if (ctx->proj_slots < 1 || ctx->proj_x != x || ctx->proj_y != y || ctx->proj_hd != hd)
    return TL_OK;
  const size_t len = (size_t)x * (size_t)y;
  auto (&G)[TL_PROJ_MAX][TL_PROJ_MAX] = ctx->proj_gram;
  if (ctx->proj_count == 0 || ctx->proj_slots == 1) {
    /* u becomes X: u . A u = u . b - u . r */
    const int xs = ctx->proj_count == 0 ? 0 : ctx->proj_xslot;
    PairList L;
    L.a[0] = L.a[1] = u;
    L.p[0] = b;
    L.p[1] = r;
    double d[2];
    int rc = dots(ctx, x, y, hd, L, 2, d);
    if (rc != TL_OK) return rc;
    G[xs][xs] = d[0] - d[1];
    TL_CUDA(cudaMemcpyAsync(slot_ptr(ctx, xs), u, len * sizeof(double),
                            cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->proj_xslot = xs;
    ctx->proj_count = 1;
    return TL_OK;
  }
  /* the new difference d = u - X goes to a free slot, else to the oldest
   * difference's (dropped) */
  const int xs = ctx->proj_xslot;
  const int nd = ctx->proj_count - 1;
  const bool full = ctx->proj_count == ctx->proj_slots;
  int ds = -1;
  if (full) {
    ds = ctx->proj_order[0];
  } else {
    for (int c = 0; c < ctx->proj_slots && ds < 0; ++c) {
      bool used = c == xs;
      for (int j = 0; j < nd; ++j) used = used || ctx->proj_order[j] == c;
      if (!used) ds = c;
    }
  }
  const int first = full ? 1 : 0;
  const int ne = nd - first;
  int eslot[kMaxVec];
  VecList E;
  for (int k = 0; k < ne; ++k) {
    eslot[k] = ctx->proj_order[first + k];
    E.v[k] = slot_ptr(ctx, eslot[k]);
  }
  proj_push_kernel<<<grid_dots(ctx), kDotThreads, 0, ctx->stream>>>(
      x, y, hd, u, slot_ptr(ctx, xs), kx, ky, diag, E, ne, slot_ptr(ctx, ds), ctx->d_proj_part);
  TL_CHECK_LAUNCH(ctx);
  double d[kMaxVec];
  int rc = sum_partials(ctx, 2 + ne, d);
  if (rc != TL_OK) return rc;
  const double dd = d[0], xd = d[1];
  /* the new X = u = X + d: its row is X's plus d's */
  for (int k = 0; k < ne; ++k) {
    const double ue = G[xs][eslot[k]] + d[2 + k];
    G[xs][eslot[k]] = G[eslot[k]][xs] = ue;
    G[ds][eslot[k]] = G[eslot[k]][ds] = d[2 + k];
  }
  G[xs][xs] = G[xs][xs] + 2.0 * xd + dd;
  G[xs][ds] = G[ds][xs] = xd + dd;
  G[ds][ds] = dd;
  TL_CUDA(cudaMemcpyAsync(slot_ptr(ctx, xs), u, len * sizeof(double), cudaMemcpyDeviceToDevice,
                          ctx->stream));
  for (int k = 0; k < ne; ++k) ctx->proj_order[k] = eslot[k];
  ctx->proj_order[ne] = ds;
  ctx->proj_count = ne + 2;
  return TL_OK;
}

extern "C" int tl_projection_reset(tl_context* ctx) {
  TL_REQUIRE(ctx, "tl_projection_reset: null context");
  ctx->proj_count = 0;
  ctx->proj_hash = 0;
  ctx->proj_x = ctx->proj_y = ctx->proj_hd = 0;
  return TL_OK;
}
