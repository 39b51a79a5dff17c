/*
 * tl_coarse.cu -- the coarse level of the two-level learned PCG
 * (TL_METHOD_MIXED_LEARNED_COARSE): M^-1 = M_learned^-1 + P (P^T A P)^-1 P^T,
 * P piecewise constant on blk x blk aggregates of the packed [H][W] field.
 *
 * The learned stencil acts within 8 cells, so the lowest modes of a large
 * grid (one smooth error spread over thousands of cells) take the inner PCG
 * most of its steps; the coarse correction removes them. Aggregates are
 * 32, 64 or 128 cells square, the smallest size that keeps the coarse grid
 * at 4096 unknowns or fewer and divides H and W, so that they line up with
 * the 128 x 64 tiles of the learned PCG kernel: a tile's epilogue sums its
 * aggregates' residuals (the restriction) without another pass over memory,
 * and one dense product with the inverse Ac^-1 gives the coarse correction
 * every step. The product reads an FP16 copy of the inverse (32 MB at 4096
 * unknowns), scaled by a power of two so that its largest entry lies in
 * [2^14, 2^15): the rounding moves an entry by at most 2^-11 of itself or
 * 2^-39 of the largest entry, whichever is larger (the second bound holds
 * for the tiny entries far from the diagonal, FP16 subnormals once scaled).
 *
 * Ac = P^T A P needs no product with A. For A = I + L (L the weighted graph
 * Laplacian of the couplings, zero flux at the field's edges) the diagonal of
 * aggregate I is blk^2 plus every coupling across I's boundary (couplings
 * inside I cancel), and the entry of neighbouring aggregates I, J is minus
 * the sum of the couplings between them: a 5-point matrix on the coarse grid
 * (oracle/coarse_oracle.py restates it in float64). Its inverse is built once
 * per operator: the bands are summed on the device in FP64, factored by a
 * banded Cholesky on the host (bandwidth ncx, about 8 M multiply-adds at
 * 4096 unknowns), and each column of the inverse is two band solves on the
 * device, one thread per column. TeaLeaf's operator does not change between
 * timesteps (density and dt are fixed), so the inverse is kept in the
 * context and rebuilt only when H, W or the couplings change (a 64-bit
 * content hash of the couplings decides).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "tl_internal.cuh"

namespace {

constexpr int kMaxCoarse = 4096;   /* coarse unknowns at most */
constexpr int kTileH = 128;        /* the learned PCG kernel's tile */
constexpr int kTileW = 64;
constexpr int kRestrictSlots = 8;  /* restriction partials per tile */

/* Order-independent 64-bit hash of the couplings (wrapping sum of mixed
 * words, so every launch gives the same value). */
__global__ void coupling_hash_kernel(const float* __restrict__ kx, const float* __restrict__ ky,
                                     size_t n, unsigned long long* out) {
  __shared__ unsigned long long s[32];
  unsigned long long h = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long v = ((unsigned long long)__float_as_uint(kx[i]) << 32) |
                           (unsigned long long)__float_as_uint(ky[i]);
    v ^= (unsigned long long)i * 0x9E3779B97F4A7C15ull;
    v ^= v >> 31;
    v *= 0xBF58476D1CE4E5B9ull;
    v ^= v >> 29;
    h += v;
  }
  for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = h;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    atomicAdd(out, t);
  }
}

/* The bands of Ac, one thread per aggregate I = Jc * ncx + Ic, summed in
 * FP64 in the order of coarse_oracle.coarse_operator: diagonal = blk^2 +
 * west + east + south + north couplings; west[I] = -(couplings to I - 1),
 * south[I] = -(couplings to I - ncx). kx[y][x] couples cells x-1 and x of
 * row y, ky[y][x] rows y-1 and y of column x. */
__global__ void coarse_bands_kernel(int W, int sh, int ncx, int ncy,
                                    const float* __restrict__ kx, const float* __restrict__ ky,
                                    double* diag, double* west, double* south) {
  const int nc = ncx * ncy;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nc) return;
  const int b = 1 << sh;
  const int Ic = I % ncx, Jc = I / ncx;
  const size_t x0 = (size_t)Ic * b, y0 = (size_t)Jc * b;
  double cw = 0.0, ce = 0.0, cs = 0.0, cn = 0.0;
  if (Ic > 0)
    for (int r = 0; r < b; ++r) cw += (double)kx[(y0 + r) * W + x0];
  if (Ic < ncx - 1)
    for (int r = 0; r < b; ++r) ce += (double)kx[(y0 + r) * W + x0 + b];
  if (Jc > 0)
    for (int c = 0; c < b; ++c) cs += (double)ky[y0 * W + x0 + c];
  if (Jc < ncy - 1)
    for (int c = 0; c < b; ++c) cn += (double)ky[(y0 + b) * W + x0 + c];
  diag[I] = (double)b * (double)b + cw + ce + cs + cn;
  west[I] = -cw;
  south[I] = -cs;
}

/* Column j of Ac^-1 = L^-T L^-1 e_j by two band solves (one thread per
 * column; the band of L, row i holding L[i][i-bw .. i], is read by all
 * threads of a warp at once). work holds the column (row-major n x n, so
 * neighbouring threads touch neighbouring words); ainv receives it in FP32. */
__global__ void coarse_inverse_kernel(int n, int bw, const double* __restrict__ band,
                                      double* work, float* ainv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int ld = bw + 1;
  for (int i = 0; i < n; ++i) {  /* L y = e_j */
    double s = (i == j) ? 1.0 : 0.0;
    const int m0 = i - bw > 0 ? i - bw : 0;
    const double* li = band + (size_t)i * ld + bw - i;  /* li[m] = L[i][m] */
    for (int m = m0; m < i; ++m) s -= li[m] * work[(size_t)m * n + j];
    work[(size_t)i * n + j] = s / li[i];
  }
  for (int i = n - 1; i >= 0; --i) {  /* L^T x = y */
    double s = work[(size_t)i * n + j];
    const int m1 = i + bw < n - 1 ? i + bw : n - 1;
    for (int m = i + 1; m <= m1; ++m) s -= band[(size_t)m * ld + bw - m + i] * work[(size_t)m * n + j];
    const double x = s / band[(size_t)i * ld + bw];
    work[(size_t)i * n + j] = x;
    ainv[(size_t)i * n + j] = (float)x;
  }
}

/* Largest |entry| of the inverse: non-negative floats order like their bit
 * patterns (a NaN orders above every finite value and is caught by the host). */
__global__ void coarse_absmax_kernel(const float* __restrict__ a, size_t n, unsigned* out) {
  unsigned m = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    m = max(m, __float_as_uint(fabsf(a[i])));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

/* The FP16 copy: a * 2^e (exact in FP32) rounded to nearest. */
__global__ void coarse_half_kernel(const float* __restrict__ a, size_t n, float scale,
                                   __half* out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2half_rn(a[i] * scale);
}

/* Banded Cholesky of the 5-point coarse matrix (bandwidth bw = ncx) into
 * band[i * (bw + 1) + (k - i + bw)] = L[i][k]. Returns false when a pivot is
 * not positive (Ac is SPD, so only a broken operator gets there). */
bool band_cholesky(int n, int bw, const std::vector<double>& diag, const std::vector<double>& west,
                   const std::vector<double>& south, std::vector<double>& band) {
  const int ld = bw + 1;
  band.assign((size_t)n * ld, 0.0);
  auto A = [&](int i, int k) -> double {  /* k <= i */
    if (k == i) return diag[i];
    if (k == i - 1 && i % bw != 0) return west[i];
    if (k == i - bw) return south[i];
    return 0.0;
  };
  auto L = [&](int i, int k) -> double& { return band[(size_t)i * ld + (k - i + bw)]; };
  for (int i = 0; i < n; ++i) {
    const int k0 = i - bw > 0 ? i - bw : 0;
    for (int k = k0; k <= i; ++k) {
      double s = A(i, k);
      for (int m = k0; m < k; ++m) s -= L(i, m) * L(k, m);
      if (k == i) {
        if (!(s > 0.0)) return false;
        L(i, i) = sqrt(s);
      } else {
        L(i, k) = s / L(k, k);
      }
    }
  }
  return true;
}

int blk_shift_for(int H, int W) {
  for (int sh = 5; sh <= 7; ++sh) {
    const int b = 1 << sh;
    if (H % b != 0 || W % b != 0) continue;
    if ((size_t)(H >> sh) * (size_t)(W >> sh) <= (size_t)kMaxCoarse) return sh;
  }
  return -1;
}

template <class T>
int ensure(T** ptr, size_t* cap, size_t n, cudaStream_t stream) {
  if (n <= *cap) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(stream));
  cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  TL_CUDA(cudaMalloc(ptr, n * sizeof(T)));
  *cap = n;
  return TL_OK;
}

}  // namespace

int tl_internal_coarse_prepare(tl_context* ctx, int H, int W, const float* kx, const float* ky,
                               tl_coarse_level* out, const unsigned long long* known_hash) {
  const int sh = blk_shift_for(H, W);
  if (sh < 0) {
    return tl_set_error(TL_ERR_ARG,
                        "the coarse level needs H and W divisible by an aggregate size of 32, "
                        "64 or 128 that leaves at most 4096 coarse unknowns; got " +
                            std::to_string(H) + " x " + std::to_string(W));
  }
  const int ncx = W >> sh, ncy = H >> sh, nc = ncx * ncy;
  const size_t tiles = (size_t)((W + kTileW - 1) / kTileW) * (size_t)((H + kTileH - 1) / kTileH);
  int rc = ensure(&ctx->d_coarse_vec, &ctx->coarse_vec_cap, tiles * kRestrictSlots + (size_t)nc,
                  ctx->stream);
  if (rc != TL_OK) return rc;
  if (!ctx->d_hash) TL_CUDA(cudaMalloc(&ctx->d_hash, sizeof(unsigned long long)));
  unsigned long long hash = 0;
  if (known_hash) {
    hash = *known_hash;
  } else {
    TL_CUDA(cudaMemsetAsync(ctx->d_hash, 0, sizeof(unsigned long long), ctx->stream));
    const size_t n = (size_t)H * W;
    coupling_hash_kernel<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(kx, ky, n, ctx->d_hash);
    TL_CHECK_LAUNCH(ctx);
    TL_CUDA(cudaMemcpyAsync(&hash, ctx->d_hash, sizeof(hash), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  const bool cached = ctx->d_ainv && ctx->coarse_H == H && ctx->coarse_W == W &&
                      ctx->coarse_blk == (1 << sh) && ctx->coarse_hash == hash;
  if (!cached) {
    ctx->coarse_H = 0;
    const int bw = ncx;
    const size_t nn = (size_t)nc * nc, nband = (size_t)nc * (bw + 1);
    rc = ensure(&ctx->d_ainv, &ctx->ainv_cap, nn, ctx->stream);
    if (rc != TL_OK) return rc;
    rc = ensure(&ctx->d_coarse_work, &ctx->coarse_work_cap, nn + nband + 3 * (size_t)nc,
                ctx->stream);
    if (rc != TL_OK) return rc;
    double* work = ctx->d_coarse_work;
    double* band_d = work + nn;
    double* bands = band_d + nband;  /* diag, west, south */
    coarse_bands_kernel<<<(nc + 127) / 128, 128, 0, ctx->stream>>>(W, sh, ncx, ncy, kx, ky,
                                                                  bands, bands + nc,
                                                                  bands + 2 * nc);
    TL_CHECK_LAUNCH(ctx);
    std::vector<double> h(3 * (size_t)nc);
    TL_CUDA(cudaMemcpyAsync(h.data(), bands, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> diag(h.begin(), h.begin() + nc), west(h.begin() + nc,
                                                            h.begin() + 2 * nc),
        south(h.begin() + 2 * nc, h.end());
    std::vector<double> band;
    if (!band_cholesky(nc, bw, diag, west, south, band)) {
      return tl_set_error(TL_ERR_NUMERIC, "coarse operator is not positive definite");
    }
    TL_CUDA(cudaMemcpyAsync(band_d, band.data(), nband * sizeof(double),
                            cudaMemcpyHostToDevice, ctx->stream));
    coarse_inverse_kernel<<<(nc + 31) / 32, 32, 0, ctx->stream>>>(nc, bw, band_d, work,
                                                                  ctx->d_ainv);
    TL_CHECK_LAUNCH(ctx);
    /* the FP16 copy, scaled by 2^e: the largest entry m 2^k (m in [0.5, 1))
     * becomes m 2^15 */
    unsigned* d_max = reinterpret_cast<unsigned*>(ctx->d_hash);
    TL_CUDA(cudaMemsetAsync(d_max, 0, sizeof(unsigned), ctx->stream));
    coarse_absmax_kernel<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(ctx->d_ainv, nn, d_max);
    TL_CHECK_LAUNCH(ctx);
    unsigned max_bits = 0;
    TL_CUDA(cudaMemcpyAsync(&max_bits, d_max, sizeof(max_bits), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
    float amax;
    memcpy(&amax, &max_bits, sizeof(amax));
    int k = 0;
    if (isfinite(amax) && amax > 0.0f) frexpf(amax, &k);
    const int e = 15 - k;
    if (!(isfinite(amax) && amax > 0.0f) || e > 126 || e < -126) {
      return tl_set_error(TL_ERR_NUMERIC, "coarse inverse out of the FP16 copy's range");
    }
    rc = ensure(&ctx->d_ainv16, &ctx->ainv16_cap, nn, ctx->stream);
    if (rc != TL_OK) return rc;
    coarse_half_kernel<<<4 * ctx->num_sms, 256, 0, ctx->stream>>>(ctx->d_ainv, nn,
                                                                 ldexpf(1.0f, e),
                                                                 ctx->d_ainv16);
    TL_CHECK_LAUNCH(ctx);
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->coarse_exp = e;
    ctx->coarse_H = H;
    ctx->coarse_W = W;
    ctx->coarse_blk = 1 << sh;
    ctx->coarse_hash = hash;
  }
  out->blk_shift = sh;
  out->ncx = ncx;
  out->ncy = ncy;
  out->nc = nc;
  out->ainv = ctx->d_ainv;
  out->ainv16 = ctx->d_ainv16;
  out->exp16 = ctx->coarse_exp;
  out->rc_part = ctx->d_coarse_vec;
  out->ec = ctx->d_coarse_vec + tiles * kRestrictSlots;
  return TL_OK;
}

extern "C" int tl_coarse_inverse(tl_context* ctx, int H, int W, const float* kx, const float* ky,
                                 int* blk, int* nc, float* ainv_host, size_t capacity) {
  TL_REQUIRE(ctx && kx && ky && blk && nc, "tl_coarse_inverse: null argument");
  TL_REQUIRE(H >= 1 && W >= 1 && (size_t)H * W < (1ull << 31), "tl_coarse_inverse: bad shape");
  tl_coarse_level lv;
  int rc = tl_internal_coarse_prepare(ctx, H, W, kx, ky, &lv);
  if (rc != TL_OK) return rc;
  *blk = 1 << lv.blk_shift;
  *nc = lv.nc;
  if (ainv_host) {
    const size_t nn = (size_t)lv.nc * lv.nc;
    TL_REQUIRE(capacity >= nn, "tl_coarse_inverse: host array too small");
    TL_CUDA(cudaMemcpyAsync(ainv_host, lv.ainv, nn * sizeof(float), cudaMemcpyDeviceToHost,
                            ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return TL_OK;
}

extern "C" int tl_coarse_inverse_f16(tl_context* ctx, int H, int W, const float* kx,
                                     const float* ky, uint16_t* half_host, size_t capacity,
                                     int* exp2) {
  TL_REQUIRE(ctx && kx && ky && exp2, "tl_coarse_inverse_f16: null argument");
  TL_REQUIRE(H >= 1 && W >= 1 && (size_t)H * W < (1ull << 31),
             "tl_coarse_inverse_f16: bad shape");
  tl_coarse_level lv;
  int rc = tl_internal_coarse_prepare(ctx, H, W, kx, ky, &lv);
  if (rc != TL_OK) return rc;
  *exp2 = lv.exp16;
  if (half_host) {
    const size_t nn = (size_t)lv.nc * lv.nc;
    TL_REQUIRE(capacity >= nn, "tl_coarse_inverse_f16: host array too small");
    TL_CUDA(cudaMemcpyAsync(half_host, lv.ainv16, nn * sizeof(uint16_t),
                            cudaMemcpyDeviceToHost, ctx->stream));
    TL_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return TL_OK;
}
