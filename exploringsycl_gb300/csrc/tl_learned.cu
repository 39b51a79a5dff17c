/*
 * tl_learned.cu -- the learned linear preconditioner and its training
 * kernels.
 *
 * Operator. z = M^-1 r = D^-1 r + S C^T C S r, where S = diag(D^-1/2) scales each
 * cell by its operator diagonal D = 1 + kx[i+1] + kx[i] + ky[i+x] + ky[i]
 * (the local conditioning on kx/ky, independent of r so that M^-1 stays
 * linear), and C = L4 L3 L2 L1 is a stack of four 3x3 convolutions without
 * bias or activation: L1 maps 1 channel to 16, L2..L4 map 16 to 16. C^T
 * applies the adjoint convolutions in reverse order (each adjoint is the
 * correlation with the kernel flipped and its channels swapped). Zero
 * padding at the domain edge makes every adjoint exact, so S C^T C S is
 * symmetric positive semi-definite by construction, and the Jacobi term
 * D^-1 makes M^-1 positive definite with its eigenvalues bounded below by
 * those of D^-1 (a learned C can otherwise leave modes that are absent from
 * the training residuals in its null space).
 *
 * Arithmetic. Weights and activations are BF16; every convolution
 * accumulates in FP32. The 16 -> 16 convolutions run on the tensor cores
 * (mma.sync m16n8k16 BF16 -> FP32): a warp owns 64 pixels of one row and
 * all 16 output channels, the input tile and its one-pixel halo are staged
 * in shared memory (48-byte pixel stride, conflict-free ldmatrix), and the 9
 * taps x 2 output-channel halves are 18 MMAs per 16 pixels. The 1-channel
 * layers (1 -> 16 and 16 -> 1) run on the FP32 cores.
 *
 * Activation layout: [batch][H][W][C], C = 16 (32 bytes per pixel) or 1.
 * H must be a multiple of 4 and W of 64.
 *
 * Training (loss and gradients): for residual crops r with coefficients
 * kx, ky, L = sum_b sum_valid (A z - r)^2 / sum_b sum_valid r^2 with
 * z = M^-1 r (one normaliser per batch, so crops with a tiny residual cannot
 * dominate),
 * evaluated on the crop interior whose distance to the crop edge exceeds the
 * receptive field (so the zero padding outside the crop cannot leak in).
 * dL/dz = A^T (2 (A z - r) mask / sum r^2) with A symmetric; the gradient
 * flows back through S, the adjoint layers and the forward layers; weight
 * gradients are FP32 sums over pixels computed on the FP32 cores.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "tl_internal.cuh"

namespace {

constexpr int kCh = 16;       /* hidden channels */
constexpr int kLayers = 4;
constexpr int kTH = 4;        /* conv tile rows per block (one warp per row) */
constexpr int kTW = 64;       /* conv tile columns per block */
constexpr int kPixStride = 24;  /* bf16 per staged pixel: 16 channels + 8 pad */


__device__ __forceinline__ float bf2f(__nv_bfloat16 v) { return __bfloat162float(v); }

/* ------------------------------------------------ tensor-core 16 -> 16 */

/* out[b][y][x][co] = sum_{dy,dx,ci} w[tap][co][ci] * in[b][y+dy-1][x+dx-1][ci]
 * with zero padding; w is stored [tap][co][ci] (ci contiguous). */
template <bool kOutF32>
__global__ void __launch_bounds__(128) conv16_tc_kernel(const __nv_bfloat16* __restrict__ in,
                                                        const __nv_bfloat16* __restrict__ w,
                                                        void* out, int H, int W) {
  __shared__ __align__(16) __nv_bfloat16 s_in[(kTH + 2) * (kTW + 2) * kPixStride];
  __shared__ __align__(16) __nv_bfloat16 s_w[9 * kCh * kCh];
  const int b = blockIdx.z;
  const int y0 = blockIdx.y * kTH;
  const int x0 = blockIdx.x * kTW;
  const int tid = threadIdx.x;
  const size_t img = (size_t)b * H * W;

  /* weights: 9*16*16 bf16 = 288 x 16-byte chunks */
  for (int c = tid; c < 9 * kCh * kCh / 8; c += blockDim.x) {
    reinterpret_cast<uint4*>(s_w)[c] = reinterpret_cast<const uint4*>(w)[c];
  }
  /* input tile + halo: two 16-byte halves per pixel */
  const int npix = (kTH + 2) * (kTW + 2);
  for (int c = tid; c < npix * 2; c += blockDim.x) {
    const int pix = c >> 1, half = c & 1;
    const int ty = pix / (kTW + 2), tx = pix - ty * (kTW + 2);
    const int gy = y0 + ty - 1, gx = x0 + tx - 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      v = reinterpret_cast<const uint4*>(in + (img + (size_t)gy * W + gx) * kCh)[half];
    }
    *reinterpret_cast<uint4*>(s_in + pix * kPixStride + half * 8) = v;
  }
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  float acc[4][2][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;

#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3, dx = tap % 3;
    uint32_t bfrag[2][2];
#pragma unroll
    for (int n = 0; n < 2; ++n) {
      const __nv_bfloat16* wb = s_w + (tap * kCh + n * 8 + g) * kCh + 2 * t;
      bfrag[n][0] = *reinterpret_cast<const uint32_t*>(wb);
      bfrag[n][1] = *reinterpret_cast<const uint32_t*>(wb + 8);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      /* ldmatrix x4: lane L addresses pixel (L % 16) of this m-tile,
       * channels 0-7 (L < 16) or 8-15 (L >= 16). */
      const int px = m * 16 + (lane & 15) + dx;
      const __nv_bfloat16* src =
          s_in + ((warp + dy) * (kTW + 2) + px) * kPixStride + (lane >> 4) * 8;
      const uint32_t saddr = (uint32_t)__cvta_generic_to_shared(src);
      uint32_t a0, a1, a2, a3;
      asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                   : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3)
                   : "r"(saddr));
#pragma unroll
      for (int n = 0; n < 2; ++n) {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
            "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
            : "+f"(acc[m][n][0]), "+f"(acc[m][n][1]), "+f"(acc[m][n][2]), "+f"(acc[m][n][3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(bfrag[n][0]), "r"(bfrag[n][1]));
      }
    }
  }

  /* accumulator (m, n): rows g and g+8 of the m-tile, columns 2t, 2t+1 of
   * the n-half. */
  const int gy = y0 + warp;
  if (gy >= H) return;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
#pragma unroll
    for (int hr = 0; hr < 2; ++hr) {
      const int gx = x0 + m * 16 + g + hr * 8;
      if (gx >= W) continue;
      const size_t o = (img + (size_t)gy * W + gx) * kCh;
#pragma unroll
      for (int n = 0; n < 2; ++n) {
        const int co = n * 8 + 2 * t;
        const float v0 = acc[m][n][hr * 2 + 0], v1 = acc[m][n][hr * 2 + 1];
        if (kOutF32) {
          float* of = reinterpret_cast<float*>(out) + o + co;
          of[0] = v0;
          of[1] = v1;
        } else {
          *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(out) + o + co) =
              __floats2bfloat162_rn(v0, v1);
        }
      }
    }
  }
}

/* ---------------------------------------------- FP32-core 1-channel layers */

/* 1 -> 16: out[..][co] = sum_tap w[tap][co] * in[..+tap]; w fp32 [tap][co]. */
__global__ void conv1to16_kernel(const __nv_bfloat16* __restrict__ in,
                                 const float* __restrict__ w, __nv_bfloat16* __restrict__ out,
                                 int H, int W, int B) {
  __shared__ float s_w[9 * kCh];
  for (int i = threadIdx.x; i < 9 * kCh; i += blockDim.x) s_w[i] = w[i];
  __syncthreads();
  const size_t total = (size_t)B * H * W;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(p % W);
    const int yy = (int)((p / W) % H);
    const size_t img = p - ((size_t)yy * W + xx);
    float v[9];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int sy = yy + tap / 3 - 1, sx = xx + tap % 3 - 1;
      v[tap] = (sy >= 0 && sy < H && sx >= 0 && sx < W) ? bf2f(in[img + (size_t)sy * W + sx])
                                                         : 0.0f;
    }
    __align__(16) __nv_bfloat162 o[8];
#pragma unroll
    for (int c = 0; c < kCh; c += 2) {
      float a = 0.0f, bsum = 0.0f;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        a += s_w[tap * kCh + c] * v[tap];
        bsum += s_w[tap * kCh + c + 1] * v[tap];
      }
      o[c / 2] = __floats2bfloat162_rn(a, bsum);
    }
    uint4* dst = reinterpret_cast<uint4*>(out + p * kCh);
    dst[0] = *reinterpret_cast<uint4*>(&o[0]);
    dst[1] = *reinterpret_cast<uint4*>(&o[4]);
  }
}

/* 16 -> 1: out = sum_{tap,ci} w[tap][ci] * in[..+tap][ci]; fp32 output. */
__global__ void conv16to1_kernel(const __nv_bfloat16* __restrict__ in,
                                 const float* __restrict__ w, float* __restrict__ out, int H,
                                 int W, int B) {
  __shared__ float s_w[9 * kCh];
  for (int i = threadIdx.x; i < 9 * kCh; i += blockDim.x) s_w[i] = w[i];
  __syncthreads();
  const size_t total = (size_t)B * H * W;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(p % W);
    const int yy = (int)((p / W) % H);
    const size_t img = p - ((size_t)yy * W + xx);
    float acc = 0.0f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int sy = yy + tap / 3 - 1, sx = xx + tap % 3 - 1;
      if (sy < 0 || sy >= H || sx < 0 || sx >= W) continue;
      const uint4* src = reinterpret_cast<const uint4*>(in + (img + (size_t)sy * W + sx) * kCh);
      const uint4 h0 = src[0], h1 = src[1];
      const __nv_bfloat162* c0 = reinterpret_cast<const __nv_bfloat162*>(&h0);
      const __nv_bfloat162* c1 = reinterpret_cast<const __nv_bfloat162*>(&h1);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f0 = __bfloat1622float2(c0[k]);
        const float2 f1 = __bfloat1622float2(c1[k]);
        acc += s_w[tap * kCh + 2 * k] * f0.x + s_w[tap * kCh + 2 * k + 1] * f0.y;
        acc += s_w[tap * kCh + 8 + 2 * k] * f1.x + s_w[tap * kCh + 9 + 2 * k] * f1.y;
      }
    }
    out[p] = acc;
  }
}

/* ------------------------------------------------------ weight gradients */

/* dW[tap][ci][co] += sum_p x[p + tap][ci] * g[p][co] for 16 -> 16, FP32.
 * Each block accumulates over many pixel rows and writes one partial set;
 * wgrad_sum_kernel adds the partials in a fixed order. Thread j owns 9
 * (tap, ci, co) triples: tap-major over 256 threads x 9 = 2304. */
__global__ void __launch_bounds__(256) wgrad16_kernel(const __nv_bfloat16* __restrict__ x,
                                                      const __nv_bfloat16* __restrict__ gy,
                                                      float* __restrict__ partial, int H,
                                                      int W, int B) {
  __shared__ float s_x[3][(kTW + 2) * kCh];
  __shared__ float s_g[kTW * kCh];
  const int ci = (threadIdx.x >> 4) & 15, co = threadIdx.x & 15;
  float acc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = 0.0f;
  const int tiles_x = W / kTW;
  const long nrows = (long)B * H * tiles_x;
  for (long rt = blockIdx.x; rt < nrows; rt += gridDim.x) {
    const int tx = (int)(rt % tiles_x);
    const long by = rt / tiles_x;
    const int yy = (int)(by % H);
    const size_t img = (size_t)(by / H) * H * W;
    const int x0 = tx * kTW;
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * (kTW + 2) * kCh; i += blockDim.x) {
      const int r = i / ((kTW + 2) * kCh), rem = i - r * (kTW + 2) * kCh;
      const int px = rem / kCh, c = rem - px * kCh;
      const int sy = yy + r - 1, sx = x0 + px - 1;
      s_x[r][rem] = (sy >= 0 && sy < H && sx >= 0 && sx < W)
                        ? bf2f(x[(img + (size_t)sy * W + sx) * kCh + c])
                        : 0.0f;
    }
    for (int i = threadIdx.x; i < kTW * kCh; i += blockDim.x) {
      s_g[i] = bf2f(gy[(img + (size_t)yy * W + x0) * kCh + i]);
    }
    __syncthreads();
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
      float a = acc[tap];
      for (int px = 0; px < kTW; ++px) a += s_x[dy][(px + dx) * kCh + ci] * s_g[px * kCh + co];
      acc[tap] = a;
    }
  }
#pragma unroll
  for (int tap = 0; tap < 9; ++tap)
    partial[(size_t)blockIdx.x * 9 * kCh * kCh + (tap * kCh + ci) * kCh + co] = acc[tap];
}

/* dW[tap][co] += sum_p x[p + tap] * g[p][co] for 1 -> 16 (x: 1 channel). */
__global__ void __launch_bounds__(256) wgrad1to16_kernel(const __nv_bfloat16* __restrict__ x,
                                                         const __nv_bfloat16* __restrict__ gy,
                                                         float* __restrict__ partial, int H,
                                                         int W, int B) {
  const int tap = threadIdx.x >> 4, co = threadIdx.x & 15;  /* 144 active threads */
  float acc = 0.0f;
  const size_t total = (size_t)B * H * W;
  if (tap < 9) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    for (size_t p = blockIdx.x; p < total; p += gridDim.x) {
      const int xx = (int)(p % W);
      const int yy = (int)((p / W) % H);
      const size_t img = p - ((size_t)yy * W + xx);
      const int sy = yy + dy, sx = xx + dx;
      if (sy < 0 || sy >= H || sx < 0 || sx >= W) continue;
      acc += bf2f(x[img + (size_t)sy * W + sx]) * bf2f(gy[p * kCh + co]);
    }
    partial[(size_t)blockIdx.x * 9 * kCh + tap * kCh + co] = acc;
  }
}

/* dW[tap][ci] += sum_p x[p + tap][ci] * g[p] for 16 -> 1 (g: 1 channel, fp32). */
__global__ void __launch_bounds__(256) wgrad16to1_kernel(const __nv_bfloat16* __restrict__ x,
                                                         const float* __restrict__ gy,
                                                         float* __restrict__ partial, int H,
                                                         int W, int B) {
  const int tap = threadIdx.x >> 4, ci = threadIdx.x & 15;
  float acc = 0.0f;
  const size_t total = (size_t)B * H * W;
  if (tap < 9) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    for (size_t p = blockIdx.x; p < total; p += gridDim.x) {
      const int xx = (int)(p % W);
      const int yy = (int)((p / W) % H);
      const size_t img = p - ((size_t)yy * W + xx);
      const int sy = yy + dy, sx = xx + dx;
      if (sy < 0 || sy >= H || sx < 0 || sx >= W) continue;
      acc += bf2f(x[(img + (size_t)sy * W + sx) * kCh + ci]) * gy[p];
    }
    partial[(size_t)blockIdx.x * 9 * kCh + tap * kCh + ci] = acc;
  }
}

/* out[i] += sum_b partial[b][i], fixed order. */
__global__ void wgrad_sum_kernel(const float* __restrict__ partial, int nblocks, int n,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * n + i];
  out[i] += s;
}

/* ------------------------------------------------ scaling, operator, loss */

/* a0 = bf16(r * s) on [B][H][W] (1 channel). */
__global__ void scale_to_bf16_kernel(const float* __restrict__ r, const float* __restrict__ s,
                                     __nv_bfloat16* __restrict__ a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    a[i] = __float2bfloat16(r[i] * s[i]);
}

/* z = s * (b0 + s * r): the learned part plus the Jacobi term. */
__global__ void output_kernel(const float* __restrict__ b0, const float* __restrict__ r,
                              const float* __restrict__ s, float* __restrict__ z, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    z[i] = s[i] * (b0[i] + s[i] * r[i]);
}

/* z = b0 * s. */
__global__ void scale_f32_kernel(const float* __restrict__ b0, const float* __restrict__ s,
                                 float* __restrict__ z, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    z[i] = b0[i] * s[i];
}

/* q = A z - r on the crop (flux form with the crop's kx, ky; values outside
 * the crop count as 0 -- only the masked interior enters the loss), and the
 * per-sample sums of q^2 and r^2 over the valid region. kx[p] couples p and
 * its left neighbour, ky[p] p and the one below. */
__global__ void residual_loss_kernel(const float* __restrict__ z, const float* __restrict__ r,
                                     const float* __restrict__ kx, const float* __restrict__ ky,
                                     float* __restrict__ q, int H, int W, int B, int margin,
                                     double* __restrict__ sums) {
  const size_t total = (size_t)B * H * W;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(p % W);
    const int yy = (int)((p / W) % H);
    const int b = (int)(p / ((size_t)H * W));
    const bool valid = xx >= margin && xx < W - margin && yy >= margin && yy < H - margin;
    float qv = 0.0f;
    if (valid) {
      const float a = z[p];
      const float al = z[p - 1], ar = z[p + 1], ad = z[p - W], au = z[p + W];
      const float az = a + kx[p + 1] * (a - ar) + kx[p] * (a - al) + ky[p + W] * (a - au) +
                       ky[p] * (a - ad);
      qv = az - r[p];
      atomicAdd(&sums[2 * b], (double)(qv * qv));
      atomicAdd(&sums[2 * b + 1], (double)(r[p] * r[p]));
    }
    q[p] = qv;
  }
}

/* gz = A (2 q / (B * sum_r2[b])) -- q is zero outside the valid region. */
__global__ void loss_grad_kernel(const float* __restrict__ q, const float* __restrict__ kx,
                                 const float* __restrict__ ky, const double* __restrict__ sums,
                                 float* __restrict__ gz, int H, int W, int B) {
  const size_t total = (size_t)B * H * W;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(p % W);
    const int yy = (int)((p / W) % H);
    const int b = (int)(p / ((size_t)H * W));
    /* loss = sum_b num_b / sum_b den_b: one normaliser for the batch */
    double den = 0.0;
    for (int k = 0; k < B; ++k) den += sums[2 * k + 1];
    const float c = den > 0.0 ? (float)(2.0 / den) : 0.0f;
    (void)b;
    auto at = [&](int dy, int dx) -> float {
      const int sy = yy + dy, sx = xx + dx;
      if (sy < 0 || sy >= H || sx < 0 || sx >= W) return 0.0f;
      return q[p + (long)dy * W + dx];
    };
    const float a = q[p];
    /* A is symmetric: the same flux form applied to q */
    float v = a;
    if (xx + 1 < W) v += kx[p + 1] * (a - at(0, 1));
    if (xx > 0) v += kx[p] * (a - at(0, -1));
    if (yy + 1 < H) v += ky[p + W] * (a - at(1, 0));
    if (yy > 0) v += ky[p] * (a - at(-1, 0));
    gz[p] = c * v;
  }
}

/* ----------------------------------------------------------- weights */

/* bf16 working copies of the FP32 master weights: for each layer the
 * forward kernel [tap][co][ci] and the adjoint kernel (flipped taps,
 * channels swapped) in the layout its consumer reads. */
__global__ void make_weights_kernel(const float* __restrict__ master,
                                    __nv_bfloat16* __restrict__ fwd16,
                                    __nv_bfloat16* __restrict__ adj16, float* __restrict__ l1_fwd,
                                    float* __restrict__ l1_adj) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  /* master layout: layer 0 [tap][co] (144), layers 1..3 [tap][ci][co] (2304 each) */
  if (i < 9 * kCh) {
    const int tap = i / kCh, co = i % kCh;
    l1_fwd[tap * kCh + co] = master[i];
    /* adjoint of 1->16 is 16->1 with flipped tap: w'[tap][ci=co] */
    l1_adj[(8 - tap) * kCh + co] = master[i];
  }
  const int n16 = 9 * kCh * kCh;
  if (i < 3 * n16) {
    const int l = i / n16, rem = i % n16;
    const int tap = rem / (kCh * kCh), ci = (rem / kCh) % kCh, co = rem % kCh;
    const float v = master[9 * kCh + i];
    fwd16[l * n16 + (tap * kCh + co) * kCh + ci] = __float2bfloat16(v);
    /* adjoint: w'[8 - tap][co'=ci][ci'=co], stored [tap][co'][ci'] */
    adj16[l * n16 + ((8 - tap) * kCh + ci) * kCh + co] = __float2bfloat16(v);
  }
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

/* ----------------------------------------------- collapse to a stencil */

constexpr int kStencil = 17;            /* C^T C: 17 x 17 taps */
constexpr int kUmmaHalves = 17 * 2 * 256;  /* 34 B operands of 16 x 16 FP16 */
constexpr int kUmma32Halves = 17 * 512;    /* 17 B operands of 32 x 16 FP16 */

/* Composes the four layers into the 16-channel 9x9 kernel G of C (G(u)
 * multiplies the input at offset u), then K(d) = sum_u G(u).G(u + d), the
 * stencil of C^T C, and the tcgen05 B operands of its banded Toeplitz blocks
 * (tl_precond.cu), as FP16, K scaled by kscale = 2^-ceil(log2 max|K|).
 * umma (stand-alone application, N = 16) holds matrix (dy, kb) at halves
 * 256 (2 dy + kb), element (n, k) = K(dy, 16 kb + k - 8 - n) at
 * (k / 8) 128 + 8 n + k % 8 (K-major core matrices, 16 x 16). umma32 holds,
 * per dy, the 32 x 16 operand of one 16-column input window and the 32
 * output columns it reaches: element (n, k) = K(dy, k + 8 - n) at halves
 * 512 dy + (k / 8) 256 + 8 n + k % 8.
 * One block; runs whenever the weights change. */
__global__ void __launch_bounds__(256) collapse_kernel(const float* __restrict__ master,
                                                        float* __restrict__ k_out,
                                                        __half* __restrict__ umma,
                                                        __half* __restrict__ umma32,
                                                        float* __restrict__ kscale_out) {
  __shared__ float s_g[2][81 * kCh];
  __shared__ float s_k[kStencil * kStencil];
  __shared__ float s_max[8];
  const int tid = threadIdx.x;
  for (int i = tid; i < 81 * kCh; i += blockDim.x) {
    const int u = i / kCh, c = i % kCh;
    const int uy = u / 9 - 4, ux = u % 9 - 4;
    float v = 0.0f;
    if (uy >= -1 && uy <= 1 && ux >= -1 && ux <= 1) v = master[(3 * (uy + 1) + ux + 1) * kCh + c];
    s_g[0][i] = v;
  }
  __syncthreads();
  int cur = 0;
  for (int l = 0; l < 3; ++l) {
    const float* wl = master + 9 * kCh + l * 9 * kCh * kCh;  /* [tap][ci][co] */
    for (int i = tid; i < 81 * kCh; i += blockDim.x) {
      const int u = i / kCh, co = i % kCh;
      const int uy = u / 9 - 4, ux = u % 9 - 4;
      float acc = 0.0f;
      for (int tap = 0; tap < 9; ++tap) {
        const int vy = uy - (tap / 3 - 1), vx = ux - (tap % 3 - 1);
        if (vy < -4 || vy > 4 || vx < -4 || vx > 4) continue;
        const float* gv = &s_g[cur][((vy + 4) * 9 + vx + 4) * kCh];
        for (int ci = 0; ci < kCh; ++ci) acc += gv[ci] * wl[(tap * kCh + ci) * kCh + co];
      }
      s_g[cur ^ 1][i] = acc;
    }
    __syncthreads();
    cur ^= 1;
  }
  const float* gk = s_g[cur];
  float local_max = 0.0f;
  for (int d = tid; d < kStencil * kStencil; d += blockDim.x) {
    const int dy = d / kStencil - 8, dx = d % kStencil - 8;
    float acc = 0.0f;
    for (int uy = -4; uy <= 4; ++uy) {
      const int vy = uy + dy;
      if (vy < -4 || vy > 4) continue;
      for (int ux = -4; ux <= 4; ++ux) {
        const int vx = ux + dx;
        if (vx < -4 || vx > 4) continue;
        const float* a = &gk[((uy + 4) * 9 + ux + 4) * kCh];
        const float* b = &gk[((vy + 4) * 9 + vx + 4) * kCh];
        for (int c = 0; c < kCh; ++c) acc += a[c] * b[c];
      }
    }
    s_k[d] = acc;
    k_out[d] = acc;
    local_max = fmaxf(local_max, fabsf(acc));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local_max = fmaxf(local_max, __shfl_xor_sync(TL_FULL_MASK, local_max, o));
  if ((tid & 31) == 0) s_max[tid >> 5] = local_max;
  __syncthreads();
  float kmax = 0.0f;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) kmax = fmaxf(kmax, s_max[i]);
  const float kscale = kmax > 0.0f ? exp2f(-ceilf(log2f(kmax))) : 1.0f;
  if (tid == 0) *kscale_out = kscale;
  auto tap = [&](int dy, int dx) -> float {
    return (dx < -8 || dx > 8) ? 0.0f : kscale * s_k[(dy + 8) * kStencil + dx + 8];
  };
  for (int i = tid; i < kUmmaHalves; i += blockDim.x) {
    const int mat = i >> 8, e = i & 255;
    const int dyi = mat >> 1, kb = mat & 1;
    const int k = (e >> 7) * 8 + (e & 7), n = (e >> 3) & 15;
    umma[i] = __float2half_rn(tap(dyi - 8, 16 * kb + k - 8 - n));
  }
  for (int i = tid; i < kUmma32Halves; i += blockDim.x) {
    const int dyi = i >> 9, e = i & 511;
    const int k = (e >> 8) * 8 + (e & 7), n = (e >> 3) & 31;
    umma32[i] = __float2half_rn(tap(dyi - 8, k + 8 - n));
  }
}

}  // namespace

/* ============================================================== network */

struct tl_net {
  tl_context* ctx = nullptr;
  int n_params = 0;
  float* master = nullptr;      /* device, fp32 */
  float* grad = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int adam_t = 0;
  __nv_bfloat16* fwd16 = nullptr;  /* 3 layers x [tap][co][ci] */
  __nv_bfloat16* adj16 = nullptr;
  float* l1_fwd = nullptr;      /* [tap][co] */
  float* l1_adj = nullptr;      /* [tap][ci] */
  /* activation workspace */
  size_t cap_px = 0;
  __nv_bfloat16* act[kLayers + 1] = {};  /* a0 (1 ch), a1..a4 (16 ch) */
  __nv_bfloat16* bct[kLayers] = {};      /* b1..b3 (16 ch); index 0 unused */
  float* b0 = nullptr;
  float* q = nullptr;
  float* gz = nullptr;
  __nv_bfloat16* g16a = nullptr;
  __nv_bfloat16* g16b = nullptr;
  __nv_bfloat16* g1 = nullptr;
  float* gf = nullptr;
  float* partial = nullptr;
  size_t partial_cap = 0;
  float* dadj = nullptr;
  double* sums = nullptr;
  int sums_cap = 0;
  /* the network collapsed to its 17x17 stencil (collapse_kernel) */
  float* stencil_k = nullptr;     /* K, 289 floats */
  __half* stencil_umma = nullptr; /* the same as tcgen05 B operands */
  __half* stencil_umma32 = nullptr; /* window operands of N = 32 (persistent solve) */
  float* stencil_kscale = nullptr;
};

static int net_param_count() { return 9 * kCh + 3 * 9 * kCh * kCh; }

static int ensure_workspace(tl_net* net, size_t px, int batch) {
  if (px <= net->cap_px && batch <= net->sums_cap) return TL_OK;
  cudaStreamSynchronize(net->ctx->stream);
  for (auto& a : net->act) { cudaFree(a); a = nullptr; }
  for (auto& a : net->bct) { cudaFree(a); a = nullptr; }
  cudaFree(net->b0); cudaFree(net->q); cudaFree(net->gz); cudaFree(net->g16a);
  cudaFree(net->g16b); cudaFree(net->g1); cudaFree(net->gf); cudaFree(net->sums);
  TL_CUDA(cudaMalloc(&net->act[0], px * sizeof(__nv_bfloat16)));
  for (int l = 1; l <= kLayers; ++l) TL_CUDA(cudaMalloc(&net->act[l], px * kCh * 2));
  for (int l = 1; l < kLayers; ++l) TL_CUDA(cudaMalloc(&net->bct[l], px * kCh * 2));
  TL_CUDA(cudaMalloc(&net->b0, px * sizeof(float)));
  TL_CUDA(cudaMalloc(&net->q, px * sizeof(float)));
  TL_CUDA(cudaMalloc(&net->gz, px * sizeof(float)));
  TL_CUDA(cudaMalloc(&net->g16a, px * kCh * 2));
  TL_CUDA(cudaMalloc(&net->g16b, px * kCh * 2));
  TL_CUDA(cudaMalloc(&net->g1, px * 2));
  TL_CUDA(cudaMalloc(&net->gf, px * sizeof(float)));
  TL_CUDA(cudaMalloc(&net->sums, 2 * (size_t)std::max(batch, 1) * sizeof(double)));
  net->cap_px = px;
  net->sums_cap = std::max(batch, 1);
  return TL_OK;
}

static int grid1d(tl_context* ctx, size_t n) {
  size_t b = (n + 255) / 256;
  return (int)std::max<size_t>(1, std::min<size_t>(b, (size_t)ctx->num_sms * 16));
}

static int conv16(tl_net* net, const __nv_bfloat16* in, const __nv_bfloat16* w, void* out,
                  bool out_f32, int H, int W, int B) {
  dim3 grid(W / kTW, (H + kTH - 1) / kTH, B);
  if (out_f32)
    conv16_tc_kernel<true><<<grid, 128, 0, net->ctx->stream>>>(in, w, out, H, W);
  else
    conv16_tc_kernel<false><<<grid, 128, 0, net->ctx->stream>>>(in, w, out, H, W);
  TL_CHECK_LAUNCH(net->ctx);
  return TL_OK;
}

/* Forward of M^-1 on [B][H][W]: a0 = S r; a1..a4 = L1..L4; b3..b1 = L4^T..L2^T;
 * b0 = L1^T b1 (fp32); z = S (b0 + S r). Keeps every activation for the
 * backward (the Jacobi term has no weights, so dL/db0 = S dL/dz as before). */
static int net_forward(tl_net* net, const float* r, const float* s, float* z, int H, int W,
                       int B) {
  tl_context* ctx = net->ctx;
  const size_t n = (size_t)B * H * W;
  const int g = grid1d(ctx, n);
  scale_to_bf16_kernel<<<g, 256, 0, ctx->stream>>>(r, s, net->act[0], n);
  TL_CHECK_LAUNCH(ctx);
  conv1to16_kernel<<<g, 256, 0, ctx->stream>>>(net->act[0], net->l1_fwd, net->act[1], H, W, B);
  TL_CHECK_LAUNCH(ctx);
  const int n16 = 9 * kCh * kCh;
  for (int l = 1; l < kLayers; ++l) {
    int rc = conv16(net, net->act[l], net->fwd16 + (l - 1) * n16, net->act[l + 1], false, H, W, B);
    if (rc != TL_OK) return rc;
  }
  /* adjoints, last layer first: b3 = L4^T a4, b2 = L3^T b3, b1 = L2^T b2 */
  const __nv_bfloat16* src = net->act[kLayers];
  for (int l = kLayers - 1; l >= 1; --l) {
    int rc = conv16(net, src, net->adj16 + (l - 1) * n16, net->bct[l], false, H, W, B);
    if (rc != TL_OK) return rc;
    src = net->bct[l];
  }
  conv16to1_kernel<<<g, 256, 0, ctx->stream>>>(net->bct[1], net->l1_adj, net->b0, H, W, B);
  TL_CHECK_LAUNCH(ctx);
  output_kernel<<<g, 256, 0, ctx->stream>>>(net->b0, r, s, z, n);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

static int wgrad(tl_net* net, int kind, const __nv_bfloat16* x, const void* gy, float* dst,
                 int H, int W, int B) {
  /* kind 0: 16->16 (dst [tap][ci][co]); 1: 1->16 (dst [tap][co]); 2: 16->1 (dst [tap][ci]) */
  tl_context* ctx = net->ctx;
  const int nblocks = ctx->num_sms * 2;
  const int nout = kind == 0 ? 9 * kCh * kCh : 9 * kCh;
  const size_t need = (size_t)nblocks * nout;
  if (need > net->partial_cap) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(net->partial);
    TL_CUDA(cudaMalloc(&net->partial, need * sizeof(float)));
    net->partial_cap = need;
  }
  if (kind == 0)
    wgrad16_kernel<<<nblocks, 256, 0, ctx->stream>>>(x, (const __nv_bfloat16*)gy, net->partial,
                                                      H, W, B);
  else if (kind == 1)
    wgrad1to16_kernel<<<nblocks, 256, 0, ctx->stream>>>(x, (const __nv_bfloat16*)gy,
                                                         net->partial, H, W, B);
  else
    wgrad16to1_kernel<<<nblocks, 256, 0, ctx->stream>>>(x, (const float*)gy, net->partial, H,
                                                         W, B);
  TL_CHECK_LAUNCH(ctx);
  wgrad_sum_kernel<<<(nout + 255) / 256, 256, 0, ctx->stream>>>(net->partial, nblocks, nout, dst);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

namespace {

/* Gradient of an adjoint layer's weights folded back onto the forward
 * weights. wgrad returns, for a layer y = conv(x; k) with k stored
 * [tap][co][ci], the sums d[tap][ci][co] = sum_p x[p+tap][ci] g[p][co]; the
 * adjoint kernel of master weight m[tap][ci][co] sits at
 * k[8-tap][co'=ci][ci'=co], so dm[tap][ci][co] += d[8-tap][co][ci]. For the
 * 1-channel layer, m[tap][co] sits at the 16->1 kernel's [8-tap][ci'=co]. */
__global__ void fold_adjoint_grad_kernel(const float* __restrict__ dadj, float* __restrict__ dfwd,
                                         int cin_fwd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = 9 * cin_fwd * kCh;
  if (i >= n) return;
  if (cin_fwd == 1) {
    const int tap = i / kCh, co = i % kCh;
    dfwd[i] += dadj[(8 - tap) * kCh + co];
  } else {
    const int tap = i / (kCh * kCh), ci = (i / kCh) % kCh, co = i % kCh;
    dfwd[i] += dadj[((8 - tap) * kCh + co) * kCh + ci];
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ a, __nv_bfloat16* __restrict__ b,
                               size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16(a[i]);
}

static int refresh_weights(tl_net* net) {
  make_weights_kernel<<<(3 * 9 * kCh * kCh + 255) / 256, 256, 0, net->ctx->stream>>>(
      net->master, net->fwd16, net->adj16, net->l1_fwd, net->l1_adj);
  TL_CHECK_LAUNCH(net->ctx);
  collapse_kernel<<<1, 256, 0, net->ctx->stream>>>(net->master, net->stencil_k,
                                                    net->stencil_umma,
                                                    net->stencil_umma32, net->stencil_kscale);
  TL_CHECK_LAUNCH(net->ctx);
  return TL_OK;
}

/* Loss and gradients for one batch (see the file comment). Backward order:
 *   gb0 = s gz;  d(L1^T) = corr(b1, gb0);  g_b1 = L1 gb0
 *   for l = 2..4: d(Ll^T) = corr(b_l, g_b(l-1));  g_b(l) = Ll g_b(l-1)
 *   (with g_a4 = L4 g_b3 from the last of these)
 *   for l = 4..2: d(Ll) += corr(a_(l-1), g_a(l));  g_a(l-1) = Ll^T g_a(l)
 *   d(L1) += corr(a0, g_a1). */
static int net_loss_grad(tl_net* net, const float* r, const float* s, const float* kx,
                         const float* ky, int H, int W, int B, int margin, double* loss) {
  tl_context* ctx = net->ctx;
  const size_t n = (size_t)B * H * W;
  int rc = ensure_workspace(net, n, B);
  if (rc != TL_OK) return rc;
  rc = net_forward(net, r, s, net->gf, H, W, B); /* z -> gf */
  if (rc != TL_OK) return rc;
  TL_CUDA(cudaMemsetAsync(net->sums, 0, 2 * (size_t)B * sizeof(double), ctx->stream));
  const int g = grid1d(ctx, n);
  residual_loss_kernel<<<g, 256, 0, ctx->stream>>>(net->gf, r, kx, ky, net->q, H, W, B, margin,
                                                    net->sums);
  TL_CHECK_LAUNCH(ctx);
  loss_grad_kernel<<<g, 256, 0, ctx->stream>>>(net->q, kx, ky, net->sums, net->gz, H, W, B);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaMemsetAsync(net->grad, 0, net->n_params * sizeof(float), ctx->stream));
  scale_f32_kernel<<<g, 256, 0, ctx->stream>>>(net->gz, s, net->gf, n); /* gb0 */
  TL_CHECK_LAUNCH(ctx);
  const int n16 = 9 * kCh * kCh;
  float* dl1 = net->grad;
  float* dl16 = net->grad + 9 * kCh;
  float* dadj = net->dadj;
  /* L1^T */
  TL_CUDA(cudaMemsetAsync(dadj, 0, n16 * sizeof(float), ctx->stream));
  rc = wgrad(net, 2, net->bct[1], net->gf, dadj, H, W, B);
  if (rc != TL_OK) return rc;
  fold_adjoint_grad_kernel<<<1, 256, 0, ctx->stream>>>(dadj, dl1, 1);
  TL_CHECK_LAUNCH(ctx);
  to_bf16_kernel<<<g, 256, 0, ctx->stream>>>(net->gf, net->g1, n);
  TL_CHECK_LAUNCH(ctx);
  conv1to16_kernel<<<g, 256, 0, ctx->stream>>>(net->g1, net->l1_fwd, net->g16a, H, W, B);
  TL_CHECK_LAUNCH(ctx);
  /* L2^T .. L4^T: g_b(l-1) in g16a -> g_b(l) in g16b */
  __nv_bfloat16* gcur = net->g16a;
  __nv_bfloat16* gnext = net->g16b;
  for (int l = 1; l < kLayers; ++l) {
    /* layer b_l... : b_(l) = L(l+1)^T b_(l+1); input b_(l+1) (act bct[l+1] or a4) */
    const __nv_bfloat16* xin = (l + 1 < kLayers) ? net->bct[l + 1] : net->act[kLayers];
    TL_CUDA(cudaMemsetAsync(dadj, 0, n16 * sizeof(float), ctx->stream));
    rc = wgrad(net, 0, xin, gcur, dadj, H, W, B);
    if (rc != TL_OK) return rc;
    fold_adjoint_grad_kernel<<<(n16 + 255) / 256, 256, 0, ctx->stream>>>(
        dadj, dl16 + (l - 1) * n16, kCh);
    TL_CHECK_LAUNCH(ctx);
    rc = conv16(net, gcur, net->fwd16 + (l - 1) * n16, gnext, false, H, W, B);
    if (rc != TL_OK) return rc;
    std::swap(gcur, gnext);
  }
  /* gcur = g_a4. Forward layers L4..L2. */
  for (int l = kLayers - 1; l >= 1; --l) {
    rc = wgrad(net, 0, net->act[l], gcur, dl16 + (l - 1) * n16, H, W, B);
    if (rc != TL_OK) return rc;
    rc = conv16(net, gcur, net->adj16 + (l - 1) * n16, gnext, false, H, W, B);
    if (rc != TL_OK) return rc;
    std::swap(gcur, gnext);
  }
  /* gcur = g_a1; L1 */
  rc = wgrad(net, 1, net->act[0], gcur, dl1, H, W, B);
  if (rc != TL_OK) return rc;
  std::vector<double> sums(2 * (size_t)B);
  TL_CUDA(cudaMemcpyAsync(sums.data(), net->sums, sums.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  double num = 0.0, den = 0.0;
  for (int b = 0; b < B; ++b) {
    num += sums[2 * b];
    den += sums[2 * b + 1];
  }
  *loss = den > 0.0 ? num / den : 0.0;
  return TL_OK;
}

/* ------------------------------------------------------------ FPCG (FP32)
 * Flexible PCG on the packed interior [H][W] (no halo; zero-flux edges),
 * with z = M^-1 r from the network. Device-resident scalars avoid a host
 * round trip per step; the host reads r.r every few steps. */

struct FpcgScal {
  double rz, pw, alpha, beta, rr, rr0, zw;
};

__device__ __forceinline__ float apply_a_packed(const float* __restrict__ v,
                                                const float* __restrict__ kx,
                                                const float* __restrict__ ky, size_t p, int xx,
                                                int yy, int H, int W) {
  const float a = v[p];
  float s = a;
  if (xx + 1 < W) s += kx[p + 1] * (a - v[p + 1]);
  if (xx > 0) s += kx[p] * (a - v[p - 1]);
  if (yy + 1 < H) s += ky[p + W] * (a - v[p + W]);
  if (yy > 0) s += ky[p] * (a - v[p - W]);
  return s;
}

__device__ __forceinline__ void block_partial(double v, double* out) {
  __shared__ double s_red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TL_FULL_MASK, v, o);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = (lane < (int)(blockDim.x >> 5)) ? s_red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(TL_FULL_MASK, t, o);
    if (lane == 0) out[blockIdx.x] = t;
  }
  __syncthreads();
}

/* w = A p; partial p.w */
__global__ void fpcg_apply_kernel(const float* __restrict__ p, const float* __restrict__ kx,
                                  const float* __restrict__ ky, float* __restrict__ w, int H,
                                  int W, double* __restrict__ part) {
  const size_t n = (size_t)H * W;
  float acc = 0.0f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)(i / W);
    const float wv = apply_a_packed(p, kx, ky, i, xx, yy, H, W);
    w[i] = wv;
    acc += wv * p[i];
  }
  block_partial((double)acc, part);
}

/* mode 0: pw -> alpha = rz / pw.  mode 1: (z.r, z.w, r.r) -> beta, rz, rr. */
__global__ void fpcg_scalar_kernel(const double* __restrict__ part, int nblocks, int mode,
                                   FpcgScal* sc, double* rr_host) {
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[b];
    sc->pw = s;
    sc->alpha = sc->rz / s;
  } else {
    double zr = 0.0, zw = 0.0, rr = 0.0;
    for (int b = 0; b < nblocks; ++b) {
      zr += part[b];
      zw += part[nblocks + b];
      rr += part[2 * nblocks + b];
    }
    /* Polak-Ribiere: beta = z.(r_new - r_old) / rz_old, r_new - r_old = -alpha w */
    sc->beta = (mode == 2) ? 0.0 : -sc->alpha * zw / sc->rz;
    sc->rz = zr;
    sc->rr = rr;
    if (mode == 2) sc->rr0 = rr;
    *rr_host = rr;
  }
}

/* x += alpha p; r -= alpha w */
__global__ void fpcg_update_kernel(float* __restrict__ x, float* __restrict__ r,
                                   const float* __restrict__ p, const float* __restrict__ w,
                                   const FpcgScal* sc, size_t n) {
  const float a = (float)sc->alpha;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    r[i] -= a * w[i];
  }
}

/* partials of z.r, z.w, r.r (three consecutive arrays of nblocks) */
__global__ void fpcg_dots_kernel(const float* __restrict__ z, const float* __restrict__ r,
                                 const float* __restrict__ w, size_t n, double* __restrict__ part) {
  float zr = 0.f, zw = 0.f, rr = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    zr += z[i] * r[i];
    zw += z[i] * w[i];
    rr += r[i] * r[i];
  }
  block_partial((double)zr, part);
  block_partial((double)zw, part + gridDim.x);
  block_partial((double)rr, part + 2 * gridDim.x);
}

/* p = z + beta p */
__global__ void fpcg_p_kernel(float* __restrict__ p, const float* __restrict__ z,
                              const FpcgScal* sc, size_t n) {
  const float b = (float)sc->beta;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

/* packed <-> field layout helpers */
__global__ void pack_kernel(int x, int y, int hd, const double* __restrict__ src, double scale,
                            float* __restrict__ dst) {
  const int H = y - 2 * hd, W = x - 2 * hd;
  const size_t n = (size_t)H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)(i / W);
    dst[i] = (float)(src[(size_t)(yy + hd) * x + xx + hd] * scale);
  }
}

/* kx, ky and s = (diag)^-1/2 of the packed FP32 operator */
/* s = D^-1/2 of the packed operator: D = 1 + the couplings of the faces
 * inside the field. */
__global__ void packed_scaling_kernel(int H, int W, const float* __restrict__ kx,
                                      const float* __restrict__ ky, float* __restrict__ s) {
  const size_t n = (size_t)H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)(i / W);
    float d = 1.0f;
    if (xx + 1 < W) d += kx[i + 1];
    if (xx > 0) d += kx[i];
    if (yy + 1 < H) d += ky[i + W];
    if (yy > 0) d += ky[i];
    s[i] = rsqrtf(d);
  }
}

__global__ void pack_coeff_kernel(int x, int y, int hd, const double* __restrict__ kx,
                                  const double* __restrict__ ky, float* __restrict__ pkx,
                                  float* __restrict__ pky, float* __restrict__ ps) {
  const int H = y - 2 * hd, W = x - 2 * hd;
  const size_t n = (size_t)H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)(i / W);
    const size_t f = (size_t)(yy + hd) * x + xx + hd;
    pkx[i] = (float)kx[f];
    pky[i] = (float)ky[f];
    float d = 1.0f;
    if (xx + 1 < W) d += (float)kx[f + 1];
    if (xx > 0) d += (float)kx[f];
    if (yy + 1 < H) d += (float)ky[f + x];
    if (yy > 0) d += (float)ky[f];
    ps[i] = rsqrtf(d);
  }
}

__global__ void unpack_add_kernel(int x, int y, int hd, const float* __restrict__ e,
                                  double inv_scale, double* __restrict__ u) {
  const int H = y - 2 * hd, W = x - 2 * hd;
  const size_t n = (size_t)H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)(i / W);
    const size_t f = (size_t)(yy + hd) * x + xx + hd;
    u[f] = u[f] + (double)e[i] * inv_scale;
  }
}

/* Crops for training: out[b][h][w] = data[prob[b]][oy[b] + h][ox[b] + w]. */
__global__ void gather_crops_kernel(const float* __restrict__ data, int HS, int WS,
                                    const int* __restrict__ meta, int B, int H, int W,
                                    float* __restrict__ out) {
  const size_t n = (size_t)B * H * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)((i / W) % H), b = (int)(i / ((size_t)H * W));
    const int prob = meta[3 * b], oy = meta[3 * b + 1], ox = meta[3 * b + 2];
    out[i] = data[((size_t)prob * HS + oy + yy) * WS + ox + xx];
  }
}

}  // namespace

/* ================================================================= ABI */

extern "C" int tl_net_num_params(void) { return net_param_count(); }

extern "C" int tl_net_create(tl_context* ctx, tl_net** out) {
  TL_REQUIRE(ctx && out, "tl_net_create: null argument");
  tl_net* net = new tl_net();
  net->ctx = ctx;
  net->n_params = net_param_count();
  const size_t np = net->n_params;
  const int n16 = 9 * kCh * kCh;
  cudaError_t e = cudaMalloc(&net->master, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->grad, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->adam_m, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->adam_v, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->fwd16, 3 * n16 * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&net->adj16, 3 * n16 * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&net->l1_fwd, 9 * kCh * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->l1_adj, 9 * kCh * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->dadj, n16 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->stencil_k, kStencil * kStencil * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&net->stencil_umma, kUmmaHalves * sizeof(__half));
  if (e == cudaSuccess) e = cudaMalloc(&net->stencil_umma32, kUmma32Halves * sizeof(__half));
  if (e == cudaSuccess) e = cudaMalloc(&net->stencil_kscale, sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(net->master, 0, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(net->adam_m, 0, np * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(net->adam_v, 0, np * sizeof(float));
  if (e != cudaSuccess) {
    tl_net_destroy(net);
    return tl_cuda_error(e, "tl_net_create", __FILE__, __LINE__);
  }
  *out = net;
  return refresh_weights(net);
}

extern "C" int tl_net_destroy(tl_net* net) {
  if (!net) return TL_OK;
  if (net->ctx) cudaStreamSynchronize(net->ctx->stream);
  cudaFree(net->master); cudaFree(net->grad); cudaFree(net->adam_m); cudaFree(net->adam_v);
  cudaFree(net->fwd16); cudaFree(net->adj16); cudaFree(net->l1_fwd); cudaFree(net->l1_adj);
  cudaFree(net->dadj); cudaFree(net->partial);
  cudaFree(net->stencil_k); cudaFree(net->stencil_kscale);
  cudaFree(net->stencil_umma);
  cudaFree(net->stencil_umma32);
  for (auto& a : net->act) cudaFree(a);
  for (auto& a : net->bct) cudaFree(a);
  cudaFree(net->b0); cudaFree(net->q); cudaFree(net->gz); cudaFree(net->g16a);
  cudaFree(net->g16b); cudaFree(net->g1); cudaFree(net->gf); cudaFree(net->sums);
  delete net;
  return TL_OK;
}

extern "C" int tl_net_set_weights(tl_net* net, const float* host, int n) {
  TL_REQUIRE(net && host && n == net->n_params, "tl_net_set_weights: bad arguments");
  for (int i = 0; i < n; ++i) {
    if (!std::isfinite(host[i])) return tl_set_error(TL_ERR_NUMERIC, "non-finite weight");
  }
  TL_CUDA(cudaMemcpyAsync(net->master, host, n * sizeof(float), cudaMemcpyHostToDevice,
                          net->ctx->stream));
  TL_CUDA(cudaMemsetAsync(net->adam_m, 0, n * sizeof(float), net->ctx->stream));
  TL_CUDA(cudaMemsetAsync(net->adam_v, 0, n * sizeof(float), net->ctx->stream));
  net->adam_t = 0;
  int rc = refresh_weights(net);
  if (rc != TL_OK) return rc;
  TL_CUDA(cudaStreamSynchronize(net->ctx->stream));
  return TL_OK;
}

extern "C" int tl_net_get_weights(tl_net* net, float* host, int n) {
  TL_REQUIRE(net && host && n == net->n_params, "tl_net_get_weights: bad arguments");
  TL_CUDA(cudaMemcpyAsync(host, net->master, n * sizeof(float), cudaMemcpyDeviceToHost,
                          net->ctx->stream));
  TL_CUDA(cudaStreamSynchronize(net->ctx->stream));
  return TL_OK;
}

static int check_shape(int H, int W, int B) {
  TL_REQUIRE(H >= 4 && W >= kTW && H % kTH == 0 && W % kTW == 0 && B >= 1,
             "network input must be [B][H][W] with H % 4 == 0 and W % 64 == 0");
  return TL_OK;
}

extern "C" int tl_net_apply(tl_net* net, int H, int W, int B, const float* r, const float* s,
                            float* z) {
  TL_REQUIRE(net && r && s && z, "tl_net_apply: null argument");
  int rc = check_shape(H, W, B);
  if (rc != TL_OK) return rc;
  rc = ensure_workspace(net, (size_t)B * H * W, B);
  if (rc != TL_OK) return rc;
  return net_forward(net, r, s, z, H, W, B);
}

extern "C" int tl_net_loss_grad(tl_net* net, int H, int W, int B, int margin, const float* r,
                                const float* s, const float* kx, const float* ky, double* loss,
                                float* grad_host) {
  TL_REQUIRE(net && r && s && kx && ky && loss, "tl_net_loss_grad: null argument");
  int rc = check_shape(H, W, B);
  if (rc != TL_OK) return rc;
  TL_REQUIRE(margin >= 1 && 2 * margin < H && 2 * margin < W, "tl_net_loss_grad: bad margin");
  rc = net_loss_grad(net, r, s, kx, ky, H, W, B, margin, loss);
  if (rc != TL_OK) return rc;
  if (grad_host) {
    TL_CUDA(cudaMemcpyAsync(grad_host, net->grad, net->n_params * sizeof(float),
                            cudaMemcpyDeviceToHost, net->ctx->stream));
    TL_CUDA(cudaStreamSynchronize(net->ctx->stream));
  }
  return TL_OK;
}

extern "C" int tl_net_stencil(tl_net* net, float* host_k, float* kscale) {
  TL_REQUIRE(net && host_k, "tl_net_stencil: null argument");
  TL_CUDA(cudaMemcpyAsync(host_k, net->stencil_k, kStencil * kStencil * sizeof(float),
                          cudaMemcpyDeviceToHost, net->ctx->stream));
  float ks = 0.0f;
  TL_CUDA(cudaMemcpyAsync(&ks, net->stencil_kscale, sizeof(float), cudaMemcpyDeviceToHost,
                          net->ctx->stream));
  TL_CUDA(cudaStreamSynchronize(net->ctx->stream));
  if (kscale) *kscale = ks;
  return TL_OK;
}

extern "C" int tl_net_apply_stencil(tl_net* net, int H, int W, const float* r, const float* s,
                                    float* z) {
  TL_REQUIRE(net && r && s && z, "tl_net_apply_stencil: null argument");
  return tl_internal_apply_collapsed(net->ctx, net->stencil_umma, net->stencil_kscale, H, W, r,
                                     s, z);
}

extern "C" int tl_net_pcg(tl_net* net, int H, int W, const float* kx, const float* ky,
                          const float* b, float* e, float* work, double tol, int max_iters,
                          int* iters, double* rr) {
  TL_REQUIRE(net && kx && ky && b && e && work, "tl_net_pcg: null argument");
  TL_REQUIRE(H > 0 && W > 0 && W % 4 == 0, "tl_net_pcg: needs H > 0 and W % 4 == 0");
  tl_context* ctx = net->ctx;
  const size_t n = (size_t)H * W;
  float* s = work;
  float* r = work + n;
  packed_scaling_kernel<<<grid1d(ctx, n), 256, 0, ctx->stream>>>(H, W, kx, ky, s);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaMemcpyAsync(r, b, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  int it = 0;
  double rr_final = 0.0;
  const int rc = tl_internal_fpcg_collapsed(ctx, net->stencil_umma32, net->stencil_kscale, H, W,
                                            kx, ky, s, r, work + 2 * n, e, work + 3 * n,
                                            work + 4 * n, work + 5 * n, work + 6 * n, tol,
                                            max_iters, &it, &rr_final);
  if (rc != TL_OK) return rc;
  if (iters) *iters = it;
  if (rr) *rr = rr_final;
  return TL_OK;
}

int tl_internal_net_stencil(tl_net* net, const void** umma, const float** kscale) {
  TL_REQUIRE(net && umma && kscale, "tl_internal_net_stencil: null argument");
  *umma = net->stencil_umma32;
  *kscale = net->stencil_kscale;
  return TL_OK;
}

extern "C" int tl_net_adam_step(tl_net* net, float lr) {
  TL_REQUIRE(net && lr > 0.0f, "tl_net_adam_step: bad arguments");
  net->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)net->adam_t), c2 = 1.0f - powf(b2, (float)net->adam_t);
  adam_kernel<<<(net->n_params + 255) / 256, 256, 0, net->ctx->stream>>>(
      net->master, net->grad, net->adam_m, net->adam_v, net->n_params, lr, b1, b2, 1e-8f, c1, c2);
  TL_CHECK_LAUNCH(net->ctx);
  return refresh_weights(net);
}

extern "C" int tl_net_gather_crops(tl_context* ctx, const float* data, int HS, int WS,
                                   const int* meta_host, int B, int H, int W, float* out) {
  TL_REQUIRE(ctx && data && meta_host && out && B > 0, "tl_net_gather_crops: null argument");
  for (int b = 0; b < B; ++b) {
    TL_REQUIRE(meta_host[3 * b + 1] >= 0 && meta_host[3 * b + 1] + H <= HS &&
                   meta_host[3 * b + 2] >= 0 && meta_host[3 * b + 2] + W <= WS,
               "crop outside its source");
  }
  int* meta = nullptr;
  TL_CUDA(cudaMallocAsync((void**)&meta, 3 * (size_t)B * sizeof(int), ctx->stream));
  TL_CUDA(cudaMemcpyAsync(meta, meta_host, 3 * (size_t)B * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  gather_crops_kernel<<<grid1d(ctx, (size_t)B * H * W), 256, 0, ctx->stream>>>(data, HS, WS, meta,
                                                                               B, H, W, out);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaFreeAsync(meta, ctx->stream));
  return TL_OK;
}

extern "C" int tl_pack_interior(tl_context* ctx, int x, int y, int hd, const double* field,
                                double scale, float* packed) {
  TL_REQUIRE(ctx && field && packed, "tl_pack_interior: null argument");
  TL_REQUIRE(x > 2 * hd && y > 2 * hd && hd >= 1 &&
                 (size_t)x * (size_t)y <= (size_t)TL_MAX_CELLS,
             "tl_pack_interior: invalid grid dimensions");
  pack_kernel<<<grid1d(ctx, (size_t)x * y), 256, 0, ctx->stream>>>(x, y, hd, field, scale, packed);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

extern "C" int tl_pack_coefficients(tl_context* ctx, int x, int y, int hd, const double* kx,
                                    const double* ky, float* pkx, float* pky, float* ps) {
  TL_REQUIRE(ctx && kx && ky && pkx && pky && ps, "tl_pack_coefficients: null argument");
  TL_REQUIRE(x > 2 * hd && y > 2 * hd && hd >= 1 &&
                 (size_t)x * (size_t)y <= (size_t)TL_MAX_CELLS,
             "tl_pack_coefficients: invalid grid dimensions");
  pack_coeff_kernel<<<grid1d(ctx, (size_t)x * y), 256, 0, ctx->stream>>>(x, y, hd, kx, ky, pkx,
                                                                          pky, ps);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

int tl_internal_unpack_add(tl_context* ctx, int x, int y, int hd, const float* e,
                           double inv_scale, double* u) {
  unpack_add_kernel<<<grid1d(ctx, (size_t)x * y), 256, 0, ctx->stream>>>(x, y, hd, e, inv_scale,
                                                                          u);
  TL_CHECK_LAUNCH(ctx);
  return TL_OK;
}

/* Inner FPCG with the learned preconditioner, on packed FP32 arrays:
 * solves A32 e = r (r is overwritten with the final residual) until
 * r.r <= tol^2 r0.r0 or max_iters. */
int tl_internal_fpcg_learned(tl_context* ctx, tl_net* net, int H, int W, const float* kx,
                             const float* ky, const float* s, float* r, float* e, float* p,
                             float* w, float* z, double tol, int max_iters, int* iters) {
  const size_t n = (size_t)H * W;
  const int nb = std::min<int>(grid1d(ctx, n), 1024);
  int rc = tl_ensure_partials(ctx, 3 * (size_t)nb);
  if (rc != TL_OK) return rc;
  double* part = ctx->d_part;
  FpcgScal* sc = reinterpret_cast<FpcgScal*>(ctx->d_part + ctx->part_cap * 3);
  double* rr_host = ctx->h_result + 7;
  double* rr_dev = ctx->d_result + 7;
  TL_CUDA(cudaMemsetAsync(e, 0, n * sizeof(float), ctx->stream));
  TL_CUDA(cudaMemsetAsync(sc, 0, sizeof(FpcgScal), ctx->stream));
  /* z = M r; p = z; rz, rr */
  rc = tl_net_apply(net, H, W, 1, r, s, z);
  if (rc != TL_OK) return rc;
  TL_CUDA(cudaMemcpyAsync(p, z, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  TL_CUDA(cudaMemsetAsync(w, 0, n * sizeof(float), ctx->stream));
  fpcg_dots_kernel<<<nb, 256, 0, ctx->stream>>>(z, r, w, n, part);
  TL_CHECK_LAUNCH(ctx);
  fpcg_scalar_kernel<<<1, 32, 0, ctx->stream>>>(part, nb, 2, sc, rr_dev);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  const double rr0 = *(volatile double*)rr_host;
  int k = 0;
  if (rr0 > 0.0) {
    for (k = 1; k <= max_iters; ++k) {
      fpcg_apply_kernel<<<nb, 256, 0, ctx->stream>>>(p, kx, ky, w, H, W, part);
      TL_CHECK_LAUNCH(ctx);
      fpcg_scalar_kernel<<<1, 32, 0, ctx->stream>>>(part, nb, 0, sc, rr_dev);
      TL_CHECK_LAUNCH(ctx);
      fpcg_update_kernel<<<nb, 256, 0, ctx->stream>>>(e, r, p, w, sc, n);
      TL_CHECK_LAUNCH(ctx);
      rc = tl_net_apply(net, H, W, 1, r, s, z);
      if (rc != TL_OK) return rc;
      fpcg_dots_kernel<<<nb, 256, 0, ctx->stream>>>(z, r, w, n, part);
      TL_CHECK_LAUNCH(ctx);
      fpcg_scalar_kernel<<<1, 32, 0, ctx->stream>>>(part, nb, 1, sc, rr_dev);
      TL_CHECK_LAUNCH(ctx);
      fpcg_p_kernel<<<nb, 256, 0, ctx->stream>>>(p, z, sc, n);
      TL_CHECK_LAUNCH(ctx);
      if (k % 4 == 0 || k == max_iters) {
        TL_CUDA(cudaStreamSynchronize(ctx->stream));
        const double rr = *(volatile double*)rr_host;
        if (!(rr == rr)) break;
        if (rr <= tol * tol * rr0) break;
      }
    }
    if (k > max_iters) k = max_iters;
  }
  *iters = k;
  return TL_OK;
}
