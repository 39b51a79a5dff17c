/*
 * tl_context.cu -- context, field allocation and error reporting of the
 * GB300 TeaLeaf backend (C ABI in include/tealeaf_gb300.h).
 *
 * Replaces the SYCL queue and buffer management of the reference backend
 * (TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:31-125): fields are plain
 * 256-byte-aligned device allocations, and the per-call temporary reduction
 * buffers of the reference (cg.cpp:80,145,206) become scratch owned by the
 * context and reused by every call.
 */
#include <stdio.h>
#include <string.h>

#include <string>

#include "tl_internal.cuh"

static thread_local std::string g_last_error;

int tl_set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int tl_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed at %s:%d: %s (%s)", what, file, line,
           cudaGetErrorString(e), cudaGetErrorName(e));
  return tl_set_error(TL_ERR_CUDA, buf);
}

extern "C" const char* tl_last_error(void) { return g_last_error.c_str(); }

extern "C" int tl_context_create(int device, void* stream, tl_context** out) {
  TL_REQUIRE(out != nullptr, "tl_context_create: out is null");
  *out = nullptr;
  int count = 0;
  TL_CUDA(cudaGetDeviceCount(&count));
  TL_REQUIRE(device >= 0 && device < count, "tl_context_create: no such device");
  TL_CUDA(cudaSetDevice(device));
  tl_context* ctx = new tl_context();
  ctx->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete ctx;
    return tl_cuda_error(e, "cudaGetDeviceProperties", __FILE__, __LINE__);
  }
  ctx->num_sms = prop.multiProcessorCount;
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      return tl_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    ctx->owns_stream = true;
  }
  e = cudaMalloc(&ctx->d_sync, TL_SYNC_WORDS * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_sync, 0, TL_SYNC_WORDS * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
  if (e == cudaSuccess)
    e = cudaHostAlloc(&ctx->h_result, TL_NUM_SLOTS * sizeof(double), cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(&ctx->d_result, ctx->h_result, 0);
  if (e == cudaSuccess) e = cudaHostAlloc(&ctx->h_steps, 8 * sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(&ctx->d_steps, ctx->h_steps, 0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_start);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_stop);
  if (e != cudaSuccess) {
    tl_context_destroy(ctx);
    return tl_cuda_error(e, "context scratch allocation", __FILE__, __LINE__);
  }
  memset(ctx->h_result, 0, TL_NUM_SLOTS * sizeof(double));
  memset(ctx->h_steps, 0, 8 * sizeof(int));
  *out = ctx;
  return TL_OK;
}

extern "C" int tl_context_destroy(tl_context* ctx) {
  if (!ctx) return TL_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_part);
  cudaFree(ctx->d_sync);
  cudaFree(ctx->d_status);
  cudaFree(ctx->d_hist);
  cudaFree(ctx->d_stage);
  cudaFree(ctx->d_diag);
  cudaFree(ctx->d_f32);
  cudaFree(ctx->d_ainv);
  cudaFree(ctx->d_ainv16);
  cudaFree(ctx->d_proj);
  cudaFree(ctx->d_proj_part);
  cudaFree(ctx->d_hash64);
  cudaFree(ctx->d_diag64);
  cudaFree(ctx->d_coarse_work);
  cudaFree(ctx->d_coarse_vec);
  cudaFree(ctx->d_hash);
  if (ctx->h_result) cudaFreeHost(ctx->h_result);
  if (ctx->h_steps) cudaFreeHost(ctx->h_steps);
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
  if (ctx->owns_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return TL_OK;
}

extern "C" int tl_context_stream(tl_context* ctx, void** stream) {
  TL_REQUIRE(ctx && stream, "tl_context_stream: null argument");
  *stream = (void*)ctx->stream;
  return TL_OK;
}

extern "C" int tl_synchronize(tl_context* ctx) {
  TL_REQUIRE(ctx, "tl_synchronize: null context");
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_last_solve_stats(tl_context* ctx, tl_solve_stats* out) {
  TL_REQUIRE(ctx && out, "tl_last_solve_stats: null argument");
  *out = ctx->last_solve;
  return TL_OK;
}

extern "C" int tl_set_fp64_contract(tl_context* ctx, int contract) {
  TL_REQUIRE(ctx, "tl_set_fp64_contract: null context");
  TL_REQUIRE(contract == TL_FP64_EXACT || contract == TL_FP64_FUSED,
             "tl_set_fp64_contract: unknown contract");
  ctx->fp64_fused = contract == TL_FP64_FUSED;
  return TL_OK;
}

extern "C" long long tl_launch_count(tl_context* ctx) {
  return ctx ? ctx->launches : -1;
}

int tl_ensure_partials(tl_context* ctx, size_t ntiles) {
  if (ntiles > TL_MAX_TILES) {
    return tl_set_error(TL_ERR_ARG, "grid too large for the reduction scratch");
  }
  if (ntiles <= ctx->part_cap) return TL_OK;
  size_t cap = ntiles < 1024 ? 1024 : ntiles;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d_part);
  ctx->d_part = nullptr;
  ctx->part_cap = 0;
  TL_CUDA(cudaMalloc(&ctx->d_part, 4 * cap * sizeof(double)));
  ctx->part_cap = cap;
  return TL_OK;
}

int tl_ensure_history(tl_context* ctx, size_t n) {
  if (n <= ctx->hist_cap) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d_hist);
  ctx->d_hist = nullptr;
  ctx->hist_cap = 0;
  TL_CUDA(cudaMalloc(&ctx->d_hist, 2 * n * sizeof(double)));
  ctx->hist_cap = n;
  return TL_OK;
}

int tl_ensure_stage(tl_context* ctx, size_t n) {
  if (n <= ctx->stage_cap) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d_stage);
  ctx->d_stage = nullptr;
  ctx->stage_cap = 0;
  TL_CUDA(cudaMalloc(&ctx->d_stage, n * sizeof(double)));
  ctx->stage_cap = n;
  return TL_OK;
}

int tl_ensure_diag(tl_context* ctx, size_t n) {
  if (n <= ctx->diag_cap) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d_diag);
  ctx->d_diag = nullptr;
  ctx->diag_cap = 0;
  TL_CUDA(cudaMalloc(&ctx->d_diag, n * sizeof(double)));
  ctx->diag_cap = n;
  return TL_OK;
}

extern "C" int tl_field_alloc(tl_context* ctx, size_t count, double** dev_out) {
  TL_REQUIRE(ctx && dev_out, "tl_field_alloc: null argument");
  *dev_out = nullptr;
  void* p = nullptr;
  TL_CUDA(cudaMalloc(&p, (count ? count : 1) * sizeof(double)));
  cudaError_t e = cudaMemsetAsync(p, 0, (count ? count : 1) * sizeof(double), ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(p);
    return tl_cuda_error(e, "cudaMemsetAsync", __FILE__, __LINE__);
  }
  *dev_out = (double*)p;
  return TL_OK;
}

extern "C" int tl_field_free(tl_context* ctx, double* dev) {
  TL_REQUIRE(ctx, "tl_field_free: null context");
  if (!dev) return TL_OK;
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  TL_CUDA(cudaFree(dev));
  return TL_OK;
}

extern "C" int tl_copy_to_device(tl_context* ctx, double* dev, const double* host,
                                 size_t count) {
  TL_REQUIRE(ctx && (count == 0 || (dev && host)), "tl_copy_to_device: null argument");
  if (count == 0) return TL_OK;
  TL_CUDA(cudaMemcpyAsync(dev, host, count * sizeof(double), cudaMemcpyHostToDevice,
                          ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

extern "C" int tl_copy_to_host(tl_context* ctx, double* host, const double* dev,
                               size_t count) {
  TL_REQUIRE(ctx && (count == 0 || (dev && host)), "tl_copy_to_host: null argument");
  if (count == 0) return TL_OK;
  TL_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(double), cudaMemcpyDeviceToHost,
                          ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}

/* One block waits at the grid barrier for an arrival that never comes
 * (expected = 2 with a single block), for budget_ms; the barrier gives up,
 * records TL_ERR_TIMEOUT and the kernel returns. */
static __global__ void barrier_selftest_kernel(unsigned* sync, int* status,
                                               unsigned long long budget_ns) {
  tl_grid_barrier_n(sync, status, 2u, budget_ns);
}

extern "C" int tl_selftest_barrier_timeout(tl_context* ctx, int budget_ms, int* status) {
  TL_REQUIRE(ctx && status && budget_ms > 0 && budget_ms <= 1000,
             "tl_selftest_barrier_timeout: budget must be in (0, 1000] ms");
  TL_CUDA(cudaMemsetAsync(ctx->d_sync + TL_SYNC_BAR_COUNT, 0, 2 * sizeof(unsigned), ctx->stream));
  TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  barrier_selftest_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_sync, ctx->d_status,
                                                     (unsigned long long)budget_ms * 1000000ull);
  TL_CHECK_LAUNCH(ctx);
  TL_CUDA(cudaMemcpyAsync(status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  /* leave the barrier words clean for the next persistent kernel */
  TL_CUDA(cudaMemsetAsync(ctx->d_sync + TL_SYNC_BAR_COUNT, 0, 2 * sizeof(unsigned), ctx->stream));
  TL_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  TL_CUDA(cudaStreamSynchronize(ctx->stream));
  return TL_OK;
}
