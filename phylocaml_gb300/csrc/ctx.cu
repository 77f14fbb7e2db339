// Context management, error reporting and the grow-only device buffers.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>

#include "pgpu_internal.cuh"

pgpu_status pgpu_set_err(pgpu_ctx *ctx, pgpu_status st, const char *fmt, ...) {
  if (ctx) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    ctx->err = msg;
  }
  return st;
}

pgpu_status pgpu_buf(pgpu_ctx *ctx, int slot, size_t bytes, void **out) {
  if (bytes == 0) bytes = 16;
  if (ctx->cap[slot] < bytes) {
    if (ctx->buf[slot]) {
      // the previous contents may still be in use by queued work
      PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      PGPU_CUDA(ctx, cudaFree(ctx->buf[slot]));
      ctx->buf[slot] = nullptr;
      ctx->cap[slot] = 0;
    }
    size_t want = (bytes + 255) & ~size_t(255);
    PGPU_CUDA(ctx, cudaMalloc(&ctx->buf[slot], want));
    ctx->cap[slot] = want;
  }
  *out = ctx->buf[slot];
  return PGPU_OK;
}

pgpu_status pgpu_after_launch(pgpu_ctx *ctx, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgpu_set_err(ctx, PGPU_ERR_CUDA, "launch of %s failed: %s", what,
                        cudaGetErrorString(e));
  ctx->launches++;
  return PGPU_OK;
}

pgpu_status pgpu_check_flag(pgpu_ctx *ctx, const char *what) {
  int flag = 0;
  PGPU_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    PGPU_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    if (flag & PGPU_FLAG_TIMEOUT)
      return pgpu_set_err(ctx, PGPU_ERR_TIMEOUT, "%s: a device wait gave up", what);
    if (flag & PGPU_FLAG_BADCODE)
      return pgpu_set_err(ctx, PGPU_ERR_ARG, "%s: a tip code is outside the code table", what);
    if (flag & PGPU_FLAG_NAN)
      return pgpu_set_err(ctx, PGPU_ERR_NAN, "%s: NaN or Inf in Q or pi (or pi <= 0)", what);
    if (flag & PGPU_FLAG_NONREV)
      return pgpu_set_err(ctx, PGPU_ERR_NONREVERSIBLE, "%s: Q is not reversible w.r.t. pi", what);
    if (flag & PGPU_FLAG_EIGEN)
      return pgpu_set_err(ctx, PGPU_ERR_EIGEN, "%s: eigendecomposition did not converge", what);
    return pgpu_set_err(ctx, PGPU_ERR_CUDA, "%s: device error flag %d", what, flag);
  }
  return PGPU_OK;
}

pgpu_status pgpu_settle_copies(pgpu_ctx *ctx, pgpu_status st) {
  if (st != PGPU_OK) {
    for (cudaStream_t cs : {ctx->stream, ctx->copy_stream, ctx->d2h_stream, ctx->aux_stream})
      if (cs) cudaStreamSynchronize(cs);
    (void)cudaGetLastError();
  }
  return st;
}

void *pgpu_host_view(const void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

pgpu_status pgpu_copy_stream(pgpu_ctx *ctx) {
  if (ctx->copy_stream) return PGPU_OK;
  PGPU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  PGPU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking));
  for (cudaEvent_t &e : ctx->copy_ev)
    PGPU_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (cudaEvent_t &e : ctx->done_ev)
    PGPU_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  PGPU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
  for (cudaEvent_t &e : ctx->aux_ev)
    PGPU_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return PGPU_OK;
}

extern "C" {

int pgpu_version(void) { return 100; }

pgpu_status pgpu_create(pgpu_ctx **out, int device) {
  if (!out) return PGPU_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    (void)cudaGetLastError();
    return PGPU_ERR_UNSUPPORTED;
  }
  if (device < 0 || device >= n) return PGPU_ERR_ARG;
  pgpu_ctx *ctx = new pgpu_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  cudaDeviceProp prop;
  if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, device);
  if (e == cudaSuccess) {
    ctx->num_sms = prop.multiProcessorCount;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) ctx->own_stream = true;
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_flag, 256);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_flag, 0, 256);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_pinned, 4096);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    pgpu_destroy(ctx);
    return e == cudaErrorMemoryAllocation ? PGPU_ERR_OOM : PGPU_ERR_CUDA;
  }
  if (ctx->cc_major < 10) {
    // the kernels use sm_100-family instructions (bulk copies, mbarrier tx)
    pgpu_destroy(ctx);
    return PGPU_ERR_UNSUPPORTED;
  }
  *out = ctx;
  return PGPU_OK;
}

void pgpu_destroy(pgpu_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < BUF_COUNT; ++i)
    if (ctx->buf[i]) cudaFree(ctx->buf[i]);
  if (ctx->d_flag) cudaFree(ctx->d_flag);
  for (int k = 0; k < 2; ++k) {
    if (ctx->stage_h[k]) cudaFreeHost(ctx->stage_h[k]);
    if (ctx->stage_d[k]) cudaFree(ctx->stage_d[k]);
    if (ctx->stage_ev[k]) cudaEventDestroy(ctx->stage_ev[k]);
  }
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  for (cudaStream_t cs : {ctx->copy_stream, ctx->d2h_stream, ctx->aux_stream})
    if (cs) {
      cudaStreamSynchronize(cs);
      cudaStreamDestroy(cs);
    }
  for (cudaEvent_t &e : ctx->copy_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t &e : ctx->done_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t &e : ctx->aux_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  (void)cudaGetLastError();
  delete ctx;
}

const char *pgpu_last_error(const pgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }


pgpu_status pgpu_set_stream(pgpu_ctx *ctx, void *cuda_stream) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->own_stream) {
    cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
  }
  if (cuda_stream) {
    ctx->stream = (cudaStream_t)cuda_stream;
  } else {
    PGPU_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
  }
  return PGPU_OK;
}

pgpu_status pgpu_synchronize(pgpu_ctx *ctx) {
  if (!ctx) return PGPU_ERR_ARG;
  PGPU_CUDA(ctx, cudaSetDevice(ctx->device));
  PGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return pgpu_check_flag(ctx, "synchronize");
}

uint64_t pgpu_kernel_launches(const pgpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

void *pgpu_get_stream(const pgpu_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

}  // extern "C"
