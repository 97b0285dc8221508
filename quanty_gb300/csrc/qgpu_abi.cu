// Context, error handling and small shared services of the C ABI (include/qgpu.h).
#include <cstdio>
#include <cstring>

#include "qgpu_internal.cuh"

qg_status qg_cuda_fail(qg_context ctx, cudaError_t e, const char *what) {
  if (ctx) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    ctx->last_error = buf;
  }
  cudaGetLastError();  // clear a non-sticky error
  return e == cudaErrorMemoryAllocation ? QG_ERR_OOM : QG_ERR_CUDA;
}

qg_status qg_check_launch(qg_context ctx, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, what);
  return QG_OK;
}

// Read and clear the device error word (synchronises the stream).
qg_status qg_check_device_error(qg_context ctx, const char *what) {
  unsigned int h = 0, zero = 0;
  cudaError_t e = cudaMemcpyAsync(&h, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->d_err, &zero, 4, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, what);
  if (h & QG_DEVERR_TIMEOUT) {
    ctx->last_error = std::string(what) + ": bounded wait on a bulk copy gave up";
    return QG_ERR_TIMEOUT;
  }
  if (h & QG_DEVERR_PROBE) {
    ctx->last_error = std::string(what) + ": hash probe limit reached";
    return QG_ERR_TIMEOUT;
  }
  if (h & (QG_DEVERR_TABLE_FULL | QG_DEVERR_OVERFLOW)) {
    ctx->last_error = std::string(what) + ": device table or list full";
    return QG_ERR_TABLE_FULL;
  }
  return QG_OK;
}

qg_status qg_ensure_scratch(qg_context ctx, size_t bytes) {
  if (ctx->scratch_bytes >= bytes) return QG_OK;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_scratch);
  ctx->d_scratch = nullptr;
  ctx->scratch_bytes = 0;
  size_t b = bytes < 65536 ? 65536 : bytes;
  QG_CUDA(ctx, cudaMalloc(&ctx->d_scratch, b));
  ctx->scratch_bytes = b;
  return QG_OK;
}

qg_status qg_ensure_pinned(qg_context ctx, size_t bytes) {
  if (ctx->pinned_bytes >= bytes) return QG_OK;
  cudaFreeHost(ctx->h_pinned);
  ctx->h_pinned = nullptr;
  ctx->pinned_bytes = 0;
  QG_CUDA(ctx, cudaMallocHost(&ctx->h_pinned, bytes));
  ctx->pinned_bytes = bytes;
  return QG_OK;
}

extern "C" qg_status qg_init(int device, qg_context *out) {
  if (!out) return QG_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || device < 0 || device >= ndev) {
    cudaGetLastError();
    return QG_ERR_CUDA;
  }
  qg_context ctx = new qg_context_s();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  ctx->own_stream = true;
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_err, 4);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, 4);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    qg_cuda_fail(ctx, e, "qg_init");
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    cudaFree(ctx->d_err);
    delete ctx;
    return QG_ERR_CUDA;
  }
  *out = ctx;
  return QG_OK;
}

extern "C" qg_status qg_finalize(qg_context ctx) {
  if (!ctx) return QG_OK;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_err);
  cudaFree(ctx->d_scratch);
  cudaFreeHost(ctx->h_pinned);
  cudaFree(ctx->d_io);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return QG_OK;
}

extern "C" qg_status qg_set_stream(qg_context ctx, void *stream) {
  if (!ctx) return QG_ERR_ARG;
  cudaStreamSynchronize(ctx->stream);
  if (stream) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
  } else if (!ctx->own_stream) {
    QG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
  }
  return QG_OK;
}

extern "C" void *qg_get_stream(qg_context ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" const char *qg_last_error(qg_context ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

extern "C" int64_t qg_launch_count(qg_context ctx) { return ctx ? ctx->launches : 0; }

extern "C" qg_status qg_synchronize(qg_context ctx) {
  if (!ctx) return QG_ERR_ARG;
  QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return qg_check_device_error(ctx, "qg_synchronize");
}
