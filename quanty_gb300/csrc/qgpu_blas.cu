// Plain dense complex GEMMs of the block eigensolver through cuBLAS: the Gram products of
// Krylov blocks (V^H W), the projections (W -= V C) and the Ritz combinations (X = V Y).
// These are ordinary tall-skinny matrix products, FP64 throughout (the library's default math
// mode, no emulation); the H*psi path stays in this library's own kernels.
//
// Matrices are row-major n x k blocks (element (r, c) at r * ld + c), which is column-major
// k x n with leading dimension ld, so every product is issued on the transposed problem.
#include <cublas_v2.h>

#include "qgpu_internal.cuh"

static qg_status blas_fail(qg_context ctx, cublasStatus_t s, const char *what) {
  ctx->last_error = std::string(what) + ": cuBLAS status " + std::to_string((int)s);
  return s == CUBLAS_STATUS_ALLOC_FAILED ? QG_ERR_OOM : QG_ERR_CUDA;
}

static qg_status blas_handle(qg_context ctx, cublasHandle_t *h) {
  if (!ctx->blas) {
    cublasHandle_t nh = nullptr;
    cublasStatus_t s = cublasCreate(&nh);
    if (s != CUBLAS_STATUS_SUCCESS) return blas_fail(ctx, s, "cublasCreate");
    ctx->blas = nh;
  }
  *h = (cublasHandle_t)ctx->blas;
  cublasStatus_t s = cublasSetStream(*h, ctx->stream);
  if (s != CUBLAS_STATUS_SUCCESS) return blas_fail(ctx, s, "cublasSetStream");
  return QG_OK;
}

void qg_blas_release(qg_context ctx) {
  if (ctx->blas) cublasDestroy((cublasHandle_t)ctx->blas);
  ctx->blas = nullptr;
}

// C (ka x kb, row-major, ld kb) = A^H B over n rows; A: n x ka (ld lda), B: n x kb (ld ldb).
// Transposed: C^T (kb x ka, column-major) = B^T conj(A) = Bcm * Acm^H.
qg_status qg_zgemm_ahb(qg_context ctx, const double2 *A, int lda, int ka, const double2 *B, int ldb, int kb,
                       int64_t n, double2 *C) {
  if (ka <= 0 || kb <= 0) return QG_OK;
  if (n <= 0) {
    QG_CUDA(ctx, cudaMemsetAsync(C, 0, (size_t)ka * kb * 16, ctx->stream));
    return QG_OK;
  }
  cublasHandle_t h = nullptr;
  QG_TRY(blas_handle(ctx, &h));
  const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
  cublasStatus_t s = cublasZgemm_64(h, CUBLAS_OP_N, CUBLAS_OP_C, kb, ka, n, &one, (const cuDoubleComplex *)B, ldb,
                                    (const cuDoubleComplex *)A, lda, &zero, (cuDoubleComplex *)C, kb);
  if (s != CUBLAS_STATUS_SUCCESS) return blas_fail(ctx, s, "Gram product");
  return QG_OK;
}

// X (n x kb, ld ldx) = beta X + alpha A M; A: n x ka (ld lda), M: ka x kb row-major (ld kb).
// Transposed: X^T = beta X^T + alpha M^T A^T, with M^T the column-major view of M.
qg_status qg_zgemm_acc(qg_context ctx, const double2 *A, int lda, int ka, const double2 *M, double2 *X, int ldx,
                       int kb, int64_t n, double alpha, double beta) {
  if (kb <= 0 || n <= 0) return QG_OK;
  if (ka <= 0) return beta == 1.0 ? QG_OK : QG_ERR_ARG;  // no terms (the solver never asks to rescale)
  cublasHandle_t h = nullptr;
  QG_TRY(blas_handle(ctx, &h));
  const cuDoubleComplex a = make_cuDoubleComplex(alpha, 0.0), b = make_cuDoubleComplex(beta, 0.0);
  cublasStatus_t s;
  s = cublasZgemm_64(h, CUBLAS_OP_N, CUBLAS_OP_N, kb, n, ka, &a, (const cuDoubleComplex *)M, kb,
                     (const cuDoubleComplex *)A, lda, &b, (cuDoubleComplex *)X, ldx);
  if (s != CUBLAS_STATUS_SUCCESS) return blas_fail(ctx, s, "block update");
  return QG_OK;
}

// out (n x np, row-major) = sum_i K_i C[i][:]: the vectors K_i (vector-major, K[i * n + r],
// i < ntri) combined with C (ntri x np, row-major).  Transposed: out^T = C^T K^T.
qg_status qg_zgemm_combine(qg_context ctx, const double2 *K, int64_t n, int ntri, const double2 *C, int np,
                           double2 *out) {
  if (n <= 0 || np <= 0) return QG_OK;
  if (ntri <= 0) {
    QG_CUDA(ctx, cudaMemsetAsync(out, 0, (size_t)n * np * 16, ctx->stream));
    return QG_OK;
  }
  cublasHandle_t h = nullptr;
  QG_TRY(blas_handle(ctx, &h));
  const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
  cublasStatus_t s = cublasZgemm_64(h, CUBLAS_OP_N, CUBLAS_OP_T, np, n, ntri, &one, (const cuDoubleComplex *)C, np,
                                    (const cuDoubleComplex *)K, n, &zero, (cuDoubleComplex *)out, np);
  if (s != CUBLAS_STATUS_SUCCESS) return blas_fail(ctx, s, "Krylov combination");
  return QG_OK;
}
