// The dense path for small bases (the reference switches to it below DenseBorder = 1513
// determinants): the operator as a dense matrix on a determinant basis, and spectra from a list
// of poles.
//
// * qg_operator_dense: OperatorToDeterminantMatrix (Core/MatrixOperator.cpp:1149).  Column c of
//   the matrix is op applied to the unit vector of row c, so the whole matrix is one
//   multi-vector apply of the identity block (n vectors on n rows).
// * qg_poles_spectra: ListOfPolesToSpectrum (Core/Spectral.cpp:1516, the Gamma > 0 branch
//   :1576-1588): G(w) = a0 + sum_k b_k / (w - a_k + i Gamma/2) at w = emin + k de + e0, every
//   (spectrum, frequency) pair in one kernel.
#include "qgpu_internal.cuh"

__global__ void k_identity(double2 *m, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * n) return;
  m[i] = make_double2((i / n) == (i % n) ? 1.0 : 0.0, 0.0);
}

// one thread per (spectrum, frequency); poles and weights of spectrum s at [s * npole ..]
__global__ void k_poles(int nspec, int npole, const double *__restrict__ pa, const double *__restrict__ pb,
                        const double *__restrict__ e0, double emin, double de, int ne, double gamma,
                        double2 *__restrict__ g) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t tot = (int64_t)nspec * (ne + 1);
  if (i >= tot) return;
  int s = (int)(i / (ne + 1));
  int k = (int)(i % (ne + 1));
  double w = (double)k * de + emin + e0[s];
  double hg = gamma / 2.0, hg2 = hg * hg;
  double re = 0.0, im = 0.0;
  const double *a = pa + (size_t)s * npole, *b = pb + (size_t)s * npole;
  for (int p = 0; p < npole; p++) {
    double d = w - a[p];
    double den = hg2 + d * d;
    re += b[p] * d / den;
    im += b[p] * (-hg) / den;
  }
  g[i] = make_double2(re, im);
}

extern "C" qg_status qg_operator_dense(qg_context ctx, qg_operator op, qg_basis b, double *m_host) {
  if (!ctx || !op || !b || !m_host || op->nf != b->nf) return QG_ERR_ARG;
  int64_t n = b->n;
  if (n == 0) return QG_OK;
  if (n > 16384) {
    ctx->last_error = "qg_operator_dense: more than 16384 determinants";
    return QG_ERR_ARG;
  }
  double2 *I = nullptr, *M = nullptr;
  cudaError_t e = cudaMalloc(&I, (size_t)n * n * 16);
  if (e == cudaSuccess) e = cudaMalloc(&M, (size_t)n * n * 16);
  if (e != cudaSuccess) {
    cudaFree(I);
    cudaFree(M);
    ctx->last_error = "qg_operator_dense: out of device memory";
    return QG_ERR_OOM;
  }
  k_identity<<<(unsigned)((n * n + 255) / 256), 256, 0, ctx->stream>>>(I, n);
  ctx->launches++;
  // (M)[r][c] = (op e_c)_r: the n unit vectors as one block of n vectors
  qg_status st = qg_apply(ctx, op, b, b, (const double *)I, (double *)M, (int32_t)n);
  if (st == QG_OK) {
    e = cudaMemcpyAsync(m_host, M, (size_t)n * n * 16, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_operator_dense");
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(I);
  cudaFree(M);
  if (st == QG_OK) st = qg_check_device_error(ctx, "qg_operator_dense");
  return st;
}

extern "C" qg_status qg_poles_spectra(qg_context ctx, int32_t nspec, int32_t npole, const double *a_host,
                                      const double *b_host, const double *e0_host, double emin, double de,
                                      int32_t ne, double gamma, double *g_host) {
  if (!ctx || nspec <= 0 || npole < 0 || ne < 0 || !(gamma > 0) || !e0_host || !g_host ||
      (npole && (!a_host || !b_host)))
    return QG_ERR_ARG;
  cudaStream_t s = ctx->stream;
  size_t pb = (size_t)nspec * std::max(npole, 1) * 8, gb = (size_t)nspec * (ne + 1) * 16;
  double *da = nullptr, *db = nullptr, *de0 = nullptr;
  double2 *dg = nullptr;
  cudaError_t e = cudaMalloc(&da, pb);
  if (e == cudaSuccess) e = cudaMalloc(&db, pb);
  if (e == cudaSuccess) e = cudaMalloc(&de0, (size_t)nspec * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dg, gb);
  if (e == cudaSuccess && npole) e = cudaMemcpyAsync(da, a_host, (size_t)nspec * npole * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && npole) e = cudaMemcpyAsync(db, b_host, (size_t)nspec * npole * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(de0, e0_host, (size_t)nspec * 8, cudaMemcpyHostToDevice, s);
  qg_status st = QG_OK;
  if (e == cudaSuccess) {
    int64_t tot = (int64_t)nspec * (ne + 1);
    k_poles<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(nspec, npole, da, db, de0, emin, de, ne, gamma, dg);
    ctx->launches++;
    st = qg_check_launch(ctx, "qg_poles_spectra");
    if (st == QG_OK) e = cudaMemcpyAsync(g_host, dg, gb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess && st == QG_OK) st = qg_cuda_fail(ctx, e, "qg_poles_spectra");
  cudaStreamSynchronize(s);
  cudaFree(da);
  cudaFree(db);
  cudaFree(de0);
  cudaFree(dg);
  return st;
}
