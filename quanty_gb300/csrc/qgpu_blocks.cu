// Dense products of Krylov blocks, FP64 complex: the Gram products of the block eigensolver
// (C = V^H W, Core/BlockLanczos.cpp:5498-5527 forms them column by column), its projections
// and Ritz combinations (W -= V C, X = V Y, :5554-5573), and the Krylov combination of RIXS
// (a sum of stored Krylov vectors with the projected resolvent's coefficients,
// Core/ResonantSpectra.cpp:123-195).
//
// Blocks are tall and skinny (millions of rows, tens to hundreds of columns).  On GB300 FP64
// issues at 2 lanes per SM per clock, so these products are bound by the FP64 pipe long before
// shared memory or HBM: a complex multiply-add is 4 FMAs against two 16-byte shared-memory
// reads, which the shared memory serves 4x faster than the pipe consumes them.  Tiles are
// staged in shared memory and every thread keeps its outputs in registers; no atomics, and
// every sum runs in a fixed order, so results are bitwise reproducible.
//
// Layouts: row-major blocks (element (r, c) at r * ld + c); the second factor of a row product
// may be addressed with arbitrary row and column strides (the RIXS Krylov vectors are stored
// vector-major).
#include <algorithm>

#include "qgpu_internal.cuh"

#define QG_GT 16  // Gram tile edge (outputs per block: QG_GT x QG_GT)

// part[chunk][i * kb + j] = sum over the chunk's rows r of conj(A[r][i]) B[r][j].  REAL: both
// blocks are real (zero imaginary parts), one FMA per term instead of four.
template <bool REAL>
__global__ void __launch_bounds__(256) k_block_gram_part(const double2 *__restrict__ A, int lda, int ka,
                                                         const double2 *__restrict__ B, int ldb, int kb, int64_t n,
                                                         int64_t rows_per_chunk, double2 *__restrict__ part) {
  __shared__ double2 sa[QG_GT][QG_GT + 1], sb[QG_GT][QG_GT + 1];  // [row][column]
  const int tiles_j = (kb + QG_GT - 1) / QG_GT;
  const int i0 = (blockIdx.x / tiles_j) * QG_GT, j0 = (blockIdx.x % tiles_j) * QG_GT;
  const int tx = threadIdx.x % QG_GT, ty = threadIdx.x / QG_GT;
  const int64_t r0 = blockIdx.y * rows_per_chunk;
  const int64_t r1 = min(n, r0 + rows_per_chunk);
  double re = 0.0, im = 0.0;
  for (int64_t rb = r0; rb < r1; rb += QG_GT) {
    const int64_t r = rb + ty;
    sa[ty][tx] = (r < r1 && i0 + tx < ka) ? A[r * lda + i0 + tx] : make_double2(0.0, 0.0);
    sb[ty][tx] = (r < r1 && j0 + tx < kb) ? B[r * ldb + j0 + tx] : make_double2(0.0, 0.0);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < QG_GT; q++) {
      const double2 a = sa[q][ty], b = sb[q][tx];
      re = fma(a.x, b.x, re);
      if (!REAL) {
        re = fma(a.y, b.y, re);
        im = fma(a.x, b.y, im);
        im = fma(-a.y, b.x, im);
      }
    }
    __syncthreads();
  }
  if (i0 + ty < ka && j0 + tx < kb)
    part[(int64_t)blockIdx.y * ka * kb + (int64_t)(i0 + ty) * kb + j0 + tx] = make_double2(re, im);
}

// out[q] = sum over chunks c (in order) of part[c][q]
__global__ void k_block_gram_sum(const double2 *__restrict__ part, int nchunk, int m, double2 *__restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunk; c++) {
    const double2 v = part[(int64_t)c * m + q];
    re += v.x;
    im += v.y;
  }
  out[q] = make_double2(re, im);
}

// C (ka x kb, row-major) = A^H B over n rows; A: n x ka (ld lda), B: n x kb (ld ldb).  The rows
// are split into chunks whose partial tiles (in `work`, `work_elems` complex entries) are summed
// in chunk order.
qg_status qg_block_gram(qg_context ctx, const double2 *A, int lda, int ka, const double2 *B, int ldb, int kb,
                        int64_t n, double2 *C, double2 *work, int64_t work_elems, bool real) {
  if (ka <= 0 || kb <= 0) return QG_OK;
  const int64_t m = (int64_t)ka * kb;
  if (n <= 0) {
    QG_CUDA(ctx, cudaMemsetAsync(C, 0, (size_t)m * 16, ctx->stream));
    return QG_OK;
  }
  const int tiles = ((ka + QG_GT - 1) / QG_GT) * ((kb + QG_GT - 1) / QG_GT);
  // enough blocks for every SM several times over, each chunk a multiple of the tile height
  int64_t nchunk = std::max<int64_t>(1, (8LL * ctx->num_sms + tiles - 1) / tiles);
  nchunk = std::min<int64_t>(nchunk, std::max<int64_t>(1, n / (4 * QG_GT)));
  nchunk = std::min<int64_t>(nchunk, std::max<int64_t>(1, work_elems / m));
  nchunk = std::min<int64_t>(nchunk, 65535);
  if (work_elems < m) {
    ctx->last_error = "qg_block_gram: work buffer too small";
    return QG_ERR_ARG;
  }
  int64_t rows = (n + nchunk - 1) / nchunk;
  rows = (rows + QG_GT - 1) / QG_GT * QG_GT;
  nchunk = (n + rows - 1) / rows;
  if (real)
    k_block_gram_part<true><<<dim3((unsigned)tiles, (unsigned)nchunk), 256, 0, ctx->stream>>>(A, lda, ka, B, ldb, kb,
                                                                                              n, rows, work);
  else
    k_block_gram_part<false><<<dim3((unsigned)tiles, (unsigned)nchunk), 256, 0, ctx->stream>>>(A, lda, ka, B, ldb,
                                                                                               kb, n, rows, work);
  k_block_gram_sum<<<(unsigned)((m + 255) / 256), 256, 0, ctx->stream>>>(work, (int)nchunk, (int)m, C);
  ctx->launches += 2;
  return qg_check_launch(ctx, "qg_block_gram");
}

// X[r][j] = beta X[r][j] + alpha sum_i A(r, i) M[i][j] for the rows and columns of this block,
// A(r, i) = A[r * ars + i * acs].  JT columns per block, 256 / JT thread rows, 4 rows per
// thread; the factor tiles (IT values of i at a time) staged in shared memory.
template <int JT, bool REAL>
__global__ void __launch_bounds__(256) k_block_mul(const double2 *__restrict__ A, int64_t ars, int64_t acs, int ka,
                                                   const double2 *__restrict__ M, int ldm, double2 *__restrict__ X,
                                                   int ldx, int kb, int64_t n, double alpha, double beta) {
  constexpr int TY = 256 / JT, RT = 4 * TY, IT = 16;
  __shared__ double2 sa[IT][RT + 1];
  __shared__ double2 sm[IT][JT];
  const int tx = threadIdx.x % JT, ty = threadIdx.x / JT;
  const int64_t r0 = (int64_t)blockIdx.x * RT;
  const int j0 = blockIdx.y * JT;
  double2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; q++) acc[q] = make_double2(0.0, 0.0);
  for (int i0 = 0; i0 < ka; i0 += IT) {
    // the A tile: IT x RT values; walk the contiguous direction of A with consecutive threads
    for (int t = threadIdx.x; t < IT * RT; t += 256) {
      int ii, rr;
      if (acs == 1) {
        ii = t % IT;
        rr = t / IT;
      } else {
        rr = t % RT;
        ii = t / RT;
      }
      const int64_t r = r0 + rr;
      const int i = i0 + ii;
      sa[ii][rr] = (r < n && i < ka) ? A[r * ars + (int64_t)i * acs] : make_double2(0.0, 0.0);
    }
    for (int t = threadIdx.x; t < IT * JT; t += 256) {
      const int ii = t / JT, jj = t % JT;
      sm[ii][jj] = (i0 + ii < ka && j0 + jj < kb) ? M[(int64_t)(i0 + ii) * ldm + j0 + jj] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int ii = 0; ii < IT; ii++) {
      const double2 mv = sm[ii][tx];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const double2 a = sa[ii][ty + q * TY];
        acc[q].x = fma(a.x, mv.x, acc[q].x);
        if (!REAL) {
          acc[q].x = fma(-a.y, mv.y, acc[q].x);
          acc[q].y = fma(a.x, mv.y, acc[q].y);
          acc[q].y = fma(a.y, mv.x, acc[q].y);
        }
      }
    }
    __syncthreads();
  }
  const int j = j0 + tx;
  if (j >= kb) return;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int64_t r = r0 + ty + q * TY;
    if (r >= n) continue;
    double2 *o = X + r * ldx + j;
    double2 v = make_double2(alpha * acc[q].x, alpha * acc[q].y);
    if (beta != 0.0) {
      const double2 x = *o;
      v.x = fma(beta, x.x, v.x);
      v.y = fma(beta, x.y, v.y);
    }
    *o = v;
  }
}

template <bool REAL>
static void block_mul_t(qg_context ctx, const double2 *A, int64_t ars, int64_t acs, int ka, const double2 *M, int ldm,
                        double2 *X, int ldx, int kb, int64_t n, double alpha, double beta) {
  cudaStream_t s = ctx->stream;
  if (kb <= 8) {
    dim3 g((unsigned)((n + 127) / 128), (unsigned)((kb + 7) / 8));
    k_block_mul<8, REAL><<<g, 256, 0, s>>>(A, ars, acs, ka, M, ldm, X, ldx, kb, n, alpha, beta);
  } else if (kb <= 16) {
    dim3 g((unsigned)((n + 63) / 64), (unsigned)((kb + 15) / 16));
    k_block_mul<16, REAL><<<g, 256, 0, s>>>(A, ars, acs, ka, M, ldm, X, ldx, kb, n, alpha, beta);
  } else {
    dim3 g((unsigned)((n + 31) / 32), (unsigned)((kb + 31) / 32));
    k_block_mul<32, REAL><<<g, 256, 0, s>>>(A, ars, acs, ka, M, ldm, X, ldx, kb, n, alpha, beta);
  }
}

static qg_status block_mul(qg_context ctx, const double2 *A, int64_t ars, int64_t acs, int ka, const double2 *M,
                           int ldm, double2 *X, int ldx, int kb, int64_t n, double alpha, double beta,
                           bool real = false) {
  if (kb <= 0 || n <= 0) return QG_OK;
  if (real)
    block_mul_t<true>(ctx, A, ars, acs, ka, M, ldm, X, ldx, kb, n, alpha, beta);
  else
    block_mul_t<false>(ctx, A, ars, acs, ka, M, ldm, X, ldx, kb, n, alpha, beta);
  ctx->launches++;
  return qg_check_launch(ctx, "block product");
}

// X (n x kb, ld ldx) = beta X + alpha A M; A: n x ka (ld lda), M: ka x kb row-major (ld kb).
// ka == 0 leaves beta X (beta must then be 1: the solver never asks for a bare rescale).
qg_status qg_block_update(qg_context ctx, const double2 *A, int lda, int ka, const double2 *M, double2 *X, int ldx,
                          int kb, int64_t n, double alpha, double beta, bool real) {
  if (kb <= 0 || n <= 0) return QG_OK;
  if (ka <= 0) return beta == 1.0 ? QG_OK : QG_ERR_ARG;
  return block_mul(ctx, A, lda, 1, ka, M, kb, X, ldx, kb, n, alpha, beta, real);
}

// out (n x np row-major) = sum_i K_i C[i][:], the vectors K_i stored vector-major (K[i * n + r]).
qg_status qg_block_combine(qg_context ctx, const double2 *K, int64_t n, int ntri, const double2 *C, int np,
                           double2 *out) {
  if (n <= 0 || np <= 0) return QG_OK;
  if (ntri <= 0) {
    QG_CUDA(ctx, cudaMemsetAsync(out, 0, (size_t)n * np * 16, ctx->stream));
    return QG_OK;
  }
  return block_mul(ctx, K, 1, n, ntri, C, np, out, np, np, n, 1.0, 0.0);
}

extern "C" qg_status qg_krylov_combine(qg_context ctx, const double *K_dev, int64_t n, int32_t nk, const double *C_host,
                                       int32_t np, double *out_dev) {
  if (!ctx || n < 0 || nk < 0 || np <= 0 || (n > 0 && (!K_dev || !out_dev)) || (nk > 0 && !C_host)) return QG_ERR_ARG;
  if (n == 0) return QG_OK;
  double2 *Cd = nullptr;
  QG_CUDA(ctx, cudaMalloc(&Cd, (size_t)std::max(nk, 1) * np * 16));
  cudaError_t e = cudaMemcpyAsync(Cd, C_host, (size_t)nk * np * 16, cudaMemcpyHostToDevice, ctx->stream);
  qg_status st = e == cudaSuccess ? qg_block_combine(ctx, (const double2 *)K_dev, n, nk, Cd, np, (double2 *)out_dev)
                                  : qg_cuda_fail(ctx, e, "qg_krylov_combine");
  if (st == QG_OK) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_krylov_combine");
  }
  cudaFree(Cd);
  return st;
}

// ------------------------------------------------------------------ C ABI

// C (ka x kb row-major, device) = A^H B over n rows; A: n x ka (ld lda), B: n x kb (ld ldb).
extern "C" qg_status qg_block_adjoint_product(qg_context ctx, const double *A_dev, int32_t lda, int32_t ka,
                                              const double *B_dev, int32_t ldb, int32_t kb, int64_t n,
                                              double *C_dev) {
  if (!ctx || !A_dev || !B_dev || !C_dev || ka <= 0 || kb <= 0 || n < 0 || lda < ka || ldb < kb) return QG_ERR_ARG;
  const int64_t m = (int64_t)ka * kb;
  // partial tiles of up to 64 row chunks, at most 256 MB of them
  const int64_t work = std::max<int64_t>(m, std::min<int64_t>(64 * m, (256LL << 20) / 16));
  double2 *w = nullptr;
  QG_CUDA(ctx, cudaMalloc(&w, (size_t)work * 16));
  qg_status st = qg_block_gram(ctx, (const double2 *)A_dev, lda, ka, (const double2 *)B_dev, ldb, kb, n,
                               (double2 *)C_dev, w, work);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(w);
  return st;
}

// X (n x kb, ld ldx, device) = beta X + alpha A M; A: n x ka (ld lda), M: ka x kb row-major.
extern "C" qg_status qg_block_product(qg_context ctx, const double *A_dev, int32_t lda, int32_t ka, const double *M_dev,
                                      int32_t kb, int64_t n, double alpha, double beta, double *X_dev, int32_t ldx) {
  if (!ctx || !A_dev || !M_dev || !X_dev || ka <= 0 || kb <= 0 || n < 0 || lda < ka || ldx < kb) return QG_ERR_ARG;
  return qg_block_update(ctx, (const double2 *)A_dev, lda, ka, (const double2 *)M_dev, (double2 *)X_dev, ldx, kb, n,
                         alpha, beta);
}
