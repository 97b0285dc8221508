// Lowest eigenpairs of a Hermitian operator on a fixed basis: restarted block Lanczos with
// full (twice repeated) reorthogonalisation and Rayleigh-Ritz restarts.
//
// The reference's solver (BlockLanczosGroundStateConserveBasisKrylovComplex,
// Core/BlockLanczos.cpp:5350-5606) grows a block Krylov space with fixed-basis H*psi
// (:5489-5496), reorthogonalises twice against all Krylov vectors (:5498-5527), diagonalises
// the projected matrix with zheevd (:5530) and restarts from the Ritz vectors (:5554-5573)
// until the variance <H^2> - <H>^2 of every vector is below "Zero".  The same structure here:
// H*psi is the pull kernel, the Gram products and updates of whole blocks are plain complex
// products over the n x K Krylov block (row-major, K columns; qgpu_blocks.cu), single
// columns use the partial-sum kernels below, and the projected matrix (K <= a few hundred)
// is diagonalised on the device (cyclic Jacobi, qgpu_jacobi.cu), its lowest eigenvectors left
// in device memory for the Ritz combination.
//
// Block size: when more than three states are wanted, a few guard vectors join the block
// (up to half the wanted count, at most 8) and only the wanted states are tested for
// convergence, so a cluster of nearly degenerate states straddling the last wanted one does
// not stall the restarts.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <vector>

#include "qgpu_internal.cuh"

typedef std::complex<double> cd;

// C[i][j] partial = sum_rows conj(A[r][a0+i]) * B[r][b0+j]; thread per (i, j), gridDim.y row chunks
__global__ void k_gram_partial(const double2 *__restrict__ A, int lda, int a0, int ka, const double2 *__restrict__ B,
                               int ldb, int b0, int kb, int64_t n, int64_t chunk, double2 *part) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ka * kb) return;
  int i = q / kb, j = q % kb;  // row-major C[i * kb + j], the layout every consumer reads
  int64_t r0 = blockIdx.y * chunk, r1 = r0 + chunk;
  if (r1 > n) r1 = n;
  double sr = 0, si = 0;
  for (int64_t r = r0; r < r1; r++) {
    double2 a = A[r * lda + a0 + i], b = B[r * ldb + b0 + j];
    sr += a.x * b.x + a.y * b.y;
    si += a.x * b.y - a.y * b.x;
  }
  part[(int64_t)blockIdx.y * ka * kb + q] = make_double2(sr, si);
}

// Gram products against ONE column b (kb = 1): part[blk][i] = sum over the block's rows of
// conj(A[r][a0+i]) b[r].  With ka <= 8 a thread takes whole rows and keeps the ka sums in
// registers; with more columns a warp takes a row and its lanes take the columns (coalesced
// reads of the row).  Grid-stride over rows with many blocks, so the reduction is wide rather
// than a long serial walk per thread; sums are combined in a fixed order.
// REAL (also below): both sides are real, one multiply-add per term.
template <int KMAX, bool REAL>
__global__ void k_gram_col_rows(const double2 *__restrict__ A, int lda, int a0, int ka, const double2 *__restrict__ B,
                                int ldb, int b0, int64_t n, double2 *part) {
  __shared__ double2 sh[8][KMAX];
  double2 acc[KMAX];
#pragma unroll
  for (int i = 0; i < KMAX; i++) acc[i] = make_double2(0.0, 0.0);
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 b = B[r * ldb + b0];
#pragma unroll
    for (int i = 0; i < KMAX; i++) {
      if (i < ka) {
        double2 a = A[r * lda + a0 + i];
        if (REAL) {
          acc[i].x += a.x * b.x;
        } else {
          acc[i].x += a.x * b.x + a.y * b.y;
          acc[i].y += a.x * b.y - a.y * b.x;
        }
      }
    }
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < KMAX; i++) {
    double2 v = acc[i];
    for (int o = 16; o; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) sh[wid][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < ka) {
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      t.x += sh[w][threadIdx.x].x;
      t.y += sh[w][threadIdx.x].y;
    }
    part[(int64_t)blockIdx.x * ka + threadIdx.x] = t;
  }
}

#define QG_GRAM_LANE_COLS 8  // columns per lane at most: ka <= 256
template <int M, bool REAL>
__global__ void k_gram_col_lanes(const double2 *__restrict__ A, int lda, int a0, int ka,
                                 const double2 *__restrict__ B, int ldb, int b0, int64_t n, double2 *part) {
  __shared__ double2 sh[8][32 * M];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double2 acc[M];
#pragma unroll
  for (int m = 0; m < M; m++) acc[m] = make_double2(0.0, 0.0);
  for (int64_t r = (int64_t)blockIdx.x * nw + wid; r < n; r += (int64_t)gridDim.x * nw) {
    double2 b = B[r * ldb + b0];
#pragma unroll
    for (int m = 0; m < M; m++) {
      int i = lane + 32 * m;
      if (i < ka) {
        double2 a = A[r * lda + a0 + i];
        if (REAL) {
          acc[m].x += a.x * b.x;
        } else {
          acc[m].x += a.x * b.x + a.y * b.y;
          acc[m].y += a.x * b.y - a.y * b.x;
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < M; m++) sh[wid][lane + 32 * m] = acc[m];
  __syncthreads();
  for (int i = threadIdx.x; i < ka; i += blockDim.x) {
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < nw; w++) {
      t.x += sh[w][i].x;
      t.y += sh[w][i].y;
    }
    part[(int64_t)blockIdx.x * ka + i] = t;
  }
}

__global__ void k_gram_reduce(const double2 *part, int nchunk, int m, double2 *out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double sr = 0, si = 0;
  for (int c = 0; c < nchunk; c++) {
    sr += part[(int64_t)c * m + q].x;
    si += part[(int64_t)c * m + q].y;
  }
  out[q] = make_double2(sr, si);
}

// the same with a warp per output: lanes stride over the partials, then a shuffle tree
__global__ void k_gram_reduce_warp(const double2 *part, int nchunk, int m, double2 *out) {
  int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (q >= m) return;
  double sr = 0, si = 0;
  for (int c = lane; c < nchunk; c += 32) {
    sr += part[(int64_t)c * m + q].x;
    si += part[(int64_t)c * m + q].y;
  }
  for (int o = 16; o; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) out[q] = make_double2(sr, si);
}


// deterministic pseudo-random fill of columns c0 .. c0+k-1 (guard vectors); real entries for
// a real operator, so real start vectors keep the whole block, and the eigenvectors, real
__global__ void k_fill_cols(double2 *B, int ldb, int c0, int k, int64_t n, uint64_t salt, int real) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * k) return;
  int64_t r = i / k;
  int c = (int)(i % k);
  uint64_t h = qg_mix64((uint64_t)i * 0x9e3779b97f4a7c15ull + salt);
  double a = (double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  double b = (double)(qg_mix64(h) >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  B[r * ldb + c0 + c] = make_double2(a, real ? 0.0 : b);
}

// flag = 1 when any of the n values has a non-zero imaginary part (one global OR per block)
__global__ void k_any_imag(const double2 *__restrict__ v, int64_t n, unsigned int *flag) {
  int found = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n && !found;
       i += (int64_t)gridDim.x * blockDim.x)
    found = v[i].y != 0.0;
  if (__syncthreads_or(found) && threadIdx.x == 0) atomicOr(flag, 1u);
}

__global__ void k_copy_cols(const double2 *src, int lds, int s0, double2 *dst, int ldd, int d0, int k, int64_t n) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  int64_t r = t / k;
  int j = (int)(t % k);
  dst[r * ldd + d0 + j] = src[r * lds + s0 + j];
}

namespace {

struct Gram {
  qg_context ctx;
  int64_t n;
  double2 *part = nullptr, *out = nullptr;
  int64_t cap = 0, part_elems = 0;
  int nchunk = 1;
  int64_t chunk = 1;
  int nblk = 1;  // blocks of the one-column Gram kernels
  bool real = false;  // every vector real
  qg_status init(qg_context c, int64_t nn, int maxm, int kcol) {
    ctx = c;
    n = nn;
    chunk = std::max<int64_t>(4096, (nn + 1023) / 1024);
    nchunk = (int)((nn + chunk - 1) / chunk);
    if (nchunk < 1) nchunk = 1;
    nblk = (int)std::max<int64_t>(1, std::min<int64_t>(4LL * c->num_sms, (nn + 255) / 256));
    cap = maxm;
    // partial sums: one column against up to kcol columns (nchunk chunks, or nblk blocks of the
    // one-column kernels), or the row-chunk tiles of a block product (qg_block_gram uses as many
    // chunks as fit, at most the few dozen that fill the SMs)
    part_elems = std::max<int64_t>(std::max<int64_t>(nchunk * (int64_t)kcol, (int64_t)nblk * 32 * QG_GRAM_LANE_COLS), 16 * (int64_t)maxm);
    QG_CUDA(ctx, cudaMalloc(&part, (size_t)part_elems * 16));
    QG_CUDA(ctx, cudaMalloc(&out, (size_t)maxm * 16));
    return QG_OK;
  }
  void release() {
    cudaFree(part);
    cudaFree(out);
  }
  template <bool REAL>
  void col_gram(cudaStream_t s, const double2 *A, int lda, int a0, int ka, const double2 *B, int ldb, int b0) {
    if (ka == 1)
      k_gram_col_rows<1, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else if (ka <= 4)
      k_gram_col_rows<4, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else if (ka <= 8)
      k_gram_col_rows<8, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else if (ka <= 32)
      k_gram_col_lanes<1, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else if (ka <= 64)
      k_gram_col_lanes<2, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else if (ka <= 128)
      k_gram_col_lanes<4, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
    else
      k_gram_col_lanes<8, REAL><<<nblk, 256, 0, s>>>(A, lda, a0, ka, B, ldb, b0, n, part);
  }
  // out (device) and host = A[:, a0:a0+ka]^dag B[:, b0:b0+kb]
  qg_status run(const double2 *A, int lda, int a0, int ka, const double2 *B, int ldb, int b0, int kb,
                std::vector<cd> *host) {
    int m = ka * kb;
    if (m > cap || m <= 0) return QG_ERR_ARG;
    if (kb > 1) {  // a block against a block: tiled products, partial sums per row chunk
      QG_TRY(qg_block_gram(ctx, A + a0, lda, ka, B + b0, ldb, kb, n, out, part, part_elems, real));
    } else if (ka <= 32 * QG_GRAM_LANE_COLS) {  // one column: wide partial sums, fixed-order reduction
      cudaStream_t s = ctx->stream;
      if (real)
        col_gram<true>(s, A, lda, a0, ka, B, ldb, b0);
      else
        col_gram<false>(s, A, lda, a0, ka, B, ldb, b0);
      k_gram_reduce_warp<<<(m + 7) / 8, 256, 0, s>>>(part, nblk, m, out);
      ctx->launches += 2;
    } else {
      dim3 g((m + 127) / 128, nchunk);
      k_gram_partial<<<g, 128, 0, ctx->stream>>>(A, lda, a0, ka, B, ldb, b0, kb, n, chunk, part);
      k_gram_reduce<<<(m + 127) / 128, 128, 0, ctx->stream>>>(part, nchunk, m, out);
      ctx->launches += 2;
    }
    if (host) {
      host->resize(m);
      QG_CUDA(ctx, cudaMemcpyAsync(host->data(), out, m * 16, cudaMemcpyDeviceToHost, ctx->stream));
      QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return qg_check_launch(ctx, "gram");
  }
};

}  // namespace

extern "C" qg_status qg_block_groundstate(qg_context ctx, qg_operator op, qg_basis b, int32_t nwant, double *x_dev,
                                          double *energies_host, double tol, int32_t max_krylov,
                                          int32_t max_restarts, int32_t *iterations) {
  if (!ctx || !op || !b || !x_dev || !energies_host || nwant <= 0 || op->nf != b->nf) return QG_ERR_ARG;
  int64_t n = b->n;
  if (n < nwant) {
    ctx->last_error = "qg_block_groundstate: basis smaller than the number of states";
    return QG_ERR_ARG;
  }
  int guard = nwant > 3 ? std::min(nwant / 2, 8) : 0;
  int p = (int)std::min<int64_t>(nwant + guard, n);
  int K = max_krylov > 0 ? max_krylov : 128;
  if (K < 2 * p) K = 2 * p;
  if (K > n) K = (int)n;
  K = (K / p) * p;
  if (K < p) K = p;
  cudaStream_t s = ctx->stream;
  double2 *V = nullptr, *W = nullptr, *Cd = nullptr, *X = nullptr, *Md = nullptr, *Sd = nullptr;
  double *wd = nullptr;
  size_t vb = (size_t)n * K * 16, wb = (size_t)n * p * 16;
  cudaError_t e = cudaMalloc(&V, vb);
  if (e == cudaSuccess) e = cudaMalloc(&W, wb);
  if (e == cudaSuccess) e = cudaMalloc(&X, wb);
  if (e == cudaSuccess) e = cudaMalloc(&Cd, (size_t)K * std::max(K, p) * 16);
  if (e == cudaSuccess) e = cudaMalloc(&Md, (size_t)K * K * 16);
  if (e == cudaSuccess) e = cudaMalloc(&wd, (size_t)K * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&Sd, (size_t)p * p * 16);
  if (e != cudaSuccess) {
    cudaFree(V);
    cudaFree(W);
    cudaFree(X);
    cudaFree(Cd);
    cudaFree(Md);
    cudaFree(wd);
    cudaFree(Sd);
    ctx->last_error = "qg_block_groundstate: out of device memory";
    return QG_ERR_OOM;
  }
  auto grid = [](int64_t t) { return (unsigned)((t + 255) / 256); };
  // the block: the caller's start vectors, then the guard vectors
  k_copy_cols<<<grid(n * nwant), 256, 0, s>>>((const double2 *)x_dev, nwant, 0, X, p, 0, nwant, n);
  ctx->launches++;
  if (p > nwant) {
    k_fill_cols<<<grid(n * (p - nwant)), 256, 0, s>>>(X, p, nwant, p - nwant, n, 0x5eedull,
                                                      qg_operator_values_real(op) ? 1 : 0);
    ctx->launches++;
  }
  Gram G;
  qg_status st = G.init(ctx, n, K * std::max(K, p), K);
  // a real operator with real start vectors keeps every vector, every projection and the Ritz
  // vectors real (the reference's real-vector solver): the block products then run in real
  // arithmetic, one FMA per term instead of four
  if (st == QG_OK && qg_operator_values_real(op)) {
    unsigned int *d_im = nullptr, h_im = 1;
    e = cudaMalloc(&d_im, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_im, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) {
      k_any_imag<<<(unsigned)std::min<int64_t>((n * p + 255) / 256, 4LL * ctx->num_sms), 256, 0, s>>>(X, n * p, d_im);
      ctx->launches++;
      e = cudaMemcpyAsync(&h_im, d_im, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_im);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_block_groundstate");
    G.real = h_im == 0;
  }
  std::vector<double> theta(p, 0.0);
  int it = 0;
  bool converged = false;
  std::vector<cd> c, T;
  // Krylov dimension per restart: starts at p + 100 and grows by p + 10 per restart up to K
  // (the reference's NKrylovStart / NKrylovStep schedule, Core/BlockLanczos.cpp:5130, :5311)
  int Kcur = std::min(K, std::max(2 * p, ((p + 100) / p) * p));
  for (int restart = 0; restart <= max_restarts && st == QG_OK && !converged; restart++) {
    if (restart > 0) Kcur = std::min(K, ((Kcur + p + 10) / p) * p);
    // V[:, 0:p] = X, orthonormalised (modified Gram-Schmidt, twice)
    k_copy_cols<<<grid(n * p), 256, 0, s>>>(X, p, 0, V, K, 0, p, n);
    ctx->launches++;
    int k = 0;  // orthonormal columns in V
    T.assign((size_t)K * K, cd(0, 0));
    // Loewdin orthonormalisation of the ka columns of A (ld lda): the eigenvectors U and values
    // s^2 of the Gram matrix A^H A; directions with s at most 1e-10 of the largest are dropped.
    // Sm (ka x kk row-major) makes Q = A Sm orthonormal and Rm (kk x ka) gives A = Q Rm on the
    // kept span; *cond gets the smallest kept s over the largest.  Returns kk.
    auto lowdin_pass = [&](const double2 *A, int lda, int ka, std::vector<cd> &Sm, std::vector<cd> &Rm,
                           double *cond) -> int {
      std::vector<cd> Gh;
      st = G.run(A, lda, 0, ka, A, lda, 0, ka, &Gh);
      if (st != QG_OK) return 0;
      for (int r = 0; r < ka; r++)
        for (int c = r; c < ka; c++) {
          const cd h = 0.5 * (Gh[(size_t)r * ka + c] + std::conj(Gh[(size_t)c * ka + r]));
          Gh[(size_t)r * ka + c] = h;
          Gh[(size_t)c * ka + r] = std::conj(h);
        }
      std::vector<double> w(ka);
      std::vector<cd> U((size_t)ka * ka);
      st = qg_eigh_host_io(ctx, ka, (const double *)Gh.data(), w.data(), (double *)U.data(), ka);
      if (st != QG_OK) return 0;
      const double smax = std::sqrt(std::max(w[ka - 1], 0.0));
      std::vector<int> keep;
      for (int q = ka - 1; q >= 0; q--)
        if (smax > 0.0 && std::sqrt(std::max(w[q], 0.0)) > 1e-10 * smax) keep.push_back(q);
      const int kk = (int)keep.size();
      *cond = kk ? std::sqrt(std::max(w[keep[kk - 1]], 0.0)) / smax : 0.0;
      Sm.assign((size_t)ka * std::max(kk, 1), cd(0, 0));
      Rm.assign((size_t)std::max(kk, 1) * ka, cd(0, 0));
      for (int c = 0; c < kk; c++) {
        const double sv = std::sqrt(w[keep[c]]);
        for (int r = 0; r < ka; r++) {
          const cd u = U[(size_t)r * ka + keep[c]];
          Sm[(size_t)r * kk + c] = u / sv;
          Rm[(size_t)c * ka + r] = sv * std::conj(u);
        }
      }
      return kk;
    };
    // orthonormalise V[:, c0:c0+cnt] with Loewdin inside the block, twice.  The block has already
    // been projected twice against V[:, 0:c0] as a whole, which stays enough unless the block
    // is nearly dependent: when the first pass's smallest kept s is below a tenth of the largest
    // (its 1/s scaling amplifies what the projections left), the result is projected against
    // V[:, 0:c0] once more before the second pass.  The result lands in V[:, c0:c0+kept].
    // coef (c0 + cnt rows x cnt) gets R with W_j = sum_i V_i R[i][j] over old and new columns.
    auto orth_block = [&](int c0, int cnt, std::vector<cd> *coef) -> int {
      std::vector<cd> S1, R1, S2, R2, Ch;
      double cond1 = 0.0, cond2 = 0.0;
      const int k1 = lowdin_pass(V + c0, K, cnt, S1, R1, &cond1);
      if (st != QG_OK || k1 == 0) return 0;
      cudaError_t ce = cudaMemcpyAsync(Sd, S1.data(), S1.size() * 16, cudaMemcpyHostToDevice, s);
      if (ce != cudaSuccess) {
        st = qg_cuda_fail(ctx, ce, "block orthonormalisation");
        return 0;
      }
      st = qg_block_update(ctx, V + c0, K, cnt, Sd, W, p, k1, n, 1.0, 0.0, G.real);  // Q1 = V_b S1
      if (st != QG_OK) return 0;
      if (c0 > 0 && cond1 < 0.1) {  // Q1 -= V_old (V_old^H Q1)
        st = G.run(V, K, 0, c0, W, p, 0, k1, &Ch);
        if (st == QG_OK) st = qg_block_update(ctx, V, K, c0, G.out, W, p, k1, n, -1.0, 1.0, G.real);
        if (st != QG_OK) return 0;
      }
      const int k2 = lowdin_pass(W, p, k1, S2, R2, &cond2);
      if (st != QG_OK || k2 == 0) return 0;
      ce = cudaMemcpyAsync(Sd, S2.data(), S2.size() * 16, cudaMemcpyHostToDevice, s);
      if (ce != cudaSuccess) {
        st = qg_cuda_fail(ctx, ce, "block orthonormalisation");
        return 0;
      }
      st = qg_block_update(ctx, W, p, k1, Sd, V + c0, K, k2, n, 1.0, 0.0, G.real);  // Q2 = Q1 S2
      if (st != QG_OK) return 0;
      if (coef) {
        for (int i = 0; i < k2; i++)  // new columns: R2 R1
          for (int j = 0; j < cnt; j++) {
            cd a(0, 0);
            for (int t = 0; t < k1; t++) a += R2[(size_t)i * k1 + t] * R1[(size_t)t * cnt + j];
            (*coef)[(size_t)(c0 + i) * cnt + j] = a;
          }
        for (int i = 0; i < c0 && !Ch.empty(); i++)  // old columns: C R1
          for (int j = 0; j < cnt; j++) {
            cd a(0, 0);
            for (int t = 0; t < k1; t++) a += Ch[(size_t)i * k1 + t] * R1[(size_t)t * cnt + j];
            (*coef)[(size_t)i * cnt + j] += a;
          }
      }
      return k2;
    };
    k = orth_block(0, p, nullptr);
    if (st != QG_OK) break;
    if (k == 0) {
      ctx->last_error = "qg_block_groundstate: start vectors are zero";
      st = QG_ERR_ARG;
      break;
    }
    int j0 = 0, bs = k;
    while (st == QG_OK) {
      // W = H V[:, j0:j0+bs]
      st = qg_apply_strided(ctx, op, b, b, (const double *)(V + j0), K, (double *)W, p, bs, nullptr);
      it++;
      if (st != QG_OK) break;
      // T[0:k, j0:j0+bs] = V^dag W (twice, the second pass corrects), W -= V C
      for (int pass = 0; pass < 2 && st == QG_OK; pass++) {
        st = G.run(V, K, 0, k, W, p, 0, bs, &c);
        if (st != QG_OK) break;
        for (int i = 0; i < k; i++)
          for (int j = 0; j < bs; j++) T[(size_t)i * K + j0 + j] += c[(size_t)i * bs + j];
        st = qg_block_update(ctx, V, K, k, G.out, W, p, bs, n, -1.0, 1.0, G.real);
      }
      if (st != QG_OK || k + bs > Kcur) break;
      // append W as new columns and orthonormalise them
      k_copy_cols<<<grid(n * bs), 256, 0, s>>>(W, p, 0, V, K, k, bs, n);
      ctx->launches++;
      std::vector<cd> R((size_t)(k + bs) * bs, cd(0, 0));
      int kept = orth_block(k, bs, &R);
      if (st != QG_OK) break;
      // H V_j has components R on the new columns (and small corrections on old ones)
      for (int i = 0; i < kept; i++)
        for (int j = 0; j < bs; j++) T[(size_t)(k + i) * K + j0 + j] += R[(size_t)(k + i) * bs + j];
      for (int i = 0; i < k; i++)
        for (int j = 0; j < bs; j++) T[(size_t)i * K + j0 + j] += R[(size_t)i * bs + j];
      if (kept == 0) break;  // the block Krylov space is invariant: the projection is exact
      j0 = k;
      k += kept;
      bs = kept;
      if (k + bs > Kcur) {
        // last block: its projections are needed for the Rayleigh quotient
        st = qg_apply_strided(ctx, op, b, b, (const double *)(V + j0), K, (double *)W, p, bs, nullptr);
        it++;
        if (st == QG_OK) st = G.run(V, K, 0, k, W, p, 0, bs, &c);
        if (st == QG_OK)
          for (int i = 0; i < k; i++)
            for (int j = 0; j < bs; j++) T[(size_t)i * K + j0 + j] = c[(size_t)i * bs + j];
        break;
      }
    }
    if (st != QG_OK) break;
    // projected matrix: Hermitian part of the k x k leading block
    std::vector<cd> M((size_t)k * k);
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++) {
        cd a = T[(size_t)i * K + j], bb = std::conj(T[(size_t)j * K + i]);
        // entries above the computed block columns are only known through symmetry
        M[(size_t)i * k + j] = (a == cd(0, 0)) ? bb : ((bb == cd(0, 0)) ? a : 0.5 * (a + bb));
      }
    // Ritz pairs on the device: the lowest p eigenvectors of M straight into Cd (k x p)
    const int nv = std::min(p, k);
    e = cudaMemcpyAsync(Md, M.data(), M.size() * 16, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nv < p) e = cudaMemsetAsync(Cd, 0, (size_t)k * p * 16, s);
    if (e != cudaSuccess) {
      st = qg_cuda_fail(ctx, e, "projected matrix upload");
      break;
    }
    st = qg_eigh_device(ctx, k, Md, wd, Cd, nv);
    if (st != QG_OK) break;
    if (nv < p) {  // eigenvectors packed k x nv; spread them to k x p (the remaining columns stay zero)
      std::vector<cd> Yp((size_t)k * nv), Yw((size_t)k * p, cd(0, 0));
      e = cudaMemcpyAsync(Yp.data(), Cd, Yp.size() * 16, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      for (int i = 0; i < k && e == cudaSuccess; i++)
        for (int j = 0; j < nv; j++) Yw[(size_t)i * p + j] = Yp[(size_t)i * nv + j];
      if (e == cudaSuccess) e = cudaMemcpyAsync(Cd, Yw.data(), Yw.size() * 16, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) {
        st = qg_cuda_fail(ctx, e, "ritz vectors");
        break;
      }
    }
    st = qg_block_update(ctx, V, K, k, Cd, X, p, p, n, 1.0, 0.0, G.real);
    if (st != QG_OK) break;
    std::vector<double> w(nv);
    e = cudaMemcpyAsync(w.data(), wd, (size_t)nv * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      st = qg_cuda_fail(ctx, e, "ritz values");
      break;
    }
    for (int j = 0; j < p; j++) theta[j] = j < nv ? w[j] : 0.0;
    // convergence: variance <(H - theta)^2> = |H x - theta x|^2 per vector, formed from the
    // residual itself (no cancellation between <H^2> and <H>^2)
    st = qg_apply_strided(ctx, op, b, b, (const double *)X, p, (double *)W, p, p, nullptr);
    it++;
    if (st != QG_OK) break;
    {
      std::vector<cd> th((size_t)p * p, cd(0, 0));
      for (int j = 0; j < p; j++) th[(size_t)j * p + j] = theta[j];
      e = cudaMemcpyAsync(Cd, th.data(), th.size() * 16, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) {
        st = qg_cuda_fail(ctx, e, "residual");
        break;
      }
      st = qg_block_update(ctx, X, p, p, Cd, W, p, p, n, -1.0, 1.0, G.real);
      if (st != QG_OK) break;
    }
    std::vector<cd> hh;
    double worst = 0;
    for (int j = 0; j < nwant && st == QG_OK; j++) {
      st = G.run(W, p, j, 1, W, p, j, 1, &hh);
      if (st != QG_OK) break;
      worst = std::max(worst, std::fabs(hh[0].real()));
    }
    if (worst < tol) converged = true;
  }
  G.release();
  if (st == QG_OK) {
    k_copy_cols<<<grid(n * nwant), 256, 0, s>>>(X, p, 0, (double2 *)x_dev, nwant, 0, nwant, n);
    ctx->launches++;
  }
  cudaStreamSynchronize(s);
  cudaFree(V);
  cudaFree(W);
  cudaFree(X);
  cudaFree(Cd);
  cudaFree(Md);
  cudaFree(wd);
  cudaFree(Sd);
  for (int j = 0; j < nwant; j++) energies_host[j] = theta[j];
  if (iterations) *iterations = it;
  if (st == QG_OK) st = qg_check_device_error(ctx, "qg_block_groundstate");
  if (st == QG_OK && !converged) {
    ctx->last_error = "qg_block_groundstate: not converged within the restart limit";
    return QG_ERR_TIMEOUT;
  }
  return st;
}
