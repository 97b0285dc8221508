// Block Lanczos tridiagonalisation for tensor spectra: the block Krylov space of m start vectors
// under H, reduced to a block tridiagonal matrix (LanczosBlockTriDiagonalize{RR,RC,CC,...},
// Core/BlockLanczos.cpp:1647-2660, called by CreateSpectra with Tensor = true,
// LuaInterface/ssp.cpp:2753-2800), and the m x m matrix of spectra from it by the block continued
// fraction (BlockTriDiagonalMatrixToSpectraWithBroadening,
// Core/BasicMathBlock/BasicMath_BlockTypeConversion.cpp:1636).
//
// The recursion, with Q_k the k-th orthonormal block (n x m_k, device, row-major, ld m):
//   Q_1 C_0 = V_0                                (Loewdin orthonormalisation, twice)
//   W = H Q_k;  A_k = Q_k^H W;  B_{k-1} = Q_{k-1}^H W
//   W -= Q_k (Q_k^H W) and Q_{k-1} (Q_{k-1}^H W), in the reference's order of six passes
//   Q_{k+1} = Loewdin(W) (twice), then entries with |a| < epsilon are zeroed
// with the reference's deflation: a direction of the overlap whose singular value is not above
// max(SingularValue, 3 sqrt(DBL_EPSILON) s_max) is dropped, so m_{k+1} <= m_k, and a block that
// deflates to nothing ends the recursion (the remaining blocks are zero).  The Loewdin transform
// is the symmetric one, X = U diag(1/s) U^H on the kept directions, as the reference's
// (ComplexWaveFunctionListSVDOrthogonalizeOnce, Core/ComplexWaveFunctionArithmetic.cpp:1600ff).
// Every product over the basis runs on the device (multi-vector H*psi, block Gram and update
// kernels, qgpu_blocks.cu; the m x m eigenproblems on the device Jacobi, qgpu_jacobi.cu); only
// the m x m coefficient matrices are assembled on the host.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <vector>

#include "qgpu_internal.cuh"

typedef std::complex<double> cd;

__global__ void k_block_trunc(double2 *v, int ld, int k, int64_t n, double eps2) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  const int64_t r = t / k;
  const int c = (int)(t % k);
  double2 *p = v + r * ld + c;
  const double2 a = *p;
  if (a.x * a.x + a.y * a.y < eps2) *p = make_double2(0.0, 0.0);
}

// the orthonormal block Q (n x m row-major, k live columns) as Krylov vectors k0 .. k0+m-1,
// vector-major (K[(k0 + c) * n + r]), the columns beyond k zero
__global__ void k_store_block(const double2 *__restrict__ Q, int m, int k, int64_t n, double2 *__restrict__ K,
                              int64_t k0) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n * m) return;
  const int c = (int)(t / n);
  const int64_t r = t % n;
  K[(k0 + c) * n + r] = c < k ? Q[r * m + c] : make_double2(0.0, 0.0);
}

namespace {

struct BlockCtx {
  qg_context ctx;
  int64_t n;
  int m;
  double2 *work = nullptr, *C = nullptr;  // Gram partials; a device m x m coefficient matrix
  int64_t work_elems = 0;
  double sv;

  // host copy of X^H Y (kx x ky) for blocks of ld m
  qg_status gram(const double2 *X, int kx, const double2 *Y, int ky, std::vector<cd> &out) {
    QG_TRY(qg_block_gram(ctx, X, m, kx, Y, m, ky, n, C, work, work_elems));
    out.resize((size_t)kx * ky);
    QG_CUDA(ctx, cudaMemcpyAsync(out.data(), C, out.size() * 16, cudaMemcpyDeviceToHost, ctx->stream));
    QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QG_OK;
  }

  // Y[:, 0:ky] -= X[:, 0:kx] (X^H Y)
  qg_status project(const double2 *X, int kx, double2 *Y, int ky) {
    if (kx <= 0 || ky <= 0) return QG_OK;
    QG_TRY(qg_block_gram(ctx, X, m, kx, Y, m, ky, n, C, work, work_elems));
    return qg_block_update(ctx, X, m, kx, C, Y, m, ky, n, -1.0, 1.0);
  }

  // One Loewdin pass: V (k columns) -> out (k' columns) = V X, X = U diag(1/s) U^H when every
  // direction is kept, U_kept diag(1/s) (k x k') when some are dropped; returns k'.  reduce =
  // false keeps every direction (the second pass).
  qg_status lowdin_once(const double2 *V, int k, double2 *out, bool reduce, int *kout) {
    std::vector<cd> S;
    QG_TRY(gram(V, k, V, k, S));
    for (int i = 0; i < k; i++)  // exactly Hermitian
      for (int j = 0; j < i; j++) {
        cd h = 0.5 * (S[(size_t)i * k + j] + std::conj(S[(size_t)j * k + i]));
        S[(size_t)i * k + j] = h;
        S[(size_t)j * k + i] = std::conj(h);
      }
    std::vector<double> w(k);
    std::vector<cd> U((size_t)k * k);
    QG_TRY(qg_eigh_host_io(ctx, k, (const double *)S.data(), w.data(), (double *)U.data(), k));
    double smax = 0.0;
    std::vector<double> s(k);
    for (int i = 0; i < k; i++) {
      s[i] = std::sqrt(std::max(0.0, w[i]));
      smax = std::max(smax, s[i]);
    }
    const double zero = std::max(sv, 3.0 * std::sqrt(DBL_EPSILON) * smax);
    std::vector<int> keep;
    for (int i = 0; i < k; i++)
      if ((!reduce && s[i] > 0.0) || s[i] > zero) keep.push_back(i);
    const int kp = (int)keep.size();
    *kout = kp;
    if (kp == 0) return QG_OK;
    std::vector<cd> X((size_t)k * kp, cd(0, 0));
    if (kp == k) {  // symmetric: X = U diag(1/s) U^H
      for (int r = 0; r < k; r++)
        for (int c = 0; c < k; c++) {
          cd t = 0;
          for (int q = 0; q < k; q++) t += U[(size_t)r * k + q] * (1.0 / s[q]) * std::conj(U[(size_t)c * k + q]);
          X[(size_t)r * k + c] = t;
        }
    } else {
      for (int r = 0; r < k; r++)
        for (int c = 0; c < kp; c++) X[(size_t)r * kp + c] = U[(size_t)r * k + keep[c]] * (1.0 / s[keep[c]]);
    }
    QG_CUDA(ctx, cudaMemcpyAsync(C, X.data(), X.size() * 16, cudaMemcpyHostToDevice, ctx->stream));
    return qg_block_update(ctx, V, m, k, C, out, m, kp, n, 1.0, 0.0);
  }

  // Loewdin twice (the second pass restores orthonormality to rounding), V -> out
  qg_status lowdin(const double2 *V, int k, double2 *out, double2 *tmp, int *kout) {
    int k1 = 0, k2 = 0;
    QG_TRY(lowdin_once(V, k, tmp, true, &k1));
    *kout = k1;
    if (k1 == 0) return QG_OK;
    QG_TRY(lowdin_once(tmp, k1, out, false, &k2));
    *kout = k2;
    return QG_OK;
  }
};

}  // namespace

extern "C" qg_status qg_block_lanczos(qg_context ctx, qg_operator op, qg_basis b, const double *v0_dev, int32_t m,
                                      int32_t ntri, double eps, double singular_value, double *a_host, double *b_host,
                                      int32_t *sizes_host, double *krylov_dev) {
  if (!ctx || !op || !b || !v0_dev || m <= 0 || ntri <= 0 || !a_host || !b_host || !sizes_host || op->nf != b->nf)
    return QG_ERR_ARG;
  const int64_t n = b->n;
  const size_t mm = (size_t)m * m;
  std::vector<cd> A((size_t)(ntri + 1) * mm, cd(0, 0)), B((size_t)ntri * mm, cd(0, 0));
  std::vector<int32_t> sizes(ntri + 1, 0);
  sizes[0] = m;
  if (n == 0) {
    std::copy(A.begin(), A.end(), (cd *)a_host);
    std::copy(B.begin(), B.end(), (cd *)b_host);
    std::copy(sizes.begin(), sizes.end(), sizes_host);
    return QG_OK;
  }
  cudaStream_t s = ctx->stream;
  BlockCtx bc;
  bc.ctx = ctx;
  bc.n = n;
  bc.m = m;
  bc.sv = singular_value;
  double2 *Qp = nullptr, *Q = nullptr, *W = nullptr, *T = nullptr;
  const size_t vb = (size_t)n * m * 16;
  bc.work_elems = std::max<int64_t>(64 * (int64_t)mm, 1 << 16);
  cudaError_t e = cudaMalloc(&Qp, vb);
  if (e == cudaSuccess) e = cudaMalloc(&Q, vb);
  if (e == cudaSuccess) e = cudaMalloc(&W, vb);
  if (e == cudaSuccess) e = cudaMalloc(&T, vb);
  if (e == cudaSuccess) e = cudaMalloc(&bc.work, (size_t)bc.work_elems * 16);
  if (e == cudaSuccess) e = cudaMalloc(&bc.C, mm * 16);
  qg_status st = e == cudaSuccess ? QG_OK : QG_ERR_OOM;
  if (st != QG_OK) ctx->last_error = "qg_block_lanczos: out of device memory";
  if (st == QG_OK) {
    e = cudaMemsetAsync(Qp, 0, vb, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(Q, 0, vb, s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_block_lanczos");
  }
  // Q_1 C_0 = V_0; b_0(i, j) = <q_j | v0_i>
  int k = 0, kprev = 0;
  std::vector<cd> G;
  if (st == QG_OK) st = bc.lowdin((const double2 *)v0_dev, m, Q, T, &k);
  if (st == QG_OK && k > 0) st = bc.gram(Q, k, (const double2 *)v0_dev, m, G);
  if (st == QG_OK)
    for (int i = 0; i < m; i++)
      for (int j = 0; j < k; j++) B[(size_t)i * m + j] = G[(size_t)j * m + i];
  if (st == QG_OK) sizes[1] = k;
  const double eps2 = eps * eps;
  if (st == QG_OK && krylov_dev) {  // every block is written, deflated ones as zeros
    e = cudaMemsetAsync(krylov_dev, 0, (size_t)ntri * m * n * 16, s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_block_lanczos");
  }
  for (int it = 1; st == QG_OK && k > 0 && it <= ntri; it++) {
    if (krylov_dev) {
      k_store_block<<<(unsigned)((n * m + 255) / 256), 256, 0, s>>>(Q, m, k, n, (double2 *)krylov_dev,
                                                                    (int64_t)(it - 1) * m);
      ctx->launches++;
    }
    // W = H Q_it
    st = qg_apply_strided(ctx, op, b, b, (const double *)Q, m, (double *)W, m, k, nullptr);
    if (st != QG_OK) break;
    st = bc.gram(Q, k, W, k, G);  // A_it
    if (st != QG_OK) break;
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++) A[(size_t)it * mm + (size_t)i * m + j] = G[(size_t)i * k + j];
    if (it > 1) {
      st = bc.gram(Qp, kprev, W, k, G);  // B_{it-1}
      if (st != QG_OK) break;
      for (int i = 0; i < kprev; i++)
        for (int j = 0; j < k; j++) B[(size_t)(it - 1) * mm + (size_t)i * m + j] = G[(size_t)i * k + j];
    }
    if (it == ntri) break;  // the last block: its coefficients are all that is needed
    // orthogonalise W against Q_it and Q_{it-1}: Q, Q, Qp, Qp, Q, Qp
    const int kp = it > 1 ? kprev : 0;
    for (int pass = 0; pass < 6 && st == QG_OK; pass++) {
      const bool cur = pass == 0 || pass == 1 || pass == 4;
      st = cur ? bc.project(Q, k, W, k) : bc.project(Qp, kp, W, k);
    }
    if (st != QG_OK) break;
    int knew = 0;
    st = bc.lowdin(W, k, T, Qp, &knew);  // Q_{it-1} is no longer needed: its buffer is scratch
    if (st != QG_OK) break;
    if (knew > 0 && eps2 > 0.0) {
      k_block_trunc<<<(unsigned)((n * knew + 255) / 256), 256, 0, s>>>(T, m, knew, n, eps2);
      ctx->launches++;
      st = qg_check_launch(ctx, "qg_block_lanczos");
    }
    if (it + 1 <= ntri) sizes[it + 1] = knew;
    // rotate: Qp <- Q_it, Q <- Q_{it+1}
    std::swap(Qp, Q);
    std::swap(Q, T);
    kprev = k;
    k = knew;
  }
  if (st == QG_OK) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_block_lanczos");
  }
  cudaFree(Qp);
  cudaFree(Q);
  cudaFree(W);
  cudaFree(T);
  cudaFree(bc.work);
  cudaFree(bc.C);
  if (st != QG_OK) return st;
  std::copy(A.begin(), A.end(), (cd *)a_host);
  std::copy(B.begin(), B.end(), (cd *)b_host);
  std::copy(sizes.begin(), sizes.end(), sizes_host);
  return qg_check_device_error(ctx, "qg_block_lanczos");
}

// ------------------------------------------------------------------ block continued fraction

#define QG_BCF_MAXM 8

// in-place inverse of an m x m complex matrix (Gauss-Jordan, partial pivoting)
__device__ void bcf_inverse(double2 *M, int m) {
  double2 I[QG_BCF_MAXM * QG_BCF_MAXM];
  for (int i = 0; i < m * m; i++) I[i] = make_double2((i / m) == (i % m) ? 1.0 : 0.0, 0.0);
  for (int c = 0; c < m; c++) {
    int p = c;
    double best = -1.0;
    for (int r = c; r < m; r++) {
      const double a = M[r * m + c].x * M[r * m + c].x + M[r * m + c].y * M[r * m + c].y;
      if (a > best) {
        best = a;
        p = r;
      }
    }
    if (p != c)
      for (int j = 0; j < m; j++) {
        double2 t = M[c * m + j];
        M[c * m + j] = M[p * m + j];
        M[p * m + j] = t;
        t = I[c * m + j];
        I[c * m + j] = I[p * m + j];
        I[p * m + j] = t;
      }
    const double2 d = M[c * m + c];
    const double dn = d.x * d.x + d.y * d.y;
    const double2 inv = make_double2(d.x / dn, -d.y / dn);
    for (int j = 0; j < m; j++) {
      const double2 a = M[c * m + j], b = I[c * m + j];
      M[c * m + j] = make_double2(a.x * inv.x - a.y * inv.y, a.x * inv.y + a.y * inv.x);
      I[c * m + j] = make_double2(b.x * inv.x - b.y * inv.y, b.x * inv.y + b.y * inv.x);
    }
    for (int r = 0; r < m; r++) {
      if (r == c) continue;
      const double2 f = M[r * m + c];
      for (int j = 0; j < m; j++) {
        const double2 a = M[c * m + j], b = I[c * m + j];
        M[r * m + j].x -= f.x * a.x - f.y * a.y;
        M[r * m + j].y -= f.x * a.y + f.y * a.x;
        I[r * m + j].x -= f.x * b.x - f.y * b.y;
        I[r * m + j].y -= f.x * b.y + f.y * b.x;
      }
    }
  }
  for (int i = 0; i < m * m; i++) M[i] = I[i];
}

// G(w) = conj(b_0) [w - A_1 + i g/2 - B_1 [w - A_2 + i g/2 - ...]^-1 B_1^H]^-1 b_0^T at
// w = emin + k de + e0, one thread per frequency, from the bottom block up (the reference's
// order, Core/BasicMathBlock/BasicMath_BlockTypeConversion.cpp:1666-1700); g[(i*m + j)*(ne+1) + k].
__global__ void k_block_cf(int m, int nblk, const double2 *__restrict__ a, const double2 *__restrict__ b, double e0,
                           double emin, double de, int ne, double gamma, double2 *__restrict__ g) {
  const int kf = blockIdx.x * blockDim.x + threadIdx.x;
  if (kf > ne) return;
  const double w = emin + kf * de + e0;
  const int mm = m * m;
  double2 G[QG_BCF_MAXM * QG_BCF_MAXM], T[QG_BCF_MAXM * QG_BCF_MAXM];
  for (int i = 0; i < mm; i++) G[i] = make_double2(0.0, 0.0);
  for (int blk = nblk; blk >= 1; blk--) {
    const double2 *A = a + (size_t)blk * mm;
    for (int i = 0; i < mm; i++) {
      G[i].x = -(G[i].x + A[i].x);
      G[i].y = -(G[i].y + A[i].y);
    }
    for (int i = 0; i < m; i++) {
      G[i * m + i].x += w;
      G[i * m + i].y += 0.5 * gamma;
    }
    bcf_inverse(G, m);
    const double2 *Bm = b + (size_t)(blk - 1) * mm;
    // T = B G (conj(b_0) G for the first block)
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < m; q++) {
          double2 bb = Bm[i * m + q];
          if (blk == 1) bb.y = -bb.y;
          const double2 gg = G[q * m + j];
          t.x += bb.x * gg.x - bb.y * gg.y;
          t.y += bb.x * gg.y + bb.y * gg.x;
        }
        T[i * m + j] = t;
      }
    // G = T B^H for the inner blocks, T b_0^T for the first: (B^H)[q][j] = conj(B[j][q]),
    // (b_0^T)[q][j] = b_0[j][q]
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < m; q++) {
          double2 bb = Bm[j * m + q];
          if (blk != 1) bb.y = -bb.y;
          const double2 tt = T[i * m + q];
          t.x += tt.x * bb.x - tt.y * bb.y;
          t.y += tt.x * bb.y + tt.y * bb.x;
        }
        G[i * m + j] = t;
      }
  }
  for (int i = 0; i < mm; i++) g[(size_t)i * (ne + 1) + kf] = G[i];
}

extern "C" qg_status qg_block_cf_spectra(qg_context ctx, int32_t m, int32_t ntri, const double *a_host,
                                         const double *b_host, double e0, double emin, double de, int32_t ne,
                                         double gamma, double *g_host) {
  if (!ctx || m <= 0 || m > QG_BCF_MAXM || ntri <= 0 || ne < 0 || !a_host || !b_host || !g_host) return QG_ERR_ARG;
  const size_t mm = (size_t)m * m;
  double2 *a = nullptr, *b = nullptr, *g = nullptr;
  const size_t ab = (size_t)(ntri + 1) * mm * 16, bb = (size_t)ntri * mm * 16, gb = mm * (ne + 1) * 16;
  cudaError_t e = cudaMalloc(&a, ab);
  if (e == cudaSuccess) e = cudaMalloc(&b, bb);
  if (e == cudaSuccess) e = cudaMalloc(&g, gb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a, a_host, ab, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b, b_host, bb, cudaMemcpyHostToDevice, ctx->stream);
  qg_status st = e == cudaSuccess ? QG_OK : qg_cuda_fail(ctx, e, "qg_block_cf_spectra");
  if (st == QG_OK) {
    k_block_cf<<<(unsigned)((ne + 1 + 127) / 128), 128, 0, ctx->stream>>>(m, ntri, a, b, e0, emin, de, ne, gamma, g);
    ctx->launches++;
    st = qg_check_launch(ctx, "qg_block_cf_spectra");
  }
  if (st == QG_OK) {
    e = cudaMemcpyAsync(g_host, g, gb, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_block_cf_spectra");
  }
  cudaFree(a);
  cudaFree(b);
  cudaFree(g);
  return st;
}
