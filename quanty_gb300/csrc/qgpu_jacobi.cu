// Hermitian eigenproblems on the device, the entry point for every dense eigenproblem of the
// library: the projected Krylov matrix of the block eigensolver (the reference's LAPACK zheevd,
// Core/BlockLanczos.cpp:5530), the dense H below DenseBorder (BlockLanczosGroundStateConserveBasisDense,
// :370-501; HermitianCompactMatrixToListOfPoles, Core/BasicMath/BasicMath_CompactMatrixVector.cpp:3990)
// and the resolvents of RIXS.
//
// Matrices up to QG_JAC_SMALL run here, in one block with A and the rotations in shared memory,
// by cyclic Jacobi with the round-robin (tournament) ordering, so that every step rotates k/2
// disjoint index pairs at once; it resolves degenerate multiplets -- the rule in atomic and
// impurity spectra -- without reorthogonalisation, and its eigenvalues carry relative accuracy
// near machine precision.  Larger matrices go through the tridiagonal reduction
// (qgpu_hermitian.cu), whose cost grows as k^3 once instead of k^3 per sweep.
//
// One rotation on the pair (p, q) of a Hermitian matrix with b = A[p][q] = |b| e^{i phi}:
//   tau = (A[q][q] - A[p][p]) / (2 |b|),  t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
//   c = 1 / sqrt(1 + t^2),  s = t c,  J = [[c, s e^{i phi}], [-s e^{-i phi}, c]],
// and A <- J^H A J zeroes A[p][q] (the real symmetric rotation conjugated by diag(1, e^{-i phi})).
// A step applies the row rotations of all its pairs (J^H from the left), then the column
// rotations (J from the right) and accumulates V <- V J; the eigenvectors are kept as the rows
// of Vt = V^T so that both updates read and write whole rows.  Sweeps run until the
// off-diagonal norm falls below 1e-15 of the Frobenius norm (at most QG_JAC_SWEEPS sweeps).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "qgpu_internal.cuh"

#define QG_JAC_SMALL 40
#define QG_JAC_SWEEPS 60
#define QG_JAC_TOL2 1e-30  // (off-diagonal norm / Frobenius norm)^2 at convergence

struct JacRot {
  double c, s;    // cosine and sine of the real rotation
  double er, ei;  // e^{i phi}
  int skip;       // A[p][q] == 0: identity
};

__device__ __forceinline__ JacRot jac_rotation(double app, double aqq, double2 b) {
  JacRot r;
  const double ab = hypot(b.x, b.y);
  // below 1e-20 of the diagonal a rotation changes nothing representable; k^2 such entries stay
  // far below the convergence threshold (1e-30 of the squared Frobenius norm) for k < 10^4
  if (ab == 0.0 || ab < 1e-20 * (fabs(app) + fabs(aqq))) {
    r.c = 1.0;
    r.s = 0.0;
    r.er = 1.0;
    r.ei = 0.0;
    r.skip = 1;
    return r;
  }
  const double tau = (aqq - app) / (2.0 * ab);
  // the smaller root of t^2 + 2 tau t - 1 = 0 (|t| <= 1); 1 / (2 tau) where tau^2 would overflow
  const double t = fabs(tau) > 1e100 ? 0.5 / tau : (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
  r.c = 1.0 / sqrt(1.0 + t * t);
  r.s = t * r.c;
  r.er = b.x / ab;
  r.ei = b.y / ab;
  r.skip = 0;
  return r;
}

// the round-robin pair m of step s among kk (even) indices: index kk - 1 stays, the others turn
__host__ __device__ __forceinline__ void jac_pair(int kk, int s, int m, int &p, int &q) {
  int a, b;
  if (m == 0) {
    a = kk - 1;
    b = s;
  } else {
    a = (s + m) % (kk - 1);
    b = (s - m + kk - 1) % (kk - 1);
  }
  p = a < b ? a : b;
  q = a < b ? b : a;
}

// x_p' = c x_p - s e^{i phi} x_q,  x_q' = s e^{-i phi} x_p + c x_q  (rows under J^H)
__device__ __forceinline__ void jac_left(const JacRot &r, double2 &xp, double2 &xq) {
  const double2 p = xp, q = xq;
  // e q and conj(e) p
  const double eqx = r.er * q.x - r.ei * q.y, eqy = r.er * q.y + r.ei * q.x;
  const double epx = r.er * p.x + r.ei * p.y, epy = r.er * p.y - r.ei * p.x;
  xp = make_double2(r.c * p.x - r.s * eqx, r.c * p.y - r.s * eqy);
  xq = make_double2(r.s * epx + r.c * q.x, r.s * epy + r.c * q.y);
}

// y_p' = c y_p - s e^{-i phi} y_q,  y_q' = s e^{i phi} y_p + c y_q  (columns under J; the rows
// of Vt = V^T transform the same way)
__device__ __forceinline__ void jac_right(const JacRot &r, double2 &yp, double2 &yq) {
  const double2 p = yp, q = yq;
  const double cqx = r.er * q.x + r.ei * q.y, cqy = r.er * q.y - r.ei * q.x;  // conj(e) q
  const double epx = r.er * p.x - r.ei * p.y, epy = r.er * p.y + r.ei * p.x;  // e p
  yp = make_double2(r.c * p.x - r.s * cqx, r.c * p.y - r.s * cqy);
  yq = make_double2(r.s * epx + r.c * q.x, r.s * epy + r.c * q.y);
}

// ------------------------------------------------------------------ small matrices: one block

// A (k x k row-major, Hermitian), eigenvalues ascending into w, the eigenvectors of the lowest nv
// as the columns of V (k x nv row-major); status[0] = sweeps used (QG_JAC_SWEEPS + 1: not
// converged).
__global__ void __launch_bounds__(256) k_jacobi_small(const double2 *__restrict__ Ain, int k, int nv,
                                                      double *__restrict__ w, double2 *__restrict__ V,
                                                      int *__restrict__ status) {
  extern __shared__ double2 sh[];
  const int kk = k + (k & 1);
  double2 *A = sh;            // [kk][kk], the padding row and column stay zero
  double2 *Vt = sh + kk * kk;  // [kk][kk]
  __shared__ JacRot rot[QG_JAC_SMALL / 2 + 1];
  __shared__ double red[2][8];
  __shared__ int done;
  for (int t = threadIdx.x; t < kk * kk; t += blockDim.x) {
    const int i = t / kk, j = t % kk;
    A[t] = (i < k && j < k) ? Ain[i * k + j] : make_double2(0.0, 0.0);
    Vt[t] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  if (threadIdx.x == 0) done = 0;
  __syncthreads();
  int sweep = 0;
  for (; sweep < QG_JAC_SWEEPS; sweep++) {
    // off-diagonal and total squared norms
    double off = 0.0, tot = 0.0;
    for (int t = threadIdx.x; t < kk * kk; t += blockDim.x) {
      const double2 a = A[t];
      const double m = a.x * a.x + a.y * a.y;
      tot += m;
      if (t / kk != t % kk) off += m;
    }
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = off;
      red[1][threadIdx.x >> 5] = tot;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double o2 = 0.0, t2 = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
        o2 += red[0][i];
        t2 += red[1][i];
      }
      done = !(o2 > QG_JAC_TOL2 * t2);
    }
    __syncthreads();
    if (done) break;
    for (int s = 0; s < kk - 1; s++) {
      if (threadIdx.x < kk / 2) {
        int p, q;
        jac_pair(kk, s, threadIdx.x, p, q);
        rot[threadIdx.x] = q < k ? jac_rotation(A[p * kk + p].x, A[q * kk + q].x, A[p * kk + q])
                                 : JacRot{1.0, 0.0, 1.0, 0.0, 1};
      }
      __syncthreads();
      for (int t = threadIdx.x; t < (kk / 2) * kk; t += blockDim.x) {  // rows p, q of A and Vt
        const int m = t / kk, j = t % kk;
        const JacRot r = rot[m];
        if (r.skip) continue;
        int p, q;
        jac_pair(kk, s, m, p, q);
        jac_left(r, A[p * kk + j], A[q * kk + j]);
        jac_right(r, Vt[p * kk + j], Vt[q * kk + j]);
      }
      __syncthreads();
      for (int t = threadIdx.x; t < (kk / 2) * kk; t += blockDim.x) {  // columns p, q of A
        const int m = t / kk, i = t % kk;
        const JacRot r = rot[m];
        if (r.skip) continue;
        int p, q;
        jac_pair(kk, s, m, p, q);
        jac_right(r, A[i * kk + p], A[i * kk + q]);
      }
      __syncthreads();
      if (threadIdx.x < kk / 2 && !rot[threadIdx.x].skip) {  // exact zeros and a real diagonal
        int p, q;
        jac_pair(kk, s, threadIdx.x, p, q);
        A[p * kk + q] = make_double2(0.0, 0.0);
        A[q * kk + p] = make_double2(0.0, 0.0);
        A[p * kk + p].y = 0.0;
        A[q * kk + q].y = 0.0;
      }
      __syncthreads();
    }
  }
  // ascending order by rank (ties by index)
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const double di = A[i * kk + i].x;
    int rank = 0;
    for (int j = 0; j < k; j++) {
      const double dj = A[j * kk + j].x;
      rank += (dj < di) || (dj == di && j < i);
    }
    w[rank] = di;
    if (rank < nv)
      for (int r = 0; r < k; r++) V[r * nv + rank] = Vt[i * kk + r];
  }
  if (threadIdx.x == 0) status[0] = done ? sweep : QG_JAC_SWEEPS + 1;
}

// Eigenpairs of the Hermitian k x k matrix A (device, row-major; overwritten): eigenvalues
// ascending into w_dev (k), the eigenvectors of the lowest nv into V_dev (k x nv row-major,
// columns).  Only the Hermitian part of A is meaningful: entries are used as given.
qg_status qg_eigh_device(qg_context ctx, int k, double2 *A, double *w_dev, double2 *V_dev, int nv) {
  if (k <= 0) return QG_OK;
  if (nv < 0 || nv > k) return QG_ERR_ARG;
  cudaStream_t s = ctx->stream;
  int *d_status = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d_status, sizeof(int)));
  qg_status st = QG_OK;
  int sweeps = 0;
  if (k <= QG_JAC_SMALL) {
    const int kk = k + (k & 1);
    const size_t smem = (size_t)2 * kk * kk * sizeof(double2);
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_jacobi_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           2 * (QG_JAC_SMALL + 1) * (QG_JAC_SMALL + 1) * (int)sizeof(double2));
      attr = true;
    }
    k_jacobi_small<<<1, 256, smem, s>>>(A, k, nv, w_dev, V_dev, d_status);
    ctx->launches++;
    st = qg_check_launch(ctx, "qg_eigh_device");
    if (st == QG_OK) {
      cudaError_t e = cudaMemcpyAsync(&sweeps, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_eigh_device");
    }
  } else {
    st = qg_eigh_tridiag(ctx, k, A, w_dev, V_dev, nv);
  }
  cudaFree(d_status);
  if (st == QG_OK && sweeps > QG_JAC_SWEEPS) {
    ctx->last_error = "qg_eigh_device: Jacobi did not converge";
    return QG_ERR_TIMEOUT;
  }
  return st;
}

// Host matrix in, host eigenpairs out, computed on the device.
qg_status qg_eigh_host_io(qg_context ctx, int k, const double *a_host, double *w_host, double *v_host, int nv) {
  if (k <= 0) return QG_OK;
  double2 *A = nullptr, *V = nullptr;
  double *w = nullptr;
  const size_t ab = (size_t)k * k * sizeof(double2), vb = (size_t)k * std::max(nv, 1) * sizeof(double2);
  cudaError_t e = cudaMalloc(&A, ab);
  if (e == cudaSuccess) e = cudaMalloc(&V, vb);
  if (e == cudaSuccess) e = cudaMalloc(&w, (size_t)k * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(A, a_host, ab, cudaMemcpyHostToDevice, ctx->stream);
  qg_status st = e == cudaSuccess ? QG_OK : qg_cuda_fail(ctx, e, "qg_hermitian_eigh");
  if (st == QG_OK) st = qg_eigh_device(ctx, k, A, w, V, nv);
  if (st == QG_OK) {
    e = cudaMemcpyAsync(w_host, w, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && nv > 0 && v_host)
      e = cudaMemcpyAsync(v_host, V, (size_t)k * nv * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_hermitian_eigh");
  }
  cudaFree(A);
  cudaFree(V);
  cudaFree(w);
  return st;
}

extern "C" qg_status qg_hermitian_eigh(qg_context ctx, int32_t k, const double *a, double *w, double *v, int32_t nv) {
  if (!ctx || k < 0 || nv < 0 || nv > k || (k > 0 && (!a || !w)) || (nv > 0 && !v)) return QG_ERR_ARG;
  return qg_eigh_host_io(ctx, k, a, w, v, nv);
}
