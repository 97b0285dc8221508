// Resonant (RIXS) spectra and the Krylov-basis Lanczos they need.
//
// The reference (ResonantSpectra, Core/ResonantSpectra.cpp:6-283) computes
// <psi|T1^dag G1^dag T2^dag G2 T2 G1 T1|psi> as follows: T1|psi>; a Lanczos of H1 that keeps
// its Krylov vectors (LanczosTriDiagonalizeKrylovCC, Core/Lanczos.cpp:3705); the eigensystem
// of that tridiagonal matrix; for every incident energy w_p the Krylov-projected resolvent
// G1(w_p) T1|psi> = b0 sum_i c_i(p) K_i with c_i(p) = sum_k e_k(i) e_k(0) / (w_p - E_k + i G1/2);
// then for every T2 a Lanczos of H2 on T2 G1 T1 |psi> and the continued fraction.
//
// Here every incident energy and every T2 runs at once: the G1 T1|psi> vectors of all w_p form
// one n1 x (NE1+1) block (one combination kernel over the stored Krylov vectors), T2 is applied
// to the whole block with the multi-vector pull kernel into the common closure basis of all
// T2 targets under H2, and the NT2 (NE1+1) second-stage Lanczos recursions run as one batched
// qg_lanczos_tridiag; all spectra come from one continued-fraction kernel.
#include <cfloat>
#include <cmath>
#include <complex>
#include <vector>

#include "qgpu_internal.cuh"

typedef std::complex<double> cd;

static inline unsigned gridn(int64_t n) { return (unsigned)((n + 255) / 256); }

// ------------------------------------------------------------------ small device kernels

// y -= d * x with d a complex scalar on the device
__global__ void k_axpy_dev(int64_t n, double2 *y, const double2 *x, const double2 *d) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double2 c = *d, xv = x[r], yv = y[r];
  yv.x -= c.x * xv.x - c.y * xv.y;
  yv.y -= c.x * xv.y + c.y * xv.x;
  y[r] = yv;
}

__global__ void k_store_re(const double2 *d, double *dst) { *dst = d->x; }

// b = sqrt(<v|v>), scale = b < 100 DBL_MIN ? 0 : 1/b
__global__ void k_norm_scale(const double2 *dot, double *b_out, double *scale) {
  double b = sqrt(dot->x);
  *b_out = b;
  *scale = (b < 100 * DBL_MIN) ? 0.0 : 1.0 / b;
}

__global__ void k_scale_vec(int64_t n, double2 *v, const double *scale) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double s = *scale;
  double2 x = v[r];
  v[r] = make_double2(x.x * s, x.y * s);
}

// multiple dots: part[blk * m + j] = sum over the block's rows of conj(K_j) v, j < m
__global__ void k_multidot_partial(const double2 *K, int64_t n, int m, const double2 *v, double2 *part) {
  __shared__ double2 sh[8];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = 0; j < m; j++) {
    double2 s = make_double2(0, 0);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 a = K[(int64_t)j * n + r], b = v[r];
      s.x += a.x * b.x + a.y * b.y;
      s.y += a.x * b.y - a.y * b.x;
    }
    for (int o = 16; o; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0, 0);
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        t.x += sh[w].x;
        t.y += sh[w].y;
      }
      part[(int64_t)blockIdx.x * m + j] = t;
    }
    __syncthreads();
  }
}

// orthogonality test of the reference: sum_j |<K_j|v>|^2 (reverse order, early exit) > eps
// zeroes v; then err *= b^2/(b^2 + DBL_MIN + DBL_EPSILON a^2) and thr2 = (eps/err)^2
__global__ void k_orth_test(const double2 *part, int nblk, int m, double eps, double *zero_flag, double *err,
                            const double *a_i, const double *b_i, double *thr2) {
  double temp = 0;
  int flag = 0;
  for (int j = m - 1; j >= 0 && !flag; j--) {
    double sr = 0, si = 0;
    for (int bk = 0; bk < nblk; bk++) {
      sr += part[(int64_t)bk * m + j].x;
      si += part[(int64_t)bk * m + j].y;
    }
    temp += sr * sr + si * si;
    if (temp > eps) flag = 1;
  }
  *zero_flag = flag ? 0.0 : 1.0;
  double b = *b_i, a = *a_i;
  double e = *err * (b * b / (b * b + DBL_MIN + DBL_EPSILON * a * a));
  *err = e;
  double th = eps / e;
  *thr2 = th * th;
}

__global__ void k_trunc_vec(int64_t n, double2 *v, const double *mult, const double *thr2) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double m = *mult, t2 = *thr2;
  double2 x = v[r];
  x.x *= m;
  x.y *= m;
  if (!(x.x * x.x + x.y * x.y > t2)) x = make_double2(0, 0);
  v[r] = x;
}

// out[r][p] = sum_i K_i[r] C[i][p] (K vector-major, C row-major ntri x np)
// ------------------------------------------------------------------ Krylov-basis Lanczos

// Lanczos keeping the Krylov vectors, the reference's LanczosTriDiagonalizeKrylovCC: modified
// Gram-Schmidt of H K_{i-1} against all earlier vectors in reverse order, normalisation, the
// orthogonality test, truncation at eps/err.  K_dev: ntri * n complex (vector-major).
static qg_status lanczos_krylov(qg_context ctx, qg_operator op, qg_basis b, const double *v0, int ntri, double eps,
                                double *a_host, double *b_host, double2 *K) {
  cudaStream_t s = ctx->stream;
  int64_t n = b->n;
  int P = qg_partial_blocks(ctx, n);
  double *sc = nullptr;  // [0] scale [1] zero flag [2] err [3] thr2, then a_hist (ntri+1), b_hist (ntri)
  double2 *dots = nullptr, *part = nullptr;
  cudaError_t e = cudaMalloc(&sc, (4 + 2 * ntri + 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dots, 16);
  if (e == cudaSuccess) e = cudaMalloc(&part, (size_t)P * ntri * 16);
  if (e != cudaSuccess) {
    cudaFree(sc);
    cudaFree(dots);
    return qg_cuda_fail(ctx, e, "lanczos_krylov");
  }
  double *scale = sc, *flag = sc + 1, *err = sc + 2, *thr2 = sc + 3, *ah = sc + 4, *bh = sc + 5 + ntri;
  std::vector<double> init(4 + 2 * ntri + 1, 0.0);
  init[2] = 1.0;  // err
  init[3] = eps * eps;
  cudaMemcpyAsync(sc, init.data(), init.size() * 8, cudaMemcpyHostToDevice, s);
  qg_status st = QG_OK;
  // K_0
  cudaMemcpyAsync(K, v0, n * 16, cudaMemcpyDeviceToDevice, s);
  st = qg_dot_dev(ctx, n, 1, (const double *)K, (const double *)K, (double *)dots);
  k_norm_scale<<<1, 1, 0, s>>>(dots, bh, scale);
  k_scale_vec<<<gridn(n), 256, 0, s>>>(n, K, scale);
  ctx->launches += 2;
  {
    double one = 1.0;
    cudaMemcpyAsync(flag, &one, 8, cudaMemcpyHostToDevice, s);
  }
  k_trunc_vec<<<gridn(n), 256, 0, s>>>(n, K, flag, thr2);
  ctx->launches++;
  for (int i = 1; i < ntri && st == QG_OK; i++) {
    double2 *Ki = K + (int64_t)i * n;
    st = qg_apply_launch(ctx, op, b, b, (const double *)(K + (int64_t)(i - 1) * n), (double *)Ki, 1, nullptr);
    for (int j = i - 1; j >= 0 && st == QG_OK; j--) {
      st = qg_dot_dev(ctx, n, 1, (const double *)(K + (int64_t)j * n), (const double *)Ki, (double *)dots);
      if (j == i - 1) {
        k_store_re<<<1, 1, 0, s>>>(dots, ah + i);
        ctx->launches++;
      }
      k_axpy_dev<<<gridn(n), 256, 0, s>>>(n, Ki, K + (int64_t)j * n, dots);
      ctx->launches++;
    }
    if (st != QG_OK) break;
    st = qg_dot_dev(ctx, n, 1, (const double *)Ki, (const double *)Ki, (double *)dots);
    k_norm_scale<<<1, 1, 0, s>>>(dots, bh + i, scale);
    k_scale_vec<<<gridn(n), 256, 0, s>>>(n, Ki, scale);
    k_multidot_partial<<<P, 256, 0, s>>>(K, n, i, Ki, part);
    k_orth_test<<<1, 1, 0, s>>>(part, P, i, eps, flag, err, ah + i, bh + i, thr2);
    k_trunc_vec<<<gridn(n), 256, 0, s>>>(n, Ki, flag, thr2);
    ctx->launches += 5;
    if ((st = qg_check_launch(ctx, "lanczos_krylov")) != QG_OK) break;
  }
  // a[ntri] = <K_last|H|K_last>
  if (st == QG_OK) {
    double2 *hk = nullptr;
    e = cudaMalloc(&hk, n * 16);
    if (e == cudaSuccess) {
      st = qg_apply_launch(ctx, op, b, b, (const double *)(K + (int64_t)(ntri - 1) * n), (double *)hk, 1, nullptr);
      if (st == QG_OK) st = qg_dot_dev(ctx, n, 1, (const double *)(K + (int64_t)(ntri - 1) * n), (const double *)hk,
                                       (double *)dots);
      if (st == QG_OK) {
        k_store_re<<<1, 1, 0, s>>>(dots, ah + ntri);
        ctx->launches++;
      }
      cudaStreamSynchronize(s);
      cudaFree(hk);
    } else {
      st = qg_cuda_fail(ctx, e, "lanczos_krylov");
    }
  }
  if (st == QG_OK) {
    e = cudaMemcpyAsync(a_host, ah, (ntri + 1) * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b_host, bh, ntri * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "lanczos_krylov");
    a_host[0] = 0.0;
  }
  cudaStreamSynchronize(s);
  cudaFree(sc);
  cudaFree(dots);
  cudaFree(part);
  return st;
}

extern "C" qg_status qg_lanczos_krylov(qg_context ctx, qg_operator op, qg_basis b, const double *v0_dev, int32_t ntri,
                                       double eps, double *a_host, double *b_host, double *krylov_dev) {
  if (!ctx || !op || !b || !v0_dev || ntri <= 0 || !a_host || !b_host || !krylov_dev || op->nf != b->nf)
    return QG_ERR_ARG;
  if (!b->n) return QG_ERR_ARG;
  qg_status st = lanczos_krylov(ctx, op, b, v0_dev, ntri, eps, a_host, b_host, (double2 *)krylov_dev);
  if (st == QG_OK) st = qg_check_device_error(ctx, "qg_lanczos_krylov");
  return st;
}

// ------------------------------------------------------------------ RIXS

// Lowest and highest eigenvalue of the symmetric tridiagonal matrix diag a[1..nt], off-diagonal
// b[1..nt-1] by bisection on Sturm counts inside the Gershgorin interval: only the final-state
// pole range is needed of the second-stage chains, not their eigenvectors.
static int sturm_below(int nt, const double *a, const double *b, double x) {
  int cnt = 0;
  double d = 1.0;
  for (int i = 0; i < nt; i++) {
    const double off = i ? b[i] * b[i] : 0.0;
    d = (a[i + 1] - x) - (i ? off / d : 0.0);
    if (d == 0.0) d = -1e-300;  // a zero pivot counts as negative (the limit from below)
    cnt += d < 0.0;
  }
  return cnt;
}

static void tridiag_extremes(int nt, const double *a, const double *b, double *lo, double *hi) {
  double g0 = DBL_MAX, g1 = -DBL_MAX;
  for (int i = 0; i < nt; i++) {
    const double r = (i ? std::fabs(b[i]) : 0.0) + (i + 1 < nt ? std::fabs(b[i + 1]) : 0.0);
    g0 = std::min(g0, a[i + 1] - r);
    g1 = std::max(g1, a[i + 1] + r);
  }
  for (int which = 0; which < 2; which++) {
    // the eigenvalue with (which ? nt - 1 : 0) eigenvalues below it
    const int target = which ? nt - 1 : 0;
    double l = g0, h = g1;
    for (int it = 0; it < 200 && h - l > 4 * DBL_EPSILON * std::max(std::fabs(l), std::fabs(h)); it++) {
      const double m = 0.5 * (l + h);
      if (m <= l || m >= h) break;
      if (sturm_below(nt, a, b, m) > target)
        h = m;
      else
        l = m;
    }
    (which ? *hi : *lo) = 0.5 * (l + h);
  }
}

static qg_status tridiag_eigen(qg_context ctx, int nt, const double *a, const double *b, std::vector<double> &ev,
                               std::vector<cd> &Z) {
  // diag a[1..nt], off-diagonal b[1..nt-1] (TriDiagonalMatrixToEigensystem's matrix)
  std::vector<cd> M((size_t)nt * nt, cd(0, 0));
  for (int i = 0; i < nt; i++) {
    M[(size_t)i * nt + i] = a[i + 1];
    if (i + 1 < nt) {
      M[(size_t)i * nt + i + 1] = b[i + 1];
      M[(size_t)(i + 1) * nt + i] = b[i + 1];
    }
  }
  ev.assign(nt, 0.0);
  Z.assign((size_t)nt * nt, cd(0, 0));
  return qg_eigh_host_io(ctx, nt, (const double *)M.data(), ev.data(), (double *)Z.data(), nt);
}

extern "C" qg_status qg_resonant_spectra(qg_context ctx, qg_operator H1, qg_operator H2, qg_operator T1,
                                         const qg_operator *T2, int32_t nt2, qg_basis psi_basis, const double *psi_dev,
                                         qg_rixs_settings *o, double *g_host) {
  if (!ctx || !H1 || !H2 || !T1 || !T2 || nt2 <= 0 || !psi_basis || !psi_dev || !o || !g_host) return QG_ERR_ARG;
  if (o->ntri1 <= 0 || o->ntri2 <= 0 || o->ne1 <= 0 || o->ne2 <= 0) return QG_ERR_ARG;
  cudaStream_t s = ctx->stream;
  qg_status st = QG_OK;
  // energies <psi|H|psi>/<psi|psi>
  double nrm2 = 0;
  {
    double t[2];
    QG_TRY(qg_dot(ctx, psi_basis->n, 1, psi_dev, psi_dev, t));
    nrm2 = t[0];
  }
  double div = nrm2 > DBL_EPSILON ? nrm2 : 1.0;
  if (o->energy1 == DBL_MAX) {
    double v[2];
    QG_TRY(qg_expectation(ctx, H1, psi_basis, psi_dev, 1, v));
    o->energy1 = v[0] / div;
  }
  if (o->energy2 == DBL_MAX) {
    double v[2];
    QG_TRY(qg_expectation(ctx, H2, psi_basis, psi_dev, 1, v));
    o->energy2 = v[0] / div;
  }
  // T1 |psi> on its target basis, then on the closure under H1
  qg_basis bt = nullptr, b1 = nullptr, bt2 = nullptr, b2 = nullptr;
  double *tpsi = nullptr, *x1 = nullptr, *K = nullptr, *gt = nullptr, *x2 = nullptr;
  double2 *Cd = nullptr;
  int np = o->ne1 + 1, ncol = nt2 * np;
  std::vector<double> a1(o->ntri1 + 1), b1v(o->ntri1);
  cudaError_t e = cudaSuccess;
  do {
    if ((st = qg_operator_psi_basis(ctx, T1, psi_basis, o->res1, &bt)) != QG_OK) break;
    if ((e = cudaMalloc(&tpsi, std::max<int64_t>(bt->n, 1) * 16)) != cudaSuccess) break;
    if ((st = qg_apply(ctx, T1, bt, psi_basis, psi_dev, tpsi, 1)) != QG_OK) break;
    int rounds = 0;
    if ((st = qg_basis_closure(ctx, H1, bt, o->res1, -1, &b1, &rounds)) != QG_OK) break;
    int64_t n1 = b1->n;
    if ((e = cudaMalloc(&x1, std::max<int64_t>(n1, 1) * 16)) != cudaSuccess) break;
    if ((st = qg_basis_map(ctx, bt, tpsi, b1, x1, 1)) != QG_OK) break;
    if ((e = cudaMalloc(&K, (size_t)o->ntri1 * std::max<int64_t>(n1, 1) * 16)) != cudaSuccess) break;
    if ((st = lanczos_krylov(ctx, H1, b1, x1, o->ntri1, o->epsilon, a1.data(), b1v.data(), (double2 *)K)) != QG_OK)
      break;
    std::vector<double> ev;
    std::vector<cd> Z;
    if ((st = tridiag_eigen(ctx, o->ntri1, a1.data(), b1v.data(), ev, Z)) != QG_OK) break;
    int nt = o->ntri1;
    // intermediate-state energy range defaults (Core/ResonantSpectra.cpp:80-112)
    if (o->emin1 > 0.001 * DBL_MAX && o->emax1 < -0.001 * DBL_MAX) {
      o->emin1 = 1.1 * ev[0] - 0.1 * ev[nt - 1];
      o->emax1 = 1.1 * ev[nt - 1] - 0.1 * ev[0];
    }
    if (o->emin1 > 0.001 * DBL_MAX) o->emin1 = 1.1 * ev[0] - 0.1 * o->emax1;
    if (o->emax1 < -0.001 * DBL_MAX) o->emax1 = 1.1 * ev[nt - 1] - 0.1 * o->emin1;
    if (o->gamma1 == 0 && o->ne1 == 0) {
      o->ne1 = 1000;
      o->gamma1 = 5 * (o->emax1 - o->emin1) / o->ne1;
    }
    if (o->ne1 == 0) o->ne1 = (int32_t)(5 * (o->emax1 - o->emin1) / o->gamma1);
    if (o->gamma1 == 0) o->gamma1 = 5 * (o->emax1 - o->emin1) / o->ne1;
    np = o->ne1 + 1;
    ncol = nt2 * np;
    // Krylov-projected resolvent coefficients, all incident energies
    std::vector<cd> C((size_t)nt * np);
    for (int p = 0; p < np; p++) {
      double w = o->emin1 + (o->emax1 - o->emin1) * p / (double)o->ne1 + o->energy1;
      for (int i = 0; i < nt; i++) {
        cd acc(0, 0);
        for (int k = 0; k < nt; k++) {
          cd inv = 1.0 / cd(w - ev[k], 0.5 * o->gamma1);
          acc += inv * Z[(size_t)i * nt + k] * Z[(size_t)k] * 1.0;  // e_k(i) e_k(0)
        }
        C[(size_t)i * np + p] = b1v[0] * acc;
      }
    }
    if ((e = cudaMalloc(&Cd, C.size() * 16)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(Cd, C.data(), C.size() * 16, cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
    if ((e = cudaMalloc(&gt, (size_t)std::max<int64_t>(n1, 1) * np * 16)) != cudaSuccess) break;
    if ((st = qg_block_combine(ctx, (const double2 *)K, n1, nt, Cd, np, (double2 *)gt)) != QG_OK) break;
    // T2 targets of all operators, their closure under H2: the common final-state basis
    for (int j = 0; j < nt2 && st == QG_OK; j++) {
      qg_basis tj = nullptr;
      st = qg_operator_psi_basis(ctx, T2[j], b1, o->res2, &tj);
      if (st != QG_OK) break;
      if (!bt2) {
        bt2 = tj;
      } else {
        qg_basis u = nullptr;
        st = qg_basis_union(ctx, bt2, tj, &u);
        qg_basis_destroy(bt2);
        qg_basis_destroy(tj);
        bt2 = u;
      }
    }
    if (st != QG_OK) break;
    if ((st = qg_basis_closure(ctx, H2, bt2, o->res2, -1, &b2, &rounds)) != QG_OK) break;
    int64_t n2 = b2->n;
    if ((e = cudaMalloc(&x2, (size_t)std::max<int64_t>(n2, 1) * ncol * 16)) != cudaSuccess) break;
    for (int j = 0; j < nt2 && st == QG_OK; j++)
      st = qg_apply_strided(ctx, T2[j], b2, b1, gt, np, x2 + 2 * (size_t)j * np, ncol, np, nullptr, false);
    if (st != QG_OK) break;
    // all second-stage recursions at once
    std::vector<double> a2((size_t)ncol * (o->ntri2 + 1)), b2v((size_t)ncol * o->ntri2);
    st = qg_lanczos_tridiag(ctx, H2, b2, x2, ncol, o->ntri2, o->epsilon, std::sqrt(DBL_EPSILON) + o->gamma2, a2.data(),
                            b2v.data(), nullptr);
    if (st != QG_OK) break;
    // final-state energy range from the poles (Core/ResonantSpectra.cpp:221-262)
    double lo = DBL_MAX, hi = -DBL_MAX;
    for (int c = 0; c < ncol; c++) {
      double e0, e1;
      tridiag_extremes(o->ntri2, &a2[(size_t)c * (o->ntri2 + 1)], &b2v[(size_t)c * o->ntri2], &e0, &e1);
      lo = std::min(lo, e0 - o->energy2);
      hi = std::max(hi, e1 - o->energy2);
    }
    if (o->emin2 > 0.001 * DBL_MAX || o->emax2 < -0.001 * DBL_MAX) {
      if (o->emin2 > 0.001 * DBL_MAX && o->emax2 < -0.001 * DBL_MAX) {
        o->emin2 = 1.1 * lo - 0.1 * hi;
        o->emax2 = 1.1 * hi - 0.1 * lo;
      } else if (o->emin2 > 0.001 * DBL_MAX) {
        o->emin2 = 1.1 * lo - 0.1 * o->emax2;
      } else {
        o->emax2 = 1.1 * hi - 0.1 * o->emin2;
      }
    }
    if (o->gamma2 == 0 && o->ne2 == 0) {
      o->ne2 = 1000;
      o->gamma2 = 5 * (o->emax2 - o->emin2) / o->ne2;
    }
    if (o->ne2 == 0) o->ne2 = (int32_t)(5 * (o->emax2 - o->emin2) / o->gamma2);
    if (o->gamma2 == 0) o->gamma2 = 5 * (o->emax2 - o->emin2) / o->ne2;
    std::vector<double> e0(ncol, o->energy2);
    st = qg_cf_spectra(ctx, ncol, o->ntri2, a2.data(), b2v.data(), e0.data(), o->emin2,
                       (o->emax2 - o->emin2) / o->ne2, o->ne2, o->gamma2, g_host);
  } while (0);
  if (e != cudaSuccess && st == QG_OK) st = qg_cuda_fail(ctx, e, "qg_resonant_spectra");
  cudaStreamSynchronize(s);
  cudaFree(tpsi);
  cudaFree(x1);
  cudaFree(K);
  cudaFree(Cd);
  cudaFree(gt);
  cudaFree(x2);
  qg_basis_destroy(bt);
  qg_basis_destroy(b1);
  qg_basis_destroy(bt2);
  qg_basis_destroy(b2);
  if (st == QG_OK) st = qg_check_device_error(ctx, "qg_resonant_spectra");
  return st;
}
