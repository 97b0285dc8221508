// Dense Hermitian eigenproblems on the host: the projected matrices of the block Lanczos and
// of the Krylov-basis RIXS solver (the reference calls LAPACK zheevd there,
// Core/BlockLanczos.cpp:5530, Core/ResonantSpectra.cpp).  Plain C++; no device code.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <vector>

#include "qgpu_internal.cuh"

typedef std::complex<double> cd;

// Eigenpairs of a Hermitian matrix A (row-major, k x k): all eigenvalues ascending in w, the
// eigenvectors of the lowest nv in the columns of V (row-major, k x nv).
// 1. Householder: A = Q T Q^dag with Q = H_0 H_1 ... H_{k-3}, H_j = I - 2 v_j v_j^dag acting on
//    indices j+1..k-1, T tridiagonal with complex off-diagonal e_j.
// 2. T = D T_r D^dag with D = diag(delta), delta_{j+1} = delta_j e_j / |e_j|: T_r is real
//    symmetric with off-diagonal |e_j|.
// 3. Implicit QL with Wilkinson shifts on T_r, rotations accumulated in Z.
// 4. Eigenvector j of A = Q D z_j.
void hermitian_eigh(int k, std::vector<cd> A, std::vector<double> &w, std::vector<cd> &V, int nv) {
  auto at = [&](int i, int j) -> cd & { return A[(size_t)i * k + j]; };
  std::vector<std::vector<cd>> refl(std::max(k - 2, 0));
  std::vector<cd> p(k), wv(k);
  for (int j = 0; j + 2 < k; j++) {
    int m = k - j - 1;
    double sig2 = 0;
    for (int i = 0; i < m; i++) sig2 += std::norm(at(j + 1 + i, j));
    cd x0 = at(j + 1, j);
    double ax0 = std::abs(x0);
    if (sig2 - ax0 * ax0 <= 0.0) continue;  // column already reduced: H_j = I
    double sig = std::sqrt(sig2);
    cd ph = ax0 > 0 ? x0 / ax0 : cd(1, 0);
    cd alpha = -ph * sig;
    std::vector<cd> &v = refl[j];
    v.resize(m);
    for (int i = 0; i < m; i++) v[i] = at(j + 1 + i, j);
    v[0] -= alpha;
    double vn = 0;
    for (int i = 0; i < m; i++) vn += std::norm(v[i]);
    vn = std::sqrt(vn);
    for (int i = 0; i < m; i++) v[i] /= vn;
    // p = A22 v, c = v^dag p, w = 2 p - 2 c v;  A22 <- A22 - v w^dag - w v^dag
    double c = 0;
    for (int i = 0; i < m; i++) {
      cd acc(0, 0);
      const cd *row = &A[(size_t)(j + 1 + i) * k + j + 1];
      for (int l = 0; l < m; l++) acc += row[l] * v[l];
      p[i] = acc;
      c += (std::conj(v[i]) * acc).real();
    }
    for (int i = 0; i < m; i++) wv[i] = 2.0 * p[i] - 2.0 * c * v[i];
    for (int i = 0; i < m; i++) {
      cd *row = &A[(size_t)(j + 1 + i) * k + j + 1];
      cd vi = v[i], wi = wv[i];
      for (int l = 0; l < m; l++) row[l] -= vi * std::conj(wv[l]) + wi * std::conj(v[l]);
    }
    at(j + 1, j) = alpha;
    at(j, j + 1) = std::conj(alpha);
    for (int i = 1; i < m; i++) {
      at(j + 1 + i, j) = 0;
      at(j, j + 1 + i) = 0;
    }
  }
  std::vector<double> d(k), e(k, 0.0);
  std::vector<cd> delta(k, cd(1, 0));
  for (int i = 0; i < k; i++) d[i] = at(i, i).real();
  for (int i = 0; i + 1 < k; i++) {
    cd ec = at(i + 1, i);
    double ae = std::abs(ec);
    e[i] = ae;
    delta[i + 1] = ae > 0 ? delta[i] * (ec / ae) : delta[i];
  }
  // implicit QL; Z stored by columns (Zc[col * k + row])
  std::vector<double> Zc((size_t)k * k, 0.0);
  for (int i = 0; i < k; i++) Zc[(size_t)i * k + i] = 1.0;
  for (int l = 0; l < k; l++) {
    for (int iter = 0; iter < 100; iter++) {
      int m = l;
      for (; m < k - 1; m++) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= DBL_EPSILON * dd) break;
      }
      if (m == l) break;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
      double sn = 1.0, cs = 1.0, pp = 0.0;
      bool underflow = false;
      for (int i = m - 1; i >= l; i--) {
        double f = sn * e[i], b = cs * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= pp;
          e[m] = 0.0;
          underflow = true;
          break;
        }
        sn = f / r;
        cs = g / r;
        g = d[i + 1] - pp;
        r = (d[i] - g) * sn + 2.0 * cs * b;
        pp = sn * r;
        d[i + 1] = g + pp;
        g = cs * r - b;
        double *z0 = &Zc[(size_t)i * k], *z1 = &Zc[(size_t)(i + 1) * k];
        for (int q = 0; q < k; q++) {
          double zf = z1[q];
          z1[q] = sn * z0[q] + cs * zf;
          z0[q] = cs * z0[q] - sn * zf;
        }
      }
      if (underflow) continue;
      d[l] -= pp;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  std::vector<int> idx(k);
  for (int i = 0; i < k; i++) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  w.resize(k);
  for (int i = 0; i < k; i++) w[i] = d[idx[i]];
  nv = std::min(nv, k);
  V.assign((size_t)k * nv, cd(0, 0));
  std::vector<cd> y(k);
  for (int c = 0; c < nv; c++) {
    const double *z = &Zc[(size_t)idx[c] * k];
    for (int i = 0; i < k; i++) y[i] = delta[i] * z[i];
    for (int j = k - 3; j >= 0; j--) {
      const std::vector<cd> &v = refl[j];
      if (v.empty()) continue;
      int m = (int)v.size();
      cd t(0, 0);
      for (int i = 0; i < m; i++) t += std::conj(v[i]) * y[j + 1 + i];
      t *= 2.0;
      for (int i = 0; i < m; i++) y[j + 1 + i] -= v[i] * t;
    }
    for (int i = 0; i < k; i++) V[(size_t)i * nv + c] = y[i];
  }
}

extern "C" qg_status qg_hermitian_eigh(int32_t k, const double *a, double *w, double *v, int32_t nv) {
  if (k <= 0 || nv < 0 || nv > k || !a || !w || (nv && !v)) return QG_ERR_ARG;
  std::vector<cd> A((size_t)k * k);
  for (size_t i = 0; i < A.size(); i++) A[i] = cd(a[2 * i], a[2 * i + 1]);
  std::vector<double> ww;
  std::vector<cd> V;
  hermitian_eigh(k, A, ww, V, nv);
  for (int i = 0; i < k; i++) w[i] = ww[i];
  for (size_t i = 0; i < V.size(); i++) {
    v[2 * i] = V[i].real();
    v[2 * i + 1] = V[i].imag();
  }
  return QG_OK;
}
