// Hermitian eigenproblems larger than one block's shared memory (k > QG_JAC_SMALL), by reduction
// to a real symmetric tridiagonal matrix.  The reference calls LAPACK zheevd for its dense
// matrices (Core/BlockLanczos.cpp:5530, :370-501; Core/BasicMath/BasicMath_CompactMatrixVector.cpp:3990);
// the steps here are published methods, restated for the device:
//  1. Householder tridiagonalisation (the unblocked reduction of LAPACK's zhetd2).  For column j
//     the reflector H_j = I - tau_j v_j v_j^H, v_j[0] = 1, satisfies H_j^H x = beta_j e_1 with
//     beta_j real, x = A[j+1:, j]; then p = tau A22 v, w = p - (tau/2)(p^H v) v and
//     A22 -= v w^H + w v^H.  Per column a launch in which every block forms v from row j of A
//     (the conjugate of column j), the matrix-vector product runs a warp per row and the last
//     block to finish forms w; the rank-2 update is a launch of its own for the large columns,
//     and below HH_FOLD_ROWS rows it is applied by the next column's launch to what it reads
//     (the last one by the launch that reads the last diagonal entry).
//     T = Q^H A Q, Q = H_0 H_1 ... H_(k-2), T real: diagonal d, off-diagonal beta.
//  2. Eigenvalues of T by bisection on Sturm counts (the method of LAPACK's dstebz), as
//     multisection: one warp per eigenvalue, 32 counts per round, down to the last
//     representable midpoint.
//  3. Eigenvectors of T for the lowest nv eigenvalues by inverse iteration (the method of
//     LAPACK's dstein): T - lambda I factored with partial pivoting, tiny pivots replaced by
//     eps |T|, three solves from a pseudo-random start, each followed by modified Gram-Schmidt
//     against the vectors already found in the same cluster (consecutive eigenvalues closer
//     than 1e-3 |T|_1; equal ones shifted apart by 10 eps |lambda|).  One block per cluster.
//  4. The eigenvectors of A are Q z: the reflectors applied from the last to the first, one
//     block per eight vectors with each reflector staged in shared memory.
// Every sum runs in a fixed order, so the results are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "qgpu_internal.cuh"

#define HH_WARPS 4        // rows (one per warp) per block of the reflector / matrix-vector kernel
#define HH_FOLD_ROWS 512  // below this many rows a column's rank-2 update is folded into the next
                          // column's launch; above, it is a launch of its own
#define HH_BT_VECS 8      // eigenvectors (one per warp) per block of the back-transformation
#define HH_MAX_K 12000    // shared memory holds one reflector (16 B per entry)
#define HH_INV_THREADS 128

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// block-wide sum in a fixed order (threads, then the warps in order), combined by one thread
// and shared: every thread gets it.  red holds one entry per warp plus one.
__device__ double block_sum(double s, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __syncthreads();  // red may still be read from a previous call
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += red[w];
    red[nw] = t;
  }
  __syncthreads();
  return red[nw];
}

__device__ double2 block_sum2(double2 s, double2 *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  __syncthreads();
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < nw; w++) {
      t.x += red[w].x;
      t.y += red[w].y;
    }
    red[nw] = t;
  }
  __syncthreads();
  return red[nw];
}

}  // namespace

// A22(j-1)[r][c] after the rank-2 update of column j - 1: a - (v_r conj(w_c) + w_r conj(v_c)),
// with v, w of that column indexed over A22(j-1) (entry 0 is row / column j).
__device__ __forceinline__ double2 hh_updated(double2 a, double2 vr, double2 wr, double2 vc, double2 wc) {
  a.x -= (vr.x * wc.x + vr.y * wc.y) + (wr.x * vc.x + wr.y * vc.y);
  a.y -= (vr.y * wc.x - vr.x * wc.y) + (wr.y * vc.x - wr.x * vc.y);
  return a;
}

// Column j, with the rank-2 update of column j - 1 (A22 -= v w^H + w v^H) folded in when it is
// pending: every block brings row j up to date as it reads it, and the warp that owns a row of
// the trailing matrix updates it, writes it back and uses it.  Then the reflector from x = A[j+1:, j] (read as the
// conjugate of row j), v into vbuf row j, tau_j, beta_j = e[j], d[j] = A[j][j]; p = tau A22 v
// (a warp per row, blockDim.x / 32 rows per block); the last block forms
// w = p - (tau/2)(p^H v) v into w buffer j % 2 and resets the counter.  m = k - j - 1 >= 1 rows.
__global__ void __launch_bounds__(HH_WARPS * 32)
    k_hh_col(double2 *__restrict__ A, int k, int j, double2 *__restrict__ vbuf, double2 *__restrict__ tau,
             double *__restrict__ d, double *__restrict__ e, double2 *__restrict__ p, double2 *__restrict__ wv,
             int pending, unsigned int *counter) {
  extern __shared__ double2 sv[];  // v, m entries
  __shared__ double red[HH_WARPS + 1];
  __shared__ double2 red2[HH_WARPS + 1];
  __shared__ double2 s_tau, s_sc, s_k;
  __shared__ int s_last;
  const int m = k - j - 1;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, T = blockDim.x, rows = T >> 5;
  const bool upd = pending != 0;  // column j - 1's update still to apply
  const double2 *pv = vbuf + (int64_t)(upd ? j - 1 : 0) * k;
  const double2 *pw = wv + (int64_t)((j + 1) & 1) * k;  // w of column j - 1
  double2 *wout = wv + (int64_t)(j & 1) * k;
  const double2 z = make_double2(0.0, 0.0);
  const double2 v0 = upd ? pv[0] : z, w0 = upd ? pw[0] : z;
  const double2 *rowj = A + (int64_t)j * k + j + 1;  // rowj[c] = conj(x_c), once brought up to date
  double ss = 0.0;
  for (int c = 1 + tid; c < m; c += T) {
    const double2 a = upd ? hh_updated(rowj[c], v0, w0, pv[c + 1], pw[c + 1]) : rowj[c];
    ss += a.x * a.x + a.y * a.y;
  }
  ss = block_sum(ss, red);
  if (tid == 0) {
    const double2 r0 = upd ? hh_updated(rowj[0], v0, w0, pv[1], pw[1]) : rowj[0];
    const double2 al = make_double2(r0.x, -r0.y);
    double2 tv, sc;
    double beta;
    if (ss == 0.0 && al.y == 0.0) {  // already in tridiagonal form: H = I
      tv = make_double2(0.0, 0.0);
      sc = make_double2(0.0, 0.0);
      beta = al.x;
    } else {
      const double nrm = sqrt(al.x * al.x + al.y * al.y + ss);
      beta = al.x >= 0.0 ? -nrm : nrm;
      tv = make_double2((beta - al.x) / beta, -al.y / beta);
      const double2 df = make_double2(al.x - beta, al.y);
      const double den = df.x * df.x + df.y * df.y;
      sc = make_double2(df.x / den, -df.y / den);  // 1 / (alpha - beta)
    }
    s_tau = tv;
    s_sc = sc;
    if (blockIdx.x == 0) {
      tau[j] = tv;
      e[j] = beta;
      const double2 ajj = A[(int64_t)j * k + j];
      d[j] = upd ? hh_updated(ajj, v0, w0, v0, w0).x : ajj.x;
    }
  }
  __syncthreads();
  const double2 sc = s_sc, tv = s_tau;
  for (int c = tid; c < m; c += T) {
    double2 v;
    if (c == 0) {
      v = make_double2(1.0, 0.0);
    } else {
      const double2 a = upd ? hh_updated(rowj[c], v0, w0, pv[c + 1], pw[c + 1]) : rowj[c];
      v = cmul(make_double2(a.x, -a.y), sc);
    }
    sv[c] = v;
    if (blockIdx.x == 0) vbuf[(int64_t)j * k + c] = v;
  }
  __syncthreads();
  const int r = blockIdx.x * rows + wid;
  if (r < m) {
    double2 *row = A + (int64_t)(j + 1 + r) * k + j + 1;
    const double2 vr = upd ? pv[r + 1] : z, wr = upd ? pw[r + 1] : z;
    double2 s = make_double2(0.0, 0.0);
    for (int c = lane; c < m; c += 32) {
      double2 a = row[c];
      if (upd) {
        a = hh_updated(a, vr, wr, pv[c + 1], pw[c + 1]);
        row[c] = a;
      }
      const double2 v = sv[c];
      s.x += a.x * v.x - a.y * v.y;
      s.y += a.x * v.y + a.y * v.x;
    }
    for (int o = 16; o; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) p[r] = cmul(tv, s);
  }
  // the last block to arrive forms w (no block waits for another)
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double2 dt = make_double2(0.0, 0.0);  // p^H v
  for (int c = tid; c < m; c += T) {
    const double2 pc = __ldcg(p + c), v = sv[c];
    dt.x += pc.x * v.x + pc.y * v.y;
    dt.y += pc.x * v.y - pc.y * v.x;
  }
  dt = block_sum2(dt, red2);
  if (tid == 0) {
    const double2 h = cmul(tv, dt);
    s_k = make_double2(0.5 * h.x, 0.5 * h.y);
    *counter = 0u;
  }
  __syncthreads();
  const double2 kk = s_k;
  for (int c = tid; c < m; c += T) {
    const double2 pc = __ldcg(p + c), kv = cmul(kk, sv[c]);
    wout[c] = make_double2(pc.x - kv.x, pc.y - kv.y);
  }
}

// A22 -= v w^H + w v^H over the trailing m x m block of column j, as its own launch (the large
// columns: there every block of the next column would repeat the update of row j); 32 x 32
// tiles, 8 rows per pass.
__global__ void __launch_bounds__(256)
    k_hh_rank2(double2 *__restrict__ A, int k, int j, const double2 *__restrict__ vbuf, const double2 *__restrict__ w) {
  const int m = k - j - 1;
  const int c = blockIdx.x * 32 + (threadIdx.x & 31);
  if (c >= m) return;
  const double2 *v = vbuf + (int64_t)j * k;
  const double2 vc = v[c], wc = w[c];
  const int r1 = min(m, (int)blockIdx.y * 32 + 32);
  for (int r = blockIdx.y * 32 + (threadIdx.x >> 5); r < r1; r += 8) {
    double2 *a = A + (int64_t)(j + 1 + r) * k + j + 1 + c;
    *a = hh_updated(*a, v[r], w[r], vc, wc);
  }
}

// d[k-1]: the last diagonal entry, after the rank-2 update of column k - 2 when that is pending
__global__ void k_hh_last(const double2 *A, int k, const double2 *vbuf, const double2 *wv, int pending, double *d) {
  const double2 a = A[(int64_t)(k - 1) * k + k - 1];
  if (!pending) {
    d[k - 1] = a.x;
    return;
  }
  const double2 v = vbuf[(int64_t)(k - 2) * k], w = wv[(int64_t)((k - 2) & 1) * k];
  d[k - 1] = hh_updated(a, v, w, v, w).x;
}

// number of eigenvalues of T below x (Sturm count; tiny pivots replaced by -pivmin)
__device__ int tri_sturm(const double *__restrict__ d, const double *__restrict__ e2, int k, double x, double pivmin) {
  double q = d[0] - x;
  if (fabs(q) <= pivmin) q = -pivmin;
  int cnt = q < 0.0;
  for (int i = 1; i < k; i++) {
    q = d[i] - x - e2[i - 1] / q;
    if (fabs(q) <= pivmin) q = -pivmin;
    cnt += q < 0.0;
  }
  return cnt;
}

// eigenvalue i of T (ascending), a warp per eigenvalue, by multisection of [gl, gu]: each round
// the 32 lanes take Sturm counts at 32 points spread evenly over the interval and keep the
// 33rd part holding eigenvalue i (count(lo) <= i < count(hi) throughout).  When the points fall
// onto the ends (an interval a few ulps wide) a round halves instead, and the search ends at the
// last representable midpoint, as a bisection does; 72 rounds resolve at least what 256
// halvings do.
__global__ void k_tri_bisect(const double *__restrict__ d, const double *__restrict__ e2, int k, double gl, double gu,
                             double pivmin, double *__restrict__ w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (i >= k) return;  // i is the same on every lane of a warp
  const double frac = (double)(lane + 1) * (1.0 / 33.0);
  double lo = gl, hi = gu;
  for (int it = 0; it < 72; it++) {
    const double mid = 0.5 * (lo + hi);
    if (!(mid > lo && mid < hi)) break;
    const double x = lo + (hi - lo) * frac;
    const unsigned above = __ballot_sync(0xffffffffu, tri_sturm(d, e2, k, x, pivmin) > i);
    const int f = above ? __ffs((int)above) - 1 : 32;  // the first point with count > i
    const double xl = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
    const double xh = __shfl_sync(0xffffffffu, x, f < 32 ? f : 31);
    const double nlo = f > 0 ? xl : lo, nhi = f < 32 ? xh : hi;
    if (nlo == lo && nhi == hi) {  // no point strictly inside: halve
      if (tri_sturm(d, e2, k, mid, pivmin) > i)
        hi = mid;
      else
        lo = mid;
    } else {
      lo = nlo;
      hi = nhi;
    }
  }
  if (lane == 0) w[i] = 0.5 * (lo + hi);
}

// T - lambda I = P L U with partial pivoting: U has the diagonal u0 and two superdiagonals
// u1, u2; ml the multipliers, pv whether rows i and i + 1 were exchanged.
__device__ void tri_factor(const double *__restrict__ d, const double *__restrict__ e, int k, double lam, double tol,
                           double *u0, double *u1, double *u2, double *ml, double *pv) {
  double cd = d[0] - lam;               // row i, column i
  double cs = k > 1 ? e[0] : 0.0;       // row i, column i + 1
  for (int i = 0; i < k - 1; i++) {
    const double sub = e[i];                        // row i + 1, column i
    const double nd = d[i + 1] - lam;               // row i + 1, column i + 1
    const double ns = i + 2 < k ? e[i + 1] : 0.0;   // row i + 1, column i + 2
    if (fabs(cd) >= fabs(sub)) {
      const double mu = cd != 0.0 ? sub / cd : 0.0;
      u0[i] = cd;
      u1[i] = cs;
      u2[i] = 0.0;
      ml[i] = mu;
      pv[i] = 0.0;
      cd = nd - mu * cs;
      cs = ns;
    } else {
      const double mu = cd / sub;
      u0[i] = sub;
      u1[i] = nd;
      u2[i] = ns;
      ml[i] = mu;
      pv[i] = 1.0;
      cd = cs - mu * nd;
      cs = -mu * ns;
    }
    if (fabs(u0[i]) < tol) u0[i] = u0[i] < 0.0 ? -tol : tol;
  }
  u0[k - 1] = fabs(cd) < tol ? (cd < 0.0 ? -tol : tol) : cd;
}

__device__ void tri_solve(int k, const double *u0, const double *u1, const double *u2, const double *ml,
                          const double *pv, double *x) {
  for (int i = 0; i < k - 1; i++) {
    if (pv[i] != 0.0) {
      const double t = x[i];
      x[i] = x[i + 1];
      x[i + 1] = t;
    }
    x[i + 1] -= ml[i] * x[i];
  }
  x[k - 1] /= u0[k - 1];
  if (k > 1) x[k - 2] = (x[k - 2] - u1[k - 2] * x[k - 1]) / u0[k - 2];
  for (int i = k - 3; i >= 0; i--) x[i] = (x[i] - u1[i] * x[i + 1] - u2[i] * x[i + 2]) / u0[i];
}

// a pseudo-random start in (-1, 1) from (vector, component, attempt)
__device__ __forceinline__ double start_value(int idx, int i, int salt) {
  uint64_t h = ((uint64_t)(uint32_t)idx << 32) ^ (uint64_t)(uint32_t)i ^ ((uint64_t)salt << 58);
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Inverse iteration, one block per cluster [cl[c], cl[c+1]); Z: nv x k, vector-major.
__global__ void __launch_bounds__(HH_INV_THREADS)
    k_tri_invit(const double *__restrict__ d, const double *__restrict__ e, int k, const double *__restrict__ w,
                const int *__restrict__ cl, int ncl, double *__restrict__ Z, double *__restrict__ scratch, double tol) {
  __shared__ double red[HH_INV_THREADS / 32 + 1];
  double *u0 = scratch + (int64_t)blockIdx.x * 5 * k, *u1 = u0 + k, *u2 = u1 + k, *ml = u2 + k, *pv = ml + k;
  for (int ci = blockIdx.x; ci < ncl; ci += gridDim.x) {
    const int cs = cl[ci], ce = cl[ci + 1];
    double prev = 0.0;
    for (int idx = cs; idx < ce; idx++) {
      double lam = w[idx];
      const double pert = 10.0 * 2.220446049250313e-16 * fabs(lam);
      if (idx > cs && lam - prev < pert) lam = prev + pert;
      prev = lam;
      double *x = Z + (int64_t)idx * k;
      for (int i = threadIdx.x; i < k; i += blockDim.x) x[i] = start_value(idx, i, 0);
      if (threadIdx.x == 0) tri_factor(d, e, k, lam, tol, u0, u1, u2, ml, pv);
      __syncthreads();
      for (int it = 0, salt = 0; it < 3; it++) {
        if (threadIdx.x == 0) tri_solve(k, u0, u1, u2, ml, pv, x);
        __syncthreads();
        for (int q = cs; q < idx; q++) {
          const double *zq = Z + (int64_t)q * k;
          double s = 0.0;
          for (int i = threadIdx.x; i < k; i += blockDim.x) s += zq[i] * x[i];
          s = block_sum(s, red);
          for (int i = threadIdx.x; i < k; i += blockDim.x) x[i] -= s * zq[i];
          __syncthreads();
        }
        double nn = 0.0;
        for (int i = threadIdx.x; i < k; i += blockDim.x) nn += x[i] * x[i];
        nn = block_sum(nn, red);
        if (!(nn > 0.0) || !(nn < 1e300)) {  // lost to the projections: start again (bounded)
          if (++salt < 8) it = -1;
          for (int i = threadIdx.x; i < k; i += blockDim.x) x[i] = start_value(idx, i, salt);
          __syncthreads();
          continue;
        }
        const double sc = 1.0 / sqrt(nn);
        for (int i = threadIdx.x; i < k; i += blockDim.x) x[i] *= sc;
        __syncthreads();
      }
    }
  }
}

// The eigenvectors of A: Zc = H_0 (H_1 (... H_(k-2) Z)); a warp per vector, the block's
// warps stepping through the reflectors together, each staged once in shared memory.
__global__ void __launch_bounds__(HH_BT_VECS * 32)
    k_hh_back(const double *__restrict__ Z, int k, int nv, const double2 *__restrict__ vbuf,
              const double2 *__restrict__ tau, double2 *__restrict__ Zc) {
  extern __shared__ double2 sv[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int c = blockIdx.x * HH_BT_VECS + wid;
  double2 *z = Zc + (int64_t)c * k;
  if (c < nv)
    for (int i = lane; i < k; i += 32) z[i] = make_double2(Z[(int64_t)c * k + i], 0.0);
  for (int j = k - 2; j >= 0; j--) {
    const int m = k - j - 1;
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) sv[i] = vbuf[(int64_t)j * k + i];
    __syncthreads();
    if (c < nv) {
      const double2 t = tau[j];
      double2 *zz = z + j + 1;
      double2 u = make_double2(0.0, 0.0);  // v^H z
      for (int i = lane; i < m; i += 32) {
        const double2 v = sv[i], a = zz[i];
        u.x += v.x * a.x + v.y * a.y;
        u.y += v.x * a.y - v.y * a.x;
      }
      for (int o = 16; o; o >>= 1) {
        u.x += __shfl_xor_sync(0xffffffffu, u.x, o);
        u.y += __shfl_xor_sync(0xffffffffu, u.y, o);
      }
      const double2 tu = cmul(t, u);
      for (int i = lane; i < m; i += 32) {
        const double2 s = cmul(sv[i], tu);
        zz[i].x -= s.x;
        zz[i].y -= s.y;
      }
    }
  }
}

// V (k x nv row-major, the eigenvectors as columns) from Zc (nv x k)
__global__ void k_hh_out(const double2 *__restrict__ Zc, int k, int nv, double2 *__restrict__ V) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)k * nv) return;
  const int i = (int)(t / nv), c = (int)(t % nv);
  V[t] = Zc[(int64_t)c * k + i];
}

// Eigenvalues ascending into w_dev (k), the eigenvectors of the lowest nv into V_dev (k x nv
// row-major); A (k x k row-major, Hermitian, full storage) is overwritten.
qg_status qg_eigh_tridiag(qg_context ctx, int k, double2 *A, double *w_dev, double2 *V_dev, int nv) {
  if (k <= 1 || k > HH_MAX_K || nv < 0 || nv > k) return QG_ERR_ARG;
  cudaStream_t s = ctx->stream;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_hh_col, cudaFuncAttributeMaxDynamicSharedMemorySize, HH_MAX_K * (int)sizeof(double2));
    cudaFuncSetAttribute(k_hh_back, cudaFuncAttributeMaxDynamicSharedMemorySize, HH_MAX_K * (int)sizeof(double2));
    attr = true;
  }
  double2 *vbuf = nullptr, *tau = nullptr, *p = nullptr, *wv = nullptr, *Zc = nullptr;
  double *d = nullptr, *e = nullptr, *e2 = nullptr, *Z = nullptr, *scratch = nullptr;
  unsigned int *counter = nullptr;
  int *cl = nullptr;
  cudaError_t ce = cudaMalloc(&vbuf, (size_t)k * k * sizeof(double2));
  if (ce == cudaSuccess) ce = cudaMalloc(&tau, (size_t)k * sizeof(double2));
  if (ce == cudaSuccess) ce = cudaMalloc(&p, (size_t)k * sizeof(double2));
  if (ce == cudaSuccess) ce = cudaMalloc(&wv, (size_t)2 * k * sizeof(double2));  // w of two columns
  if (ce == cudaSuccess) ce = cudaMalloc(&d, (size_t)k * sizeof(double));
  if (ce == cudaSuccess) ce = cudaMalloc(&e, (size_t)k * sizeof(double));
  if (ce == cudaSuccess) ce = cudaMalloc(&e2, (size_t)k * sizeof(double));
  if (ce == cudaSuccess) ce = cudaMalloc(&counter, sizeof(unsigned int));
  if (ce == cudaSuccess) ce = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e, 0, (size_t)k * sizeof(double), s);
  qg_status st = ce == cudaSuccess ? QG_OK : qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
  // 1. reduction to tridiagonal form
  int pending = 0;  // the previous column's rank-2 update is left to this column's launch
  for (int j = 0; st == QG_OK && j < k - 1; j++) {
    const int m = k - j - 1;
    k_hh_col<<<(unsigned)((m + HH_WARPS - 1) / HH_WARPS), HH_WARPS * 32, (size_t)m * sizeof(double2), s>>>(
        A, k, j, vbuf, tau, d, e, p, wv, pending, counter);
    ctx->launches++;
    pending = m < HH_FOLD_ROWS;
    if (!pending) {
      k_hh_rank2<<<dim3((unsigned)((m + 31) / 32), (unsigned)((m + 31) / 32)), 256, 0, s>>>(
          A, k, j, vbuf, wv + (size_t)(j & 1) * k);
      ctx->launches++;
    }
    if ((j & 255) == 0) st = qg_check_launch(ctx, "tridiagonal reduction");
  }
  if (st == QG_OK) {
    k_hh_last<<<1, 1, 0, s>>>(A, k, vbuf, wv, pending, d);
    ctx->launches++;
    st = qg_check_launch(ctx, "tridiagonal reduction");
  }
  std::vector<double> hd(k), he(k), he2(k, 0.0), hw;
  if (st == QG_OK) {
    ce = cudaMemcpyAsync(hd.data(), d, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(he.data(), e, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) st = qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
  }
  // 2. eigenvalues: Gershgorin interval, 1-norm, pivot floor
  double onenrm = 0.0, gl = 0.0, gu = 0.0, emax2 = 0.0;
  if (st == QG_OK) {
    for (int i = 0; i < k; i++) {
      const double r = (i > 0 ? fabs(he[i - 1]) : 0.0) + (i + 1 < k ? fabs(he[i]) : 0.0);
      onenrm = std::max(onenrm, fabs(hd[i]) + r);
      gl = i ? std::min(gl, hd[i] - r) : hd[i] - r;
      gu = i ? std::max(gu, hd[i] + r) : hd[i] + r;
      if (i + 1 < k) {
        he2[i] = he[i] * he[i];
        emax2 = std::max(emax2, he2[i]);
      }
    }
    const double pad = 2.220446049250313e-16 * onenrm * k + 1e-300;
    gl -= pad;
    gu += pad;
    const double pivmin = 2.2250738585072014e-308 * std::max(1.0, emax2);
    ce = cudaMemcpyAsync(e2, he2.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, s);
    if (ce != cudaSuccess) st = qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
    if (st == QG_OK) {
      k_tri_bisect<<<(unsigned)((k + 3) / 4), 128, 0, s>>>(d, e2, k, gl, gu, pivmin, w_dev);  // a warp each
      ctx->launches++;
      st = qg_check_launch(ctx, "bisection");
    }
  }
  // 3. eigenvectors of T, 4. back-transformation
  if (st == QG_OK && nv > 0) {
    hw.resize(nv);
    ce = cudaMemcpyAsync(hw.data(), w_dev, (size_t)nv * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) st = qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
    std::vector<int> hcl(1, 0);
    const double ortol = 1e-3 * onenrm;
    for (int i = 1; i < nv; i++)
      if (hw[i] - hw[i - 1] > ortol) hcl.push_back(i);
    hcl.push_back(nv);
    const int ncl = (int)hcl.size() - 1;
    const int grid = std::min(ncl, 1024);
    if (st == QG_OK) {
      ce = cudaMalloc(&cl, hcl.size() * sizeof(int));
      if (ce == cudaSuccess) ce = cudaMalloc(&Z, (size_t)nv * k * sizeof(double));
      if (ce == cudaSuccess) ce = cudaMalloc(&scratch, (size_t)grid * 5 * k * sizeof(double));
      if (ce == cudaSuccess) ce = cudaMalloc(&Zc, (size_t)nv * k * sizeof(double2));
      if (ce == cudaSuccess) ce = cudaMemcpyAsync(cl, hcl.data(), hcl.size() * sizeof(int), cudaMemcpyHostToDevice, s);
      if (ce != cudaSuccess) st = qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
    }
    if (st == QG_OK) {
      const double tol = 2.220446049250313e-16 * std::max(onenrm, 1e-300);
      k_tri_invit<<<(unsigned)grid, HH_INV_THREADS, 0, s>>>(d, e, k, w_dev, cl, ncl, Z, scratch, tol);
      k_hh_back<<<(unsigned)((nv + HH_BT_VECS - 1) / HH_BT_VECS), HH_BT_VECS * 32, (size_t)k * sizeof(double2), s>>>(
          Z, k, nv, vbuf, tau, Zc);
      k_hh_out<<<(unsigned)(((int64_t)k * nv + 255) / 256), 256, 0, s>>>(Zc, k, nv, V_dev);
      ctx->launches += 3;
      st = qg_check_launch(ctx, "eigenvectors");
    }
  }
  if (st == QG_OK) {
    ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) st = qg_cuda_fail(ctx, ce, "qg_eigh_tridiag");
  }
  cudaFree(vbuf);
  cudaFree(tau);
  cudaFree(p);
  cudaFree(wv);
  cudaFree(d);
  cudaFree(e);
  cudaFree(e2);
  cudaFree(counter);
  cudaFree(cl);
  cudaFree(Z);
  cudaFree(scratch);
  cudaFree(Zc);
  return st;
}
