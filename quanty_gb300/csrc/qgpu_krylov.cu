// Vector algebra, the Lanczos tridiagonalisation driver and the all-frequency continued
// fraction.
//
// Lanczos follows the reference's three-term recursion without reorthogonalisation and its
// truncation schedule (LanczosTriDiagonalizeCC, Core/Lanczos.cpp:2169-2263):
//   b0 = |v0|, v0 /= b0, drop |v0_r| <= eps;  w = H v0;  a1 = <v0|w>
//   i = 1..ntri-1:  v_i = w - a_i v_{i-1};  b_i = |v_i|;  v_i /= b_i;  drop |v_i,r| <= eps/err;
//                   err *= b_i^2/(b_i^2 + 4 gamma^2);  w = H v_i;  a_{i+1} = <v_i|w>;
//                   w -= b_i v_{i-1}
// On a basis that is closed under H, "drop" is zeroing and the growing-basis bookkeeping of
// the reference (union axpy, rehash) has no numerical effect.  Per step two kernels run: an
// axpy with the norm partials, and the fused H*psi whose gather applies the 1/b_i scale and
// the truncation on the fly, writes the stored Krylov vector, forms <v_i|H v_i> partials and
// the three-term update in its epilogue.  Two single-block kernels finish the reductions so
// the scalars stay on the device; the host reads a and b once at the end.
#include <algorithm>
#include <cmath>
#include <vector>

#include "qgpu_internal.cuh"

static const int RBLK = 256;

int qg_partial_blocks(qg_context ctx, int64_t n);
static inline int partial_blocks(qg_context ctx, int64_t n) { return qg_partial_blocks(ctx, n); }
int qg_partial_blocks(qg_context ctx, int64_t n) {
  int64_t b = (n + RBLK - 1) / RBLK;
  int64_t cap = 4LL * ctx->num_sms;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// per-vector partial sums of conj(x) y (or |x|^2 when y == nullptr) over rows
__global__ void k_dot_partial(int64_t n, int nvec, const double2 *__restrict__ x, const double2 *__restrict__ y,
                              double2 *part) {
  extern __shared__ double2 sh[];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < nvec; k++) {
    double2 s = make_double2(0.0, 0.0);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 a = x[r * nvec + k];
      if (y) {
        double2 b = y[r * nvec + k];
        s.x += a.x * b.x + a.y * b.y;
        s.y += a.x * b.y - a.y * b.x;
      } else {
        s.x += qg_norm2(a);
      }
    }
    for (int o = 16; o; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0.0, 0.0);
      for (int w = 0; w < nw; w++) {
        t.x += sh[w].x;
        t.y += sh[w].y;
      }
      part[blockIdx.x * nvec + k] = t;
    }
    __syncthreads();
  }
}

// Several vectors (rows hold nvec consecutive entries): the per-vector loops above would read
// every row once per vector, a sector at a time.  Here thread t of a block of T = m * nvec
// threads always sees entries of vector t % nvec while the block walks the flat array in
// coalesced strides of T; partial sums per vector are then combined through shared memory
// in a fixed order.
static int flat_threads(int nvec) {
  if (nvec <= 256) return nvec * (256 / nvec);
  return nvec <= 1024 ? nvec : 0;
}

__global__ void k_dot_partial_flat(int64_t len, int nvec, const double2 *__restrict__ x,
                                   const double2 *__restrict__ y, double2 *part) {
  extern __shared__ double2 sh[];
  int tid = threadIdx.x, T = blockDim.x;
  double2 s = make_double2(0.0, 0.0);
  for (int64_t i = blockIdx.x * (int64_t)T + tid; i < len; i += (int64_t)gridDim.x * T) {
    double2 a = x[i];
    if (y) {
      double2 b = y[i];
      s.x += a.x * b.x + a.y * b.y;
      s.y += a.x * b.y - a.y * b.x;
    } else {
      s.x += qg_norm2(a);
    }
  }
  sh[tid] = s;
  __syncthreads();
  if (tid < nvec) {
    double2 t = make_double2(0.0, 0.0);
    for (int j = tid; j < T; j += nvec) {
      t.x += sh[j].x;
      t.y += sh[j].y;
    }
    part[blockIdx.x * nvec + tid] = t;
  }
}

// sum nblk partials per vector (single block); out[k] = sum
__global__ void k_reduce_partials(const double2 *part, int nblk, int nvec, double2 *out) {
  __shared__ double2 sh[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < nvec; k++) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
      s.x += part[b * nvec + k].x;
      s.y += part[b * nvec + k].y;
    }
    for (int o = 16; o; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0.0, 0.0);
      for (int w = 0; w < nw; w++) {
        t.x += sh[w].x;
        t.y += sh[w].y;
      }
      out[k] = t;
    }
    __syncthreads();
  }
}

// Norm partials of the two parts of every vector (split Lanczos chains) in the orders of the
// kernels above for one part: .x the real parts, .y the imaginary parts.
__global__ void k_norm_partial_split(int64_t n, int nvec, const double2 *__restrict__ x, double2 *part) {
  extern __shared__ double2 sh[];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < nvec; k++) {
    double2 s = make_double2(0.0, 0.0);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 a = x[r * nvec + k];
      s.x += __dmul_rn(a.x, a.x);  // each product rounded alone, as in one chain
      s.y += __dmul_rn(a.y, a.y);
    }
    for (int o = 16; o; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0.0, 0.0);
      for (int w = 0; w < nw; w++) {
        t.x += sh[w].x;
        t.y += sh[w].y;
      }
      part[blockIdx.x * nvec + k] = t;
    }
    __syncthreads();
  }
}

__global__ void k_norm_partial_split_flat(int64_t len, int nvec, const double2 *__restrict__ x, double2 *part) {
  extern __shared__ double2 sh[];
  int tid = threadIdx.x, T = blockDim.x;
  double2 s = make_double2(0.0, 0.0);
  for (int64_t i = blockIdx.x * (int64_t)T + tid; i < len; i += (int64_t)gridDim.x * T) {
    double2 a = x[i];
    s.x += __dmul_rn(a.x, a.x);
    s.y += __dmul_rn(a.y, a.y);
  }
  sh[tid] = s;
  __syncthreads();
  if (tid < nvec) {
    double2 t = make_double2(0.0, 0.0);
    for (int j = tid; j < T; j += nvec) {
      t.x += sh[j].x;
      t.y += sh[j].y;
    }
    part[blockIdx.x * nvec + tid] = t;
  }
}

static void launch_dot_partial(int P, int64_t n, int nvec, const double2 *x, const double2 *y, double2 *part,
                               cudaStream_t s) {
  int T = nvec > 1 ? flat_threads(nvec) : 0;
  if (T)
    k_dot_partial_flat<<<P, T, T * sizeof(double2), s>>>(n * nvec, nvec, x, y, part);
  else
    k_dot_partial<<<P, RBLK, (RBLK / 32) * sizeof(double2), s>>>(n, nvec, x, y, part);
}

qg_status qg_dot_dev(qg_context ctx, int64_t n, int nvec, const double *x, const double *y, double *out_dev) {
  int P = partial_blocks(ctx, n);
  QG_TRY(qg_ensure_scratch(ctx, (size_t)P * nvec * 16));
  launch_dot_partial(P, n, nvec, (const double2 *)x, (const double2 *)y, (double2 *)ctx->d_scratch, ctx->stream);
  k_reduce_partials<<<1, 256, 0, ctx->stream>>>((const double2 *)ctx->d_scratch, P, nvec, (double2 *)out_dev);
  ctx->launches += 2;
  return qg_check_launch(ctx, "dot");
}

static qg_status dot_to_host(qg_context ctx, int64_t n, int nvec, const double *x, const double *y, double *host) {
  double2 *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, nvec * 16));
  qg_status st = qg_dot_dev(ctx, n, nvec, x, y, (double *)d);
  cudaError_t e = cudaSuccess;
  if (st == QG_OK) e = cudaMemcpyAsync(host, d, nvec * 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (st != QG_OK) return st;
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "dot copy");
  return QG_OK;
}

extern "C" qg_status qg_dot(qg_context ctx, int64_t n, int32_t nvec, const double *x, const double *y, double *dot_host) {
  if (!ctx || n < 0 || nvec <= 0 || !dot_host || (n && (!x || !y))) return QG_ERR_ARG;
  return dot_to_host(ctx, n, nvec, x, y, dot_host);
}

extern "C" qg_status qg_norm(qg_context ctx, int64_t n, int32_t nvec, const double *x, double *norm_host) {
  if (!ctx || n < 0 || nvec <= 0 || !norm_host || (n && !x)) return QG_ERR_ARG;
  std::vector<double> t(2 * nvec);
  QG_TRY(dot_to_host(ctx, n, nvec, x, nullptr, t.data()));
  for (int k = 0; k < nvec; k++) norm_host[k] = std::sqrt(t[2 * k]);
  return QG_OK;
}

__global__ void k_axpy(int64_t n, int nvec, const double2 *__restrict__ alpha, const double2 *__restrict__ x,
                       double2 *__restrict__ y) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * nvec) return;
  int k = (int)(i % nvec);
  double2 a = alpha[k], xv = x[i], yv = y[i];
  yv.x += a.x * xv.x - a.y * xv.y;
  yv.y += a.x * xv.y + a.y * xv.x;
  y[i] = yv;
}

extern "C" qg_status qg_axpy(qg_context ctx, int64_t n, int32_t nvec, const double *alpha_host, const double *x,
                             double *y) {
  if (!ctx || n < 0 || nvec <= 0 || !alpha_host || (n && (!x || !y))) return QG_ERR_ARG;
  if (!n) return QG_OK;
  double2 *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, nvec * 16));
  // every path from here frees d
  cudaError_t e = cudaMemcpyAsync(d, alpha_host, nvec * 16, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    int64_t tot = n * nvec;
    k_axpy<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(n, nvec, d, (const double2 *)x, (double2 *)y);
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_axpy");
  return qg_check_launch(ctx, "qg_axpy");
}

extern "C" qg_status qg_expectation(qg_context ctx, qg_operator op, qg_basis b, const double *x, int32_t nvec,
                                    double *val_host) {
  if (!ctx || !op || !b || nvec <= 0 || !val_host || op->nf != b->nf) return QG_ERR_ARG;
  if (!b->n) {
    for (int k = 0; k < 2 * nvec; k++) val_host[k] = 0;
    return QG_OK;
  }
  double *y = nullptr;
  QG_CUDA(ctx, cudaMalloc(&y, b->n * nvec * 16));
  qg_status st = qg_apply_launch(ctx, op, b, b, x, y, nvec, nullptr);
  if (st == QG_OK) st = dot_to_host(ctx, b->n, nvec, x, y, val_host);
  cudaFree(y);
  return st;
}

// ------------------------------------------------------------------ Lanczos

// v = w - a_k v_prev (a from the previous dot), norm partials of v
__global__ void k_lanczos_axpy_norm(int64_t n, int nvec, const double2 *__restrict__ w, const double2 *__restrict__ vp,
                                    const double *__restrict__ a, double2 *__restrict__ v, double2 *part, int *step) {
  extern __shared__ double2 sh[];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) *step += 1;  // the step this kernel opens
  for (int k = 0; k < nvec; k++) {
    double ak = a[k];
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 wv = w[r * nvec + k], pv = vp[r * nvec + k];
      double2 o = qg_axpy2(wv, ak, pv);
      v[r * nvec + k] = o;
      s += qg_norm2(o);
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sh[wid].x = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w2 = 0; w2 < nw; w2++) t += sh[w2].x;
      part[blockIdx.x * nvec + k] = make_double2(t, 0.0);
    }
    __syncthreads();
  }
}

// the same for several vectors, in the flat layout of k_dot_partial_flat
__global__ void k_lanczos_axpy_norm_flat(int64_t len, int nvec, const double2 *__restrict__ w,
                                         const double2 *__restrict__ vp, const double *__restrict__ a,
                                         double2 *__restrict__ v, double2 *part, int *step) {
  extern __shared__ double2 sh[];
  int tid = threadIdx.x, T = blockDim.x;
  if (blockIdx.x == 0 && tid == 0) *step += 1;  // the step this kernel opens
  double ak = a[tid % nvec];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)T + tid; i < len; i += (int64_t)gridDim.x * T) {
    double2 wv = w[i], pv = vp[i];
    double2 o = qg_axpy2(wv, ak, pv);
    v[i] = o;
    s += qg_norm2(o);
  }
  sh[tid].x = s;
  __syncthreads();
  if (tid < nvec) {
    double t = 0;
    for (int j = tid; j < T; j += nvec) t += sh[j].x;
    part[blockIdx.x * nvec + tid] = make_double2(t, 0.0);
  }
}

// The same for split chains: part k.x of every row with a[2k], part k.y with a[2k + 1]; the
// norm partials per part (.x, .y), each in its one-part kernel's order and arithmetic.
__global__ void k_lanczos_axpy_norm_split(int64_t n, int nvec, const double2 *__restrict__ w,
                                          const double2 *__restrict__ vp, const double *__restrict__ a,
                                          double2 *__restrict__ v, double2 *part, int *step) {
  extern __shared__ double2 sh[];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) *step += 1;  // the step this kernel opens
  for (int k = 0; k < nvec; k++) {
    const double aa = a[2 * k], ab = a[2 * k + 1];
    double sa = 0.0, sb = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
      double2 wv = w[r * nvec + k], pv = vp[r * nvec + k];
      double2 o = make_double2(fma(-aa, pv.x, wv.x), fma(-ab, pv.y, wv.y));
      v[r * nvec + k] = o;
      sa += __dmul_rn(o.x, o.x);
      sb += __dmul_rn(o.y, o.y);
    }
    for (int o = 16; o; o >>= 1) {
      sa += __shfl_xor_sync(0xffffffffu, sa, o);
      sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) sh[wid] = make_double2(sa, sb);
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0, tb = 0;
      for (int w2 = 0; w2 < nw; w2++) ta += sh[w2].x;
      for (int w2 = 0; w2 < nw; w2++) tb += sh[w2].y;
      part[blockIdx.x * nvec + k] = make_double2(ta, tb);
    }
    __syncthreads();
  }
}

__global__ void k_lanczos_axpy_norm_split_flat(int64_t len, int nvec, const double2 *__restrict__ w,
                                               const double2 *__restrict__ vp, const double *__restrict__ a,
                                               double2 *__restrict__ v, double2 *part, int *step) {
  extern __shared__ double2 sh[];
  int tid = threadIdx.x, T = blockDim.x;
  if (blockIdx.x == 0 && tid == 0) *step += 1;  // the step this kernel opens
  const double aa = a[2 * (tid % nvec)], ab = a[2 * (tid % nvec) + 1];
  double sa = 0.0, sb = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)T + tid; i < len; i += (int64_t)gridDim.x * T) {
    double2 wv = w[i], pv = vp[i];
    double2 o = make_double2(fma(-aa, pv.x, wv.x), fma(-ab, pv.y, wv.y));
    v[i] = o;
    sa += __dmul_rn(o.x, o.x);
    sb += __dmul_rn(o.y, o.y);
  }
  sh[tid] = make_double2(sa, sb);
  __syncthreads();
  if (tid < nvec) {
    double ta = 0, tb = 0;
    for (int j = tid; j < T; j += nvec) ta += sh[j].x;
    for (int j = tid; j < T; j += nvec) tb += sh[j].y;
    part[blockIdx.x * nvec + tid] = make_double2(ta, tb);
  }
}

// Sum of the .x parts of vector k's partials in a fixed order, by one block: threads over the
// partials with four independent accumulators (so a thread's loads overlap instead of waiting
// on one another), a shuffle tree, then the warps' sums in order.  The total on thread 0.
// c: 0 sums the .x parts, 1 the .y parts (the second chain of a split vector)
__device__ double fin_sum(const double2 *__restrict__ part, int nblk, int nvec, int k, double *sh, int c = 0) {
  const int T = blockDim.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double *pd = reinterpret_cast<const double *>(part) + c;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  int b = threadIdx.x;
  for (; b + 3 * T < nblk; b += 4 * T) {
    s0 += pd[2 * ((int64_t)b * nvec + k)];
    s1 += pd[2 * ((int64_t)(b + T) * nvec + k)];
    s2 += pd[2 * ((int64_t)(b + 2 * T) * nvec + k)];
    s3 += pd[2 * ((int64_t)(b + 3 * T) * nvec + k)];
  }
  for (; b < nblk; b += T) s0 += pd[2 * ((int64_t)b * nvec + k)];
  double s = (s0 + s1) + (s2 + s3);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sh[wid] = s;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < nw; w++) t += sh[w];
  return t;
}

#define QG_FIN_THREADS 512

// a[k] <- Re(sum of dot partials), one block per chain; also stores a into the history at
// column *step + 1.  The step counter is advanced by the next step's first kernel
// (k_lanczos_axpy_norm*), after every block here has read it, so a captured step can be
// replayed.  split: chain k is part k & 1 of vector k >> 1.
__global__ void __launch_bounds__(QG_FIN_THREADS) k_fin_a(const double2 *part, int nblk, int nvec, double *a_now,
                                                          double *a_hist, int stride, const int *step, int split) {
  __shared__ double sh[32];
  const int k = blockIdx.x;
  const int col = *step + 1;
  double t = split ? fin_sum(part, nblk, nvec, k >> 1, sh, k & 1) : fin_sum(part, nblk, nvec, k, sh);
  if (threadIdx.x == 0) {
    a_now[k] = t;
    a_hist[k * stride + col] = t;
  }
}

// b = sqrt(sum of norm partials) into the history at column *step, one block per vector;
// scale = 1/b (0 for an empty vector); truncation threshold (eps/err)^2 with the err before
// this step's update; err *= b^2/(b^2+4 gamma^2)
__global__ void __launch_bounds__(QG_FIN_THREADS) k_fin_b(const double2 *part, int nblk, int nvec, double *b_now,
                                                          double *b_hist, int stride, const int *step, double *scale,
                                                          double *thr2, double *err, double eps, double gamma,
                                                          int first, int split) {
  __shared__ double sh[32];
  const int k = blockIdx.x;
  const int col = *step;
  double t = split ? fin_sum(part, nblk, nvec, k >> 1, sh, k & 1) : fin_sum(part, nblk, nvec, k, sh);
  if (threadIdx.x == 0) {
    double b, sc, th2, e = first ? 1.0 : err[k];
    qg_lanczos_norm_scalars(t, first != 0, eps, gamma, b, sc, th2, e);
    b_now[k] = b;
    b_hist[k * stride + col] = b;
    scale[k] = sc;
    thr2[k] = th2;
    err[k] = e;
  }
}

// v_out = truncate(v_in * scale) per vector (the reference keeps |a|^2 > (eps/err)^2)
__global__ void k_scale_trunc(int64_t n, int nvec, const double2 *__restrict__ vin, const double *__restrict__ scale,
                              const double *__restrict__ thr2, double2 *__restrict__ vout) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * nvec) return;
  int k = (int)(i % nvec);
  double2 v = vin[i];
  double sc = scale[k];
  v.x *= sc;
  v.y *= sc;
  if (!(qg_norm2(v) > thr2[k])) v = make_double2(0.0, 0.0);
  vout[i] = v;
}

// split chains: part .x with scale[2k], thr2[2k]; part .y with scale[2k + 1], thr2[2k + 1]
__global__ void k_scale_trunc_split(int64_t n, int nvec, const double2 *__restrict__ vin,
                                    const double *__restrict__ scale, const double *__restrict__ thr2,
                                    double2 *__restrict__ vout) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * nvec) return;
  int k = (int)(i % nvec);
  double2 v = vin[i];
  v.x *= scale[2 * k];
  v.y *= scale[2 * k + 1];
  if (!(__dmul_rn(v.x, v.x) > thr2[2 * k])) v.x = 0.0;
  if (!(__dmul_rn(v.y, v.y) > thr2[2 * k + 1])) v.y = 0.0;
  vout[i] = v;
}

// One real chain (x one real number per row): the start norm, the axpy with its norm and the
// scaling with truncation, each in the order and arithmetic its complex kernel above uses for
// a vector whose imaginary part is zero.
__global__ void k_norm_partial_real(int64_t n, const double *__restrict__ x, double2 *part) {
  __shared__ double sh[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double s = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    s += __dmul_rn(x[r], x[r]);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sh[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += sh[w];
    part[blockIdx.x] = make_double2(t, 0.0);
  }
}

__global__ void k_lanczos_axpy_norm_real(int64_t n, const double *__restrict__ w, const double *__restrict__ vp,
                                         const double *__restrict__ a, double *__restrict__ v, double2 *part,
                                         int *step) {
  __shared__ double sh[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) *step += 1;  // the step this kernel opens
  const double ak = a[0];
  double s = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double o = fma(-ak, vp[r], w[r]);
    v[r] = o;
    s += __dmul_rn(o, o);
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sh[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w2 = 0; w2 < nw; w2++) t += sh[w2];
    part[blockIdx.x] = make_double2(t, 0.0);
  }
}

__global__ void k_scale_trunc_real(int64_t n, const double *__restrict__ vin, const double *__restrict__ scale,
                                   const double *__restrict__ thr2, double *__restrict__ vout) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = vin[i] * scale[0];
  if (!(__dmul_rn(v, v) > thr2[0])) v = 0.0;
  vout[i] = v;
}

// out[r] = part c (0 real, 1 imaginary) of v[r]
__global__ void k_take_part(int64_t n, const double2 *__restrict__ v, int c, double *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = c ? v[i].y : v[i].x;
}

__global__ void k_zero(double *p, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

__global__ void k_copy_col(const double2 *src, double2 *dst, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

// ------------------------------------------------------------------ small bases: a persistent kernel

// Bases this small run every Lanczos chain as one block that keeps its three vectors in shared
// memory and makes all NTri steps in one launch (a persistent kernel: no launch, graph node or
// host round trip per step).  Several chains run side by side, one per block.
#define QG_SMALL_N 2048      // rows: three vectors of 16 B in shared memory (96 KB)
#define QG_SMALL_NNZ 32768   // terms of the explicit rows: one block's FP64 work per step

// Each block repeats the arithmetic and summation orders of the general path for one vector --
// the list apply with its fused epilogue (rows in blocks of 256, a row's terms in the list
// kernel's order, the block partial as fused_dot_partials forms it), the axpy with its norm and
// the start norm (per 256 rows: a warp-shuffle tree, then the eight warps in order), the scaling
// with truncation, and the sum of the partials (k_fin_a / k_fin_b: for at most 32 partials, the
// shuffle tree of warp 0) -- so a chain's coefficients are bitwise those of qg_lanczos_tridiag's
// general path with one vector.  v0: n x nvec row-major; chain k = blockIdx.x.
template <bool KRY>
__global__ void __launch_bounds__(256)
    k_lanczos_small(int n, int nvec, const int *__restrict__ rowptr, const int *__restrict__ col,
                    const double2 *__restrict__ val, const unsigned char *__restrict__ kind,
                    const double2 *__restrict__ v0, int ntri, double eps, double gamma, double *__restrict__ a_hist,
                    double *__restrict__ b_hist, double2 *__restrict__ krylov) {
  extern __shared__ double2 sm_vec[];
  __shared__ double s_part[32], s_warp[8], s_dot[256], s_seg[8], s_scal[4];
  const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int P = (n + 255) / 256;
  double2 *V = sm_vec, *VP = sm_vec + n, *Wv = sm_vec + 2 * n;
  double err = 1.0;  // thread 0
  // the partial of 256 rows as k_dot_partial / k_lanczos_axpy_norm form it
  auto rows_part = [&](double sv, int vb) {
    for (int o = 16; o; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
    if (lane == 0) s_warp[wid] = sv;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < 8; w++) t += s_warp[w];
      s_part[vb] = t;
    }
    __syncthreads();
  };
  // the sum of the P partials as fin_sum forms it: warp 0's shuffle tree (lane 0)
  auto fin = [&]() -> double {
    double t = 0.0;
    if (wid == 0) {
      double s0 = 0.0;
      if (lane < P) s0 += s_part[lane];
      double sv = (s0 + 0.0) + (0.0 + 0.0);
      for (int o = 16; o; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
      t = 0.0 + sv;
    }
    return t;  // thread 0
  };
  // the norm's scalars into s_scal[1..3] (b, scale, thr2) and the history at column col
  auto norm_scalars = [&](bool first, int c) {
    const double t = fin();
    if (tid == 0) {
      double bb, sc, th2;
      qg_lanczos_norm_scalars(t, first, eps, gamma, bb, sc, th2, err);
      b_hist[(int64_t)k * ntri + c] = bb;
      s_scal[1] = bb;
      s_scal[2] = sc;
      s_scal[3] = th2;
    }
    __syncthreads();
  };
  // dst = truncate(src * scale), and the Krylov vector of step c
  auto normalise = [&](const double2 *src, double2 *dst, int c) {
    const double sc = s_scal[2], th2 = s_scal[3];
    for (int r = tid; r < n; r += 256) {
      double2 v = src[r];
      v.x *= sc;
      v.y *= sc;
      if (!(qg_norm2(v) > th2)) v = make_double2(0.0, 0.0);
      dst[r] = v;
      if (KRY) krylov[((int64_t)c * n + r) * nvec + k] = v;
    }
    __syncthreads();
  };
  // Wv = H V - beta prev (prev null: zero), a = Re <V|H V> into s_scal[0] and the history
  auto apply = [&](const double2 *prev, double beta, int c) {
    for (int vb = 0; vb < P; vb++) {
      const int r = vb * 256 + tid;
      double dv = 0.0;
      if (r < n) {
        double2 acc = make_double2(0.0, 0.0);
        const int e1 = rowptr[r + 1];
        for (int e = rowptr[r]; e < e1; e++) {
          const double2 v = val[e], xv = V[col[e]];
          const unsigned char kd = kind[e];
          if (kd < 2)
            acc = qg_diag_mul(v, xv, kd == 1);
          else if (kd == 3)
            qg_cmac(acc, v.x, v.y, true, xv);
          else
            qg_cmac(acc, v.x, 0.0, false, xv);
        }
        dv = qg_redot(V[r], acc);
        Wv[r] = qg_axpy2(acc, beta, prev ? prev[r] : make_double2(0.0, 0.0));
      }
      s_dot[tid] = dv;
      __syncthreads();
      if (tid < 8) {
        double t = 0.0;
        for (int q = 0; q < 32; q++) t += s_dot[tid * 32 + q];
        s_seg[tid] = t;
      }
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int g = 0; g < 8; g++) t += s_seg[g];
        s_part[vb] = t;
      }
      __syncthreads();
    }
    const double a = fin();
    if (tid == 0) {
      a_hist[(int64_t)k * (ntri + 1) + c] = a;
      s_scal[0] = a;
    }
    __syncthreads();
  };
  // step 0: b0 = |v0|, v = truncate(v0 / b0), w = H v, a1
  for (int vb = 0; vb < P; vb++) {
    const int r = vb * 256 + tid;
    double sv = 0.0;
    if (r < n) sv += qg_norm2(v0[(int64_t)r * nvec + k]);
    rows_part(sv, vb);
  }
  norm_scalars(true, 0);
  for (int r = tid; r < n; r += 256) Wv[r] = v0[(int64_t)r * nvec + k];
  __syncthreads();
  normalise(Wv, V, 0);
  apply(nullptr, 0.0, 1);
  for (int i = 1; i < ntri; i++) {
    // vraw = w - a v (in place of w) and its norm
    const double a = s_scal[0];
    for (int vb = 0; vb < P; vb++) {
      const int r = vb * 256 + tid;
      double sv = 0.0;
      if (r < n) {
        const double2 o = qg_axpy2(Wv[r], a, V[r]);
        Wv[r] = o;
        sv += qg_norm2(o);
      }
      rows_part(sv, vb);
    }
    norm_scalars(false, i);
    normalise(Wv, VP, i);  // VP held v_(i-2): now v_i
    double2 *t = V;
    V = VP;
    VP = t;
    apply(VP, s_scal[1], i + 1);
  }
}

// The persistent path for nvec chains on a small basis; *done = false when it does not apply
// (no connection lists, too many rows or terms), leaving the work to the general path.
static qg_status lanczos_small(qg_context ctx, qg_operator op, qg_basis b, const double *v0_dev, int nvec, int ntri,
                               double eps, double gamma, double *a_host, double *b_host, double *krylov_dev,
                               bool *done) {
  *done = false;
  if (!ctx->small_lanczos || b->n > QG_SMALL_N || nvec > 65535) return QG_OK;
  SmallCsr csr;
  QG_TRY(qg_small_csr(ctx, op, b, QG_SMALL_NNZ, &csr));
  if (!csr.rowptr) return QG_OK;
  const int n = (int)b->n;
  cudaStream_t s = ctx->stream;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_lanczos_small<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         3 * QG_SMALL_N * (int)sizeof(double2));
    cudaFuncSetAttribute(k_lanczos_small<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         3 * QG_SMALL_N * (int)sizeof(double2));
    attr = true;
  }
  double *ah = nullptr, *bh = nullptr;
  cudaError_t e = cudaMalloc(&ah, (size_t)nvec * (ntri + 1) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&bh, (size_t)nvec * ntri * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(ah, 0, (size_t)nvec * (ntri + 1) * sizeof(double), s);
  qg_status st = e == cudaSuccess ? QG_OK : qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
  if (st == QG_OK) {
    const size_t smem = (size_t)3 * n * sizeof(double2);
    if (krylov_dev)
      k_lanczos_small<true><<<(unsigned)nvec, 256, smem, s>>>(n, nvec, csr.rowptr, csr.col, csr.val, csr.kind,
                                                              (const double2 *)v0_dev, ntri, eps, gamma, ah, bh,
                                                              (double2 *)krylov_dev);
    else
      k_lanczos_small<false><<<(unsigned)nvec, 256, smem, s>>>(n, nvec, csr.rowptr, csr.col, csr.val, csr.kind,
                                                               (const double2 *)v0_dev, ntri, eps, gamma, ah, bh,
                                                               nullptr);
    ctx->launches++;
    st = qg_check_launch(ctx, "small-basis Lanczos");
  }
  if (st == QG_OK) {
    e = cudaMemcpyAsync(a_host, ah, (size_t)nvec * (ntri + 1) * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b_host, bh, (size_t)nvec * ntri * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
  }
  cudaStreamSynchronize(s);
  cudaFree(ah);
  cudaFree(bh);
  qg_small_csr_free(csr);
  if (st == QG_OK) {
    for (int q = 0; q < nvec; q++) a_host[q * (ntri + 1)] = 0.0;
    *done = true;
  }
  return st;
}

extern "C" qg_status qg_set_small_basis_lanczos(qg_context ctx, int32_t on) {
  if (!ctx) return QG_ERR_ARG;
  ctx->small_lanczos = on != 0;
  return QG_OK;
}

// The general path: nvec vectors of n rows, every step on the device.  split: each vector holds
// two real chains (real and imaginary parts; a real operator with connection lists), chain
// 2k + c being part c of vector k; the coefficients of 2 nvec chains come back.
// rv: one real chain, v0_dev one real number per row (nvec 1).
static qg_status lanczos_general(qg_context ctx, qg_operator op, qg_basis b, const double *v0_dev, int nvec,
                                 int ntri, double eps, double gamma, double *a_host, double *b_host,
                                 double *krylov_dev, int split, int rv = 0) {
  cudaStream_t s = ctx->stream;
  int64_t n = b->n;
  const int nchain = split ? 2 * nvec : nvec;
  int64_t len = n * nvec;  // complex entries per block vector
  int P = partial_blocks(ctx, n);
  int Papply = qg_apply_grid(b);
  // device state
  double2 *vp = nullptr, *vc = nullptr, *w = nullptr, *w2 = nullptr, *vraw = nullptr, *zero = nullptr;
  double2 *npart = nullptr, *dpart = nullptr;
  double *scal = nullptr;  // a_now, b_now, scale, thr2, err, zero_beta, a_hist, b_hist
  size_t vb = std::max<int64_t>(len, 1) * 16;
  cudaError_t e = cudaSuccess;
#define ALLOC(p, bytes) \
  if (e == cudaSuccess) e = cudaMalloc((void **)&p, bytes)
  ALLOC(vp, vb);
  ALLOC(vc, vb);
  ALLOC(w, vb);
  ALLOC(w2, vb);
  ALLOC(vraw, vb);
  ALLOC(zero, vb);
  ALLOC(npart, (size_t)P * nvec * 16);
  ALLOC(dpart, (size_t)Papply * nvec * 16);
  // the scalars (one per chain), then one slot for the device step counter (zeroed with them)
  size_t nscal = 6 * (size_t)nchain + (size_t)nchain * (ntri + 1) + (size_t)nchain * ntri + 1;
  ALLOC(scal, nscal * 8);
#undef ALLOC
  if (e != cudaSuccess) {
    cudaFree(vp); cudaFree(vc); cudaFree(w); cudaFree(w2); cudaFree(vraw); cudaFree(zero);
    cudaFree(npart); cudaFree(dpart); cudaFree(scal);
    ctx->last_error = "qg_lanczos_tridiag: out of device memory";
    return QG_ERR_OOM;
  }
  double *a_now = scal, *b_now = scal + nchain, *scale = scal + 2 * nchain, *thr2 = scal + 3 * nchain,
         *err = scal + 4 * nchain, *zb = scal + 5 * nchain;
  double *a_hist = scal + 6 * nchain, *b_hist = a_hist + (size_t)nchain * (ntri + 1);
  int *step_ctr = reinterpret_cast<int *>(scal + nscal - 1);
  qg_status st = QG_OK;
  k_zero<<<(unsigned)((nscal + 255) / 256), 256, 0, s>>>(scal, (int64_t)nscal);
  ctx->launches++;
  qg_status st0 = qg_check_launch(ctx, "lanczos state");
  if (st0 == QG_OK) {
    cudaError_t me = cudaMemsetAsync(zero, 0, vb, s);
    if (me != cudaSuccess) st0 = qg_cuda_fail(ctx, me, "lanczos zero vector");
  }
  if (st0 != QG_OK) {
    cudaFree(vp); cudaFree(vc); cudaFree(w); cudaFree(w2); cudaFree(vraw); cudaFree(zero);
    cudaFree(npart); cudaFree(dpart); cudaFree(scal);
    return st0;
  }
  // the normalised, truncated Krylov vector vc from a raw vector: for one vector the same
  // kernel also writes it into the basis' hash slots for the gather
  // (with connection lists the apply gathers from vc itself and the slots are not needed)
  const bool pack1 = !split && !rv && nvec == 1 && !qg_apply_uses_lists(op, b);
  auto normalise = [&](const double2 *raw) -> qg_status {
    if (pack1) return qg_pack(ctx, b, (const double *)raw, 1, scale, thr2, (double *)vc);
    if (rv)
      k_scale_trunc_real<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, (const double *)raw, scale, thr2,
                                                                      (double *)vc);
    else if (split)
      k_scale_trunc_split<<<(unsigned)((len + 255) / 256), 256, 0, s>>>(n, nvec, raw, scale, thr2, vc);
    else
      k_scale_trunc<<<(unsigned)((len + 255) / 256), 256, 0, s>>>(n, nvec, raw, scale, thr2, vc);
    ctx->launches++;
    return qg_check_launch(ctx, "scale");
  };
  // step 0: b0 = |v0|, scale, threshold eps (err = 1)
  if (rv) {
    k_norm_partial_real<<<P, RBLK, 0, s>>>(n, v0_dev, npart);
  } else if (split) {
    int T = nvec > 1 ? flat_threads(nvec) : 0;
    if (T)
      k_norm_partial_split_flat<<<P, T, T * sizeof(double2), s>>>(len, nvec, (const double2 *)v0_dev, npart);
    else
      k_norm_partial_split<<<P, RBLK, (RBLK / 32) * sizeof(double2), s>>>(n, nvec, (const double2 *)v0_dev, npart);
  } else {
    launch_dot_partial(P, n, nvec, (const double2 *)v0_dev, nullptr, npart, s);
  }
  k_fin_b<<<nchain, QG_FIN_THREADS, 0, s>>>(npart, P, nvec, b_now, b_hist, ntri, step_ctr, scale, thr2, err, eps,
                                           gamma, 1, split);
  ctx->launches += 2;
  st = qg_check_launch(ctx, "lanczos start norm");
  ApplyFuse fz;
  fz.prev = zero;
  fz.beta = zb;
  fz.dot_part = dpart;
  fz.split = split;
  fz.real_vector = rv;
  if (st == QG_OK) st = normalise((const double2 *)v0_dev);
  if (st == QG_OK)
    st = qg_apply_strided(ctx, op, b, b, (const double *)vc, nvec, (double *)w, nvec, nvec, &fz, pack1);
  if (st == QG_OK && krylov_dev)
    e = cudaMemcpyAsync(krylov_dev, vc, len * 16, cudaMemcpyDeviceToDevice, s);
  if (st == QG_OK) {
    k_fin_a<<<nchain, QG_FIN_THREADS, 0, s>>>(dpart, Papply, nvec, a_now, a_hist, ntri + 1, step_ctr, split);
    ctx->launches++;
  }
  // one step: every scalar stays on the device
  auto step = [&](int i) -> qg_status {
    std::swap(vp, vc);  // vp = v_{i-1}
    int T = nvec > 1 ? flat_threads(nvec) : 0;
    if (rv)
      k_lanczos_axpy_norm_real<<<P, RBLK, 0, s>>>(n, (const double *)w, (const double *)vp, a_now, (double *)vraw,
                                                  npart, step_ctr);
    else if (split && T)
      k_lanczos_axpy_norm_split_flat<<<P, T, T * sizeof(double2), s>>>(len, nvec, w, vp, a_now, vraw, npart,
                                                                       step_ctr);
    else if (split)
      k_lanczos_axpy_norm_split<<<P, RBLK, (RBLK / 32) * sizeof(double2), s>>>(n, nvec, w, vp, a_now, vraw, npart,
                                                                               step_ctr);
    else if (T)
      k_lanczos_axpy_norm_flat<<<P, T, T * sizeof(double2), s>>>(len, nvec, w, vp, a_now, vraw, npart, step_ctr);
    else
      k_lanczos_axpy_norm<<<P, RBLK, (RBLK / 32) * sizeof(double2), s>>>(n, nvec, w, vp, a_now, vraw, npart, step_ctr);
    k_fin_b<<<nchain, QG_FIN_THREADS, 0, s>>>(npart, P, nvec, b_now, b_hist, ntri, step_ctr, scale, thr2, err, eps,
                                             gamma, 0, split);
    ctx->launches += 2;
    qg_status sst = normalise(vraw);
    if (sst != QG_OK) return sst;
    fz.prev = vp;
    fz.beta = b_now;
    sst = qg_apply_strided(ctx, op, b, b, (const double *)vc, nvec, (double *)w2, nvec, nvec, &fz, pack1);
    std::swap(w, w2);
    if (sst == QG_OK && krylov_dev) {
      cudaError_t ce = cudaMemcpyAsync(krylov_dev + 2 * (size_t)i * len, vc, len * 16, cudaMemcpyDeviceToDevice, s);
      if (ce != cudaSuccess) return qg_cuda_fail(ctx, ce, "krylov copy");
    }
    k_fin_a<<<nchain, QG_FIN_THREADS, 0, s>>>(dpart, Papply, nvec, a_now, a_hist, ntri + 1, step_ctr, split);
    ctx->launches++;
    return sst;
  };
  // Steps 1 .. ntri-1 as CUDA graphs.  The buffer roles repeat every two steps and the step's
  // column comes from the device counter, so without stored Krylov vectors two steps are
  // captured once and replayed (ntri-1)/2 times (an odd last step runs directly); with stored
  // Krylov vectors, whose copy offset depends on the step, the whole sequence is captured.
  // If capture fails, the steps run as direct launches.
  bool graphed = false;
  if (st == QG_OK && e == cudaSuccess && ntri > 2 && ctx->use_graphs) {
    double2 *sv[6] = {vp, vc, w, w2, vraw, zero};
    int64_t l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    qg_status cst = QG_OK;
    const int span = krylov_dev ? ntri - 1 : 2;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (int i = 1; i <= span && cst == QG_OK; i++) cst = step(i);
      cudaError_t ee = cudaStreamEndCapture(s, &graph);
      if (ee == cudaSuccess && cst == QG_OK && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) graphed = true;
    }
    if (graphed) {
      const int reps = krylov_dev ? 1 : (ntri - 1) / 2;
      const int64_t per = ctx->launches - l0;  // kernels of one replay, counted while capturing
      for (int r = 0; r < reps && st == QG_OK; r++) {
        cudaError_t le = cudaGraphLaunch(exec, s);
        if (le != cudaSuccess) st = qg_cuda_fail(ctx, le, "lanczos graph launch");
      }
      ctx->launches = l0 + per * reps;
      // the buffer roles are those before step 1 again, as for every odd step
      if (st == QG_OK && !krylov_dev && (ntri - 1) % 2) st = step(ntri - 1);
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (!graphed) {
      cudaGetLastError();
      // nothing captured ran: restore the buffer roles and run the steps directly
      vp = sv[0];
      vc = sv[1];
      w = sv[2];
      w2 = sv[3];
      ctx->launches = l0;
    }
  }
  for (int i = 1; !graphed && i < ntri && st == QG_OK && e == cudaSuccess; i++) st = step(i);
  if (st == QG_OK && e == cudaSuccess) {
    e = cudaMemcpyAsync(a_host, a_hist, (size_t)nchain * (ntri + 1) * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b_host, b_hist, (size_t)nchain * ntri * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess && st == QG_OK) st = qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
  cudaStreamSynchronize(s);
  cudaFree(vp); cudaFree(vc); cudaFree(w); cudaFree(w2); cudaFree(vraw); cudaFree(zero);
  cudaFree(npart); cudaFree(dpart); cudaFree(scal);
  if (st == QG_OK) {
    for (int k = 0; k < nchain; k++) a_host[k * (ntri + 1)] = 0.0;
    st = qg_check_device_error(ctx, "qg_lanczos_tridiag");
  }
  return st;
}

// per column k of v (n x nvec): flags[2k] set when a real part is non-zero, flags[2k + 1] when an
// imaginary part is.  Each thread keeps its bits for its columns, the block merges them in
// shared memory, and one global OR per column and block remains (no contention on the flags).
__global__ void k_column_parts(int64_t n, int nvec, const double2 *__restrict__ v, unsigned int *flags) {
  extern __shared__ unsigned int sfl[];  // 2 nvec
  for (int k = threadIdx.x; k < 2 * nvec; k += blockDim.x) sfl[k] = 0u;
  __syncthreads();
  const int64_t total = n * nvec, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    const double2 a = v[i];
    const int k = (int)(i % nvec);
    if (a.x != 0.0 && !sfl[2 * k]) atomicOr(sfl + 2 * k, 1u);
    if (a.y != 0.0 && !sfl[2 * k + 1]) atomicOr(sfl + 2 * k + 1, 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 2 * nvec; k += blockDim.x)
    if (sfl[k]) atomicOr(flags + k, 1u);
}

// out (n x nout): column j takes part part[j] (0 real, 1 imaginary, -1 zero) of column src[j]
// of v into its real part, and part part2[j] of column src2[j] into its imaginary part
// (split pairs); with src2 null, whole columns (complex) are copied.
__global__ void k_pack_columns(int64_t n, int nvec, const double2 *__restrict__ v, int nout, const int *src,
                               const int *part, const int *src2, const int *part2, double2 *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * nout) return;
  const int64_t r = i / nout;
  const int j = (int)(i % nout);
  const double2 a = v[r * nvec + src[j]];
  if (!src2) {
    out[i] = a;
    return;
  }
  const double re = part[j] == 0 ? a.x : part[j] == 1 ? a.y : 0.0;
  double im = 0.0;
  if (part2[j] >= 0) {
    const double2 c = v[r * nvec + src2[j]];
    im = part2[j] == 0 ? c.x : c.y;
  }
  out[i] = make_double2(re, im);
}

extern "C" qg_status qg_lanczos_tridiag(qg_context ctx, qg_operator op, qg_basis b, const double *v0_dev, int32_t nvec,
                                        int32_t ntri, double eps, double gamma, double *a_host, double *b_host,
                                        double *krylov_dev) {
  if (!ctx || !op || !b || !v0_dev || nvec <= 0 || ntri <= 0 || !a_host || !b_host || op->nf != b->nf) {
    if (ctx) ctx->last_error = "qg_lanczos_tridiag: bad argument";
    return QG_ERR_ARG;
  }
  cudaStream_t s = ctx->stream;
  int64_t n = b->n;
  if (n == 0) {  // an empty start vector: every coefficient is zero (the spectrum vanishes)
    for (int64_t k = 0; k < (int64_t)nvec * (ntri + 1); k++) a_host[k] = 0.0;
    for (int64_t k = 0; k < (int64_t)nvec * ntri; k++) b_host[k] = 0.0;
    return QG_OK;
  }
  {
    bool done = false;
    qg_status sst = lanczos_small(ctx, op, b, v0_dev, nvec, ntri, eps, gamma, a_host, b_host, krylov_dev, &done);
    if (sst != QG_OK || done) return sst;
  }
  // Real chains.  With a real operator a start vector whose imaginary (or real) part is zero
  // stays so: a single such chain runs on real vectors (one FMA per connection, half the
  // bytes), and two share one complex vector (one apply serves both), so each costs half.  A purely imaginary vector has the coefficients of its imaginary part.
  // Each part is updated with exactly the arithmetic of its chain run alone; with one pair the
  // reductions run in the same order too and the coefficients are bitwise those of the runs
  // alone, with more pairs the multi-vector reductions add in another order (rounding only).
  if (ctx->split_chains && !krylov_dev && nvec <= 4096 && qg_operator_values_real(op) && qg_apply_uses_lists(op, b)) {
    unsigned int *d_flags = nullptr;
    std::vector<unsigned int> fl(2 * (size_t)nvec, 0u);
    cudaError_t e = cudaMalloc(&d_flags, fl.size() * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, fl.size() * sizeof(unsigned int), s);
    if (e == cudaSuccess) {
      const unsigned g = (unsigned)std::min<int64_t>((n * nvec + 255) / 256, 4LL * ctx->num_sms);
      k_column_parts<<<g, 256, 2 * nvec * sizeof(unsigned int), s>>>(n, nvec, (const double2 *)v0_dev, d_flags);
      ctx->launches++;
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(fl.data(), d_flags, fl.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_flags);
    if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
    std::vector<int> rcol, rpart, ccol;  // real chains (column, part) and complex columns
    for (int k = 0; k < nvec; k++) {
      if (fl[2 * k] && fl[2 * k + 1]) {
        ccol.push_back(k);
      } else {
        rcol.push_back(k);
        rpart.push_back(fl[2 * k + 1] ? 1 : 0);
      }
    }
    if (nvec == 1 && rcol.size() == 1) {
      double *xr = nullptr;
      e = cudaMalloc(&xr, (size_t)n * sizeof(double));
      if (e == cudaSuccess) {
        k_take_part<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, (const double2 *)v0_dev, rpart[0], xr);
        ctx->launches++;
        e = cudaGetLastError();
      }
      qg_status st = e == cudaSuccess ? lanczos_general(ctx, op, b, xr, 1, ntri, eps, gamma, a_host, b_host, nullptr, 0, 1)
                                      : qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
      cudaStreamSynchronize(s);
      cudaFree(xr);
      return st;
    }
    if (rcol.size() >= 2) {
      const int np = (int)(rcol.size() + 1) / 2, nc = (int)ccol.size();
      std::vector<int> sa(np), pa(np), sb(np), pb(np);
      for (int j = 0; j < np; j++) {
        sa[j] = rcol[2 * j];
        pa[j] = rpart[2 * j];
        const bool has = 2 * j + 1 < (int)rcol.size();
        sb[j] = has ? rcol[2 * j + 1] : 0;
        pb[j] = has ? rpart[2 * j + 1] : -1;  // an odd chain out pairs with an empty one
      }
      int *d_idx = nullptr;
      double2 *zp = nullptr, *zc = nullptr;
      const int ni = 4 * np + nc;
      std::vector<int> idx;
      idx.insert(idx.end(), sa.begin(), sa.end());
      idx.insert(idx.end(), pa.begin(), pa.end());
      idx.insert(idx.end(), sb.begin(), sb.end());
      idx.insert(idx.end(), pb.begin(), pb.end());
      idx.insert(idx.end(), ccol.begin(), ccol.end());
      e = cudaMalloc(&d_idx, (size_t)ni * sizeof(int));
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx, idx.data(), (size_t)ni * sizeof(int), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaMalloc(&zp, (size_t)n * np * sizeof(double2));
      if (e == cudaSuccess && nc) e = cudaMalloc(&zc, (size_t)n * nc * sizeof(double2));
      if (e == cudaSuccess) {
        k_pack_columns<<<(unsigned)((n * np + 255) / 256), 256, 0, s>>>(n, nvec, (const double2 *)v0_dev, np, d_idx,
                                                                       d_idx + np, d_idx + 2 * np, d_idx + 3 * np, zp);
        if (nc)
          k_pack_columns<<<(unsigned)((n * nc + 255) / 256), 256, 0, s>>>(n, nvec, (const double2 *)v0_dev, nc,
                                                                         d_idx + 4 * np, nullptr, nullptr, nullptr,
                                                                         zc);
        ctx->launches += nc ? 2 : 1;
        e = cudaGetLastError();
      }
      qg_status st = e == cudaSuccess ? QG_OK : qg_cuda_fail(ctx, e, "qg_lanczos_tridiag");
      std::vector<double> ah((size_t)2 * np * (ntri + 1)), bh((size_t)2 * np * ntri);
      if (st == QG_OK)
        st = lanczos_general(ctx, op, b, (const double *)zp, np, ntri, eps, gamma, ah.data(), bh.data(), nullptr, 1);
      if (st == QG_OK) {
        for (size_t q = 0; q < rcol.size(); q++) {
          std::copy(ah.begin() + q * (ntri + 1), ah.begin() + (q + 1) * (ntri + 1), a_host + (size_t)rcol[q] * (ntri + 1));
          std::copy(bh.begin() + q * ntri, bh.begin() + (q + 1) * ntri, b_host + (size_t)rcol[q] * ntri);
        }
      }
      if (st == QG_OK && nc) {
        std::vector<double> ac((size_t)nc * (ntri + 1)), bc((size_t)nc * ntri);
        st = lanczos_general(ctx, op, b, (const double *)zc, nc, ntri, eps, gamma, ac.data(), bc.data(), nullptr, 0);
        if (st == QG_OK)
          for (int q = 0; q < nc; q++) {
            std::copy(ac.begin() + (size_t)q * (ntri + 1), ac.begin() + (size_t)(q + 1) * (ntri + 1),
                      a_host + (size_t)ccol[q] * (ntri + 1));
            std::copy(bc.begin() + (size_t)q * ntri, bc.begin() + (size_t)(q + 1) * ntri, b_host + (size_t)ccol[q] * ntri);
          }
      }
      cudaStreamSynchronize(s);
      cudaFree(d_idx);
      cudaFree(zp);
      cudaFree(zc);
      return st;
    }
  }
  return lanczos_general(ctx, op, b, v0_dev, nvec, ntri, eps, gamma, a_host, b_host, krylov_dev, 0);
}

extern "C" qg_status qg_set_split_chains(qg_context ctx, int32_t on) {
  if (!ctx) return QG_ERR_ARG;
  ctx->split_chains = on != 0;
  return QG_OK;
}

// ------------------------------------------------------------------ continued fraction

// One thread per (spectrum, frequency); the recursion runs from the bottom of the chain as
// TriDiagonalMatrixToSpectrum does (Core/Spectral.cpp:1444-1458).
__global__ void k_cf(int nspec, int ntri, const double *__restrict__ a, const double *__restrict__ b,
                     const double *__restrict__ e0, double emin, double de, int ne, double gamma, double2 *g) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t np = (int64_t)ne + 1;
  if (t >= (int64_t)nspec * np) return;
  int s = (int)(t / np);
  int k = (int)(t % np);
  const double *as = a + (size_t)s * (ntri + 1);
  const double *bs = b + (size_t)s * ntri;
  double hg = gamma * 0.5;
  double w = (double)k * de + emin + e0[s];
  double dn = w - as[ntri];
  double den = hg * hg + dn * dn;
  double vr = dn / den, vi = -hg / den;
  for (int j = (ntri > 1 ? ntri : 1) - 1; j >= 1; j--) {
    double b2 = bs[j] * bs[j];
    double zr = w - as[j] - vr * b2, zi = hg - vi * b2;
    den = zi * zi + zr * zr;
    vr = zr / den;
    vi = (vi * b2 - hg) / den;
  }
  double b02 = bs[0] * bs[0];
  g[t] = make_double2(as[0] + vr * b02, vi * b02);
}

extern "C" qg_status qg_cf_spectra(qg_context ctx, int32_t nspec, int32_t ntri, const double *a_host,
                                   const double *b_host, const double *e0_host, double emin, double de, int32_t ne,
                                   double gamma, double *g_host) {
  if (!ctx || nspec <= 0 || ntri <= 0 || ne < 0 || !a_host || !b_host || !e0_host || !g_host) return QG_ERR_ARG;
  cudaStream_t s = ctx->stream;
  double *d = nullptr;
  size_t na = (size_t)nspec * (ntri + 1), nb = (size_t)nspec * ntri, ng = (size_t)nspec * (ne + 1);
  QG_CUDA(ctx, cudaMalloc(&d, (na + nb + nspec) * 8 + ng * 16));
  double *da = d, *db = d + na, *de0 = db + nb;
  double2 *dg = (double2 *)(de0 + nspec);
  cudaError_t e = cudaMemcpyAsync(da, a_host, na * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(db, b_host, nb * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(de0, e0_host, nspec * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_cf<<<(unsigned)((ng + 127) / 128), 128, 0, s>>>(nspec, ntri, da, db, de0, emin, de, ne, gamma, dg);
    ctx->launches++;
    e = cudaMemcpyAsync(g_host, dg, ng * 16, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_cf_spectra");
  return qg_check_launch(ctx, "qg_cf_spectra");
}
