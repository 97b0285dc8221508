// H*psi in pull form.
//
// The reference pushes: every source determinant applies every term and adds into the
// target under `omp atomic` (OperatorPsiConserveBasisPreAllocatedCC,
// Core/OperatorWaveFunction.cpp:784-838; ComplexWaveFunctionAddElementConserveBasis,
// Core/ComplexWaveFunctionArithmetic.cpp:355-398).  Here every row gathers:
//   y_i = sum_t V_t <i|t|j> x_j,   j = i ^ flip_t,   <i|t|j> = sign(t^dag, i),
// evaluated with the adjoint masks (need1 group test, need0 test, popcount parity), the
// source row found through the source basis' hash table.  No float atomics; each row's sum
// has a fixed order, so results are deterministic run to run.
//
// One thread per row; a warp covers 32 consecutive rows of a sorted basis, which share their
// leading (impurity) orbitals, so the group and term tests are mostly warp-uniform.  The
// group headers and terms are read through the read-only path: every lane of a warp reads the
// same address (a broadcast).  NV vectors are processed per pass; wider blocks loop over
// chunks of NV columns.
#include "qgpu_internal.cuh"

static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <int W, int NV, bool FUSE>
__global__ void __launch_bounds__(256) k_apply(const Key<W> *__restrict__ rows, int64_t n_rows,
                                               const GroupDev<W> *__restrict__ groups, int ngroups,
                                               const TermDev<W> *__restrict__ terms,
                                               const Slot<W> *__restrict__ src_slots, uint64_t hmask, int same_basis,
                                               const double2 *__restrict__ x, int xs, double2 *__restrict__ y,
                                               int ys, int vec0, ApplyFuse fz, unsigned int *err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool live = r < n_rows;
  double2 acc[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) acc[k] = make_double2(0.0, 0.0);
  double sc[NV], t2[NV];
  if (FUSE) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      sc[k] = fz.src_scale[vec0 + k];
      t2[k] = fz.thr2[vec0 + k];
    }
  }
  if (live) {
    Key<W> d = rows[r];
    for (int g = 0; g < ngroups; g++) {
      uint64_t n1[W];
#pragma unroll
      for (int i = 0; i < W; i++) n1[i] = __ldg(&groups[g].need1[i]);
      bool ok = true;
#pragma unroll
      for (int i = 0; i < W; i++) ok &= (d.w[i] & n1[i]) == n1[i];
      if (!ok) continue;
      int tb = __ldg(&groups[g].begin), te = __ldg(&groups[g].end);
      for (int t = tb; t < te; t++) {
        const TermDev<W> *T = terms + t;
        bool app = true, diag = true;
        uint64_t fl[W];
#pragma unroll
        for (int i = 0; i < W; i++) {
          app &= (d.w[i] & __ldg(&T->need0[i])) == 0;
          fl[i] = __ldg(&T->flip[i]);
          diag &= fl[i] == 0;
        }
        if (!app) continue;
        int64_t j;
        if (diag && same_basis) {
          j = r;
        } else {
          Key<W> s;
#pragma unroll
          for (int i = 0; i < W; i++) s.w[i] = d.w[i] ^ fl[i];
          j = qg_lookup<W>(src_slots, hmask, s, err);
          if (j < 0) continue;
        }
        int par = 0;
#pragma unroll
        for (int i = 0; i < W; i++) par += __popcll(d.w[i] & __ldg(&T->sgn[i]));
        double vr = __ldg(&T->vre), vi = __ldg(&T->vim);
        if (par & 1) {
          vr = -vr;
          vi = -vi;
        }
        const double2 *xp = x + j * xs + vec0;
#pragma unroll
        for (int k = 0; k < NV; k++) {
          double2 xv = __ldg(xp + k);
          if (FUSE) {
            xv.x *= sc[k];
            xv.y *= sc[k];
            if (!(xv.x * xv.x + xv.y * xv.y > t2[k])) continue;  // reference keeps |a|^2 > eps^2
          }
          acc[k].x = fma(vr, xv.x, fma(-vi, xv.y, acc[k].x));
          acc[k].y = fma(vr, xv.y, fma(vi, xv.x, acc[k].y));
        }
      }
    }
  }
  if (!FUSE) {
    if (live) {
#pragma unroll
      for (int k = 0; k < NV; k++) y[r * ys + vec0 + k] = acc[k];
    }
    return;
  }
  // fused epilogue: own scaled row, dot partials, three-term update
  __shared__ double2 red[NV][8];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double2 dv = make_double2(0.0, 0.0);
    if (live) {
      double2 xv = x[r * xs + vec0 + k];
      xv.x *= sc[k];
      xv.y *= sc[k];
      if (!(xv.x * xv.x + xv.y * xv.y > t2[k])) xv = make_double2(0.0, 0.0);
      fz.own_out[r * xs + vec0 + k] = xv;
      // conj(x) * Hx
      dv.x = xv.x * acc[k].x + xv.y * acc[k].y;
      dv.y = xv.x * acc[k].y - xv.y * acc[k].x;
      double2 pv = fz.prev[r * ys + vec0 + k];
      double be = fz.beta[vec0 + k];
      y[r * ys + vec0 + k] = make_double2(acc[k].x - be * pv.x, acc[k].y - be * pv.y);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      dv.x += __shfl_xor_sync(0xffffffffu, dv.x, o);
      dv.y += __shfl_xor_sync(0xffffffffu, dv.y, o);
    }
    if (lane == 0) red[k][wid] = dv;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    int k = threadIdx.x;
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      s.x += red[k][w].x;
      s.y += red[k][w].y;
    }
    fz.dot_part[blockIdx.x * ys + vec0 + k] = s;
  }
}

template <int W, int NV, bool FUSE>
static void launch_apply_t(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double2 *x, int xs,
                           double2 *y, int ys, int vec0, const ApplyFuse &fz) {
  unsigned grid = grid_for(dst->n, 256);
  k_apply<W, NV, FUSE><<<grid, 256, 0, ctx->stream>>>(
      (const Key<W> *)dst->d_keys, dst->n, (const GroupDev<W> *)op->pull.d_groups, op->pull.ngroups,
      (const TermDev<W> *)op->pull.d_terms, (const Slot<W> *)src->d_slots, (uint64_t)(src->hcap - 1), dst == src,
      x, xs, y, ys, vec0, fz, ctx->d_err);
  ctx->launches++;
}

template <int W, bool FUSE>
static void launch_apply_w(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double2 *x, int xs,
                           double2 *y, int ys, int nvec, const ApplyFuse &fz) {
  int v = 0;
  while (v < nvec) {
    int left = nvec - v;
    if (left >= 8) {
      launch_apply_t<W, 8, FUSE>(ctx, op, dst, src, x, xs, y, ys, v, fz);
      v += 8;
    } else if (left >= 4) {
      launch_apply_t<W, 4, FUSE>(ctx, op, dst, src, x, xs, y, ys, v, fz);
      v += 4;
    } else if (left >= 2) {
      launch_apply_t<W, 2, FUSE>(ctx, op, dst, src, x, xs, y, ys, v, fz);
      v += 2;
    } else {
      launch_apply_t<W, 1, FUSE>(ctx, op, dst, src, x, xs, y, ys, v, fz);
      v += 1;
    }
  }
}

qg_status qg_apply_strided(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                           double *y, int ys, int nvec, const ApplyFuse *fz) {
  ApplyFuse none;
  const double2 *x2 = (const double2 *)x;
  double2 *y2 = (double2 *)y;
  if (op->W == 1) {
    if (fz)
      launch_apply_w<1, true>(ctx, op, dst, src, x2, xs, y2, ys, nvec, *fz);
    else
      launch_apply_w<1, false>(ctx, op, dst, src, x2, xs, y2, ys, nvec, none);
  } else {
    if (fz)
      launch_apply_w<2, true>(ctx, op, dst, src, x2, xs, y2, ys, nvec, *fz);
    else
      launch_apply_w<2, false>(ctx, op, dst, src, x2, xs, y2, ys, nvec, none);
  }
  return qg_check_launch(ctx, "qg_apply");
}

qg_status qg_apply_launch(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, double *y,
                          int nvec, const ApplyFuse *fz) {
  return qg_apply_strided(ctx, op, dst, src, x, nvec, y, nvec, nvec, fz);
}

extern "C" qg_status qg_apply(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x_dev,
                              double *y_dev, int32_t nvec) {
  if (!ctx || !op || !dst || !src || nvec <= 0 || op->nf != dst->nf || op->nf != src->nf) {
    if (ctx) ctx->last_error = "qg_apply: bad argument";
    return QG_ERR_ARG;
  }
  if (!dst->n) return QG_OK;
  if (!src->n) {
    QG_CUDA(ctx, cudaMemsetAsync(y_dev, 0, dst->n * nvec * 16, ctx->stream));
    return QG_OK;
  }
  return qg_apply_launch(ctx, op, dst, src, x_dev, y_dev, nvec, nullptr);
}

extern "C" qg_status qg_apply_host(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x_host,
                                   double *y_host, int32_t nvec) {
  if (!ctx || !op || !dst || !src || nvec <= 0 || !x_host || !y_host || op->nf != dst->nf || op->nf != src->nf)
    return QG_ERR_ARG;
  size_t xb = (size_t)src->n * nvec * 16, yb = (size_t)dst->n * nvec * 16;
  size_t need = xb + yb;
  if (ctx->io_bytes < need) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_io);
    ctx->d_io = nullptr;
    ctx->io_bytes = 0;
    QG_CUDA(ctx, cudaMalloc(&ctx->d_io, need));
    ctx->io_bytes = need;
  }
  double *dx = ctx->d_io, *dy = ctx->d_io + xb / 8;
  if (xb) QG_CUDA(ctx, cudaMemcpyAsync(dx, x_host, xb, cudaMemcpyHostToDevice, ctx->stream));
  qg_status st = qg_apply(ctx, op, dst, src, dx, dy, nvec);
  if (st != QG_OK) return st;
  if (yb) QG_CUDA(ctx, cudaMemcpyAsync(y_host, dy, yb, cudaMemcpyDeviceToHost, ctx->stream));
  QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return qg_check_device_error(ctx, "qg_apply_host");
}

// ------------------------------------------------------------------ nnz count

template <int W>
__global__ void k_count(const Key<W> *__restrict__ rows, int64_t n, const GroupDev<W> *__restrict__ groups,
                        int ngroups, const TermDev<W> *__restrict__ terms, const Slot<W> *__restrict__ slots,
                        uint64_t hmask, unsigned long long *out, unsigned int *err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (r < n) {
    Key<W> d = rows[r];
    for (int g = 0; g < ngroups; g++) {
      bool ok = true;
#pragma unroll
      for (int i = 0; i < W; i++) ok &= (d.w[i] & groups[g].need1[i]) == groups[g].need1[i];
      if (!ok) continue;
      for (int t = groups[g].begin; t < groups[g].end; t++) {
        bool app = true;
        Key<W> s;
#pragma unroll
        for (int i = 0; i < W; i++) {
          app &= (d.w[i] & terms[t].need0[i]) == 0;
          s.w[i] = d.w[i] ^ terms[t].flip[i];
        }
        if (!app) continue;
        if (qg_lookup<W>(slots, hmask, s, err) >= 0) c++;
      }
    }
  }
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

extern "C" qg_status qg_count_nnz(qg_context ctx, qg_operator op, qg_basis b, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf) return QG_ERR_ARG;
  *nnz = 0;
  if (!b->n) return QG_OK;
  unsigned long long *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, 8));
  QG_CUDA(ctx, cudaMemsetAsync(d, 0, 8, ctx->stream));
  if (op->W == 1)
    k_count<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>(
        (const Key<1> *)b->d_keys, b->n, (const GroupDev<1> *)op->pull.d_groups, op->pull.ngroups,
        (const TermDev<1> *)op->pull.d_terms, (const Slot<1> *)b->d_slots, b->hcap - 1, d, ctx->d_err);
  else
    k_count<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>(
        (const Key<2> *)b->d_keys, b->n, (const GroupDev<2> *)op->pull.d_groups, op->pull.ngroups,
        (const TermDev<2> *)op->pull.d_terms, (const Slot<2> *)b->d_slots, b->hcap - 1, d, ctx->d_err);
  ctx->launches++;
  unsigned long long h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_count_nnz");
  *nnz = (int64_t)h;
  return qg_check_device_error(ctx, "qg_count_nnz");
}
