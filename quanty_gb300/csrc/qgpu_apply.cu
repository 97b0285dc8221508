// H*psi in pull form.
//
// The reference pushes: every source determinant applies every term and adds into the
// target under `omp atomic` (OperatorPsiConserveBasisPreAllocatedCC,
// Core/OperatorWaveFunction.cpp:784-838; ComplexWaveFunctionAddElementConserveBasis,
// Core/ComplexWaveFunctionArithmetic.cpp:355-398).  Here every row gathers:
//   y_i = D_i x_i + sum_{t off-diagonal} V_t <i|t|j> x_j,   j = i ^ flip_t,
//   <i|t|j> = sign(t^dag, i),
// with the adjoint masks (need1 group test, need0 test, popcount parity).  No float
// atomics; each row's sum has a fixed order, so results are deterministic run to run.
//
// Memory path, per connection one 32-byte DRAM sector: before the gather kernel runs, a pack
// kernel writes the source amplitudes into the hash slots next to their keys, so the probe
// that finds the source also delivers its amplitude.  A source that violates the occupation
// windows the basis was built under cannot be in the basis and is not probed.  The diagonal
// D (all flip == 0 terms) is computed once per (operator, basis) and cached.
//
// Compute path: one thread per row; a warp covers 32 consecutive rows of a sorted basis,
// which share their leading (impurity) orbitals, so group and term tests are mostly
// warp-uniform.  The term table (groups + terms, one allocation) is staged into shared
// memory with bulk asynchronous copies (cp.async.bulk, completion on an mbarrier with a
// bounded wait) when it fits; otherwise it is read through the read-only cache.
#include <algorithm>

#include "qgpu_internal.cuh"

static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

#define QG_SMEM_TABLE_MAX (96 * 1024)
#define QG_MBAR_SPIN_LIMIT (1 << 24)

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < QG_MBAR_SPIN_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Stage `bytes` (multiple of 16) from global to shared with bulk copies; returns the table
// pointer to use (shared on success, global if the bounded wait gave up).
__device__ __forceinline__ const unsigned char *stage_table(const unsigned char *g, uint32_t bytes, unsigned char *s,
                                                            unsigned long long *bar, unsigned int *err, bool &pending) {
  uint32_t b = smem_addr(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    const uint32_t chunk = 16384;
    for (uint32_t off = 0; off < bytes; off += chunk) {
      uint32_t sz = bytes - off < chunk ? bytes - off : chunk;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_addr(s + off)),
                   "l"(g + off), "r"(sz), "r"(b)
                   : "memory");
    }
  }
  bool ok = mbar_wait_bounded(b, 0);
  pending = !ok;
  if (!ok) {
    atomicOr(err, QG_DEVERR_TIMEOUT);
    return g;
  }
  return s;
}

struct SrcView {
  const Slot *slots;
  const uint32_t *slot_row;
  uint64_t hmask;
  int nres;
  const uint64_t *rmask;
  const int32_t *rmin, *rmax;
};

template <int W>
__device__ __forceinline__ bool in_windows(const Key<W> &s, const SrcView &v) {
  for (int q = 0; q < v.nres; q++) {
    int c = 0;
#pragma unroll
    for (int i = 0; i < W; i++) c += __popcll(s.w[i] & __ldg(v.rmask + q * W + i));
    if (c < __ldg(v.rmin + q) || c > __ldg(v.rmax + q)) return false;
  }
  return true;
}

template <int W, int NV, bool FUSE, bool SMEM>
__global__ void __launch_bounds__(256) k_apply(const Key<W> *__restrict__ rows, int64_t n_rows,
                                               const unsigned char *__restrict__ gtab, uint32_t tab_bytes,
                                               int ngroups, const double2 *__restrict__ diag, SrcView src,
                                               int packed, int same_basis, const double2 *__restrict__ x, int xs,
                                               double2 *__restrict__ y, int ys, int vec0, ApplyFuse fz,
                                               unsigned int *err) {
  extern __shared__ __align__(128) unsigned char s_tab[];
  __shared__ __align__(8) unsigned long long s_bar;
  bool pending = false;
  const unsigned char *tab = gtab;
  if (SMEM) tab = stage_table(gtab, tab_bytes, s_tab, &s_bar, err, pending);
  const GroupDev<W> *groups = reinterpret_cast<const GroupDev<W> *>(tab);
  const TermDev<W> *terms = reinterpret_cast<const TermDev<W> *>(tab + (size_t)ngroups * sizeof(GroupDev<W>));

  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool live = r < n_rows;
  double2 acc[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) acc[k] = make_double2(0.0, 0.0);
  if (live) {
    Key<W> d = rows[r];
    if (diag) {
      double2 dg = diag[r];
#pragma unroll
      for (int k = 0; k < NV; k++) {
        double2 xv = x[r * xs + vec0 + k];
        acc[k].x = dg.x * xv.x - dg.y * xv.y;
        acc[k].y = dg.x * xv.y + dg.y * xv.x;
      }
    }
    for (int g = 0; g < ngroups; g++) {
      bool ok = true;
#pragma unroll
      for (int i = 0; i < W; i++) {
        uint64_t n1 = groups[g].need1[i];
        ok &= (d.w[i] & n1) == n1;
      }
      if (!ok) continue;
      int tb = groups[g].begin, te = groups[g].end;
      for (int t = tb; t < te; t++) {
        const TermDev<W> &T = terms[t];
        bool app = true, dg = true;
        Key<W> s;
#pragma unroll
        for (int i = 0; i < W; i++) {
          app &= (d.w[i] & T.need0[i]) == 0;
          uint64_t fl = T.flip[i];
          s.w[i] = d.w[i] ^ fl;
          dg &= fl == 0;
        }
        if (!app) continue;
        int64_t h = -1, j = -1;
        if (dg && same_basis) {
          j = r;
        } else {
          if (src.nres && !in_windows<W>(s, src)) continue;
          h = qg_find_slot<W>(src.slots, src.hmask, s, err);
          if (h < 0) continue;
          if (!(NV == 1 && packed)) j = (int64_t)__ldg(src.slot_row + h);
        }
        int par = 0;
#pragma unroll
        for (int i = 0; i < W; i++) par += __popcll(d.w[i] & T.sgn[i]);
        double vr = T.vre, vi = T.vim;
        if (par & 1) {
          vr = -vr;
          vi = -vi;
        }
#pragma unroll
        for (int k = 0; k < NV; k++) {
          double2 xv;
          if (NV == 1 && packed && h >= 0)
            xv = __ldg(reinterpret_cast<const double2 *>(src.slots + h) + 1);
          else
            xv = __ldg(x + j * xs + vec0 + k);
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
  } else {
    // fused epilogue: dot partials conj(x_r) (Hx)_r and the three-term update
    __shared__ double2 red[NV][8];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double2 dv = make_double2(0.0, 0.0);
      if (live) {
        double2 xv = x[r * xs + vec0 + k];
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
  if (SMEM && pending) mbar_wait_bounded(smem_addr(&s_bar), 0);  // never leave with a copy in flight
}

int qg_apply_grid(qg_basis dst) { return (int)std::max<int64_t>(1, (dst->n + 255) / 256); }

template <int W, int NV, bool FUSE, bool SMEM>
static void launch_apply_t(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int vec0, const ApplyFuse &fz) {
  size_t smem = SMEM ? tab.bytes : 0;
  if (SMEM) {
    static bool attr_done = false;
    if (!attr_done) {
      cudaFuncSetAttribute(k_apply<W, NV, FUSE, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, QG_SMEM_TABLE_MAX);
      attr_done = true;
    }
  }
  SrcView sv{src->d_slots, src->d_slot_row, (uint64_t)(src->hcap - 1), src->nres, src->d_rmask, src->d_rmin,
             src->d_rmax};
  k_apply<W, NV, FUSE, SMEM><<<qg_apply_grid(dst), 256, smem, ctx->stream>>>(
      (const Key<W> *)dst->d_keys, dst->n, (const unsigned char *)tab.d_blob, (uint32_t)tab.bytes, tab.ngroups, diag, sv,
      packed, dst == src, x, xs, y, ys, vec0, fz, ctx->d_err);
  ctx->launches++;
}

template <int W, bool FUSE, bool SMEM>
static void launch_apply_w(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int nvec, const ApplyFuse &fz) {
  int v = 0;
  while (v < nvec) {
    int left = nvec - v;
    if (left >= 8) {
      launch_apply_t<W, 8, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz);
      v += 8;
    } else if (left >= 4) {
      launch_apply_t<W, 4, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz);
      v += 4;
    } else if (left >= 2) {
      launch_apply_t<W, 2, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz);
      v += 2;
    } else {
      launch_apply_t<W, 1, FUSE, SMEM>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, v, fz);
      v += 1;
    }
  }
}

template <int W, bool FUSE>
static void launch_apply_s(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int nvec, const ApplyFuse &fz) {
  if (tab.bytes <= QG_SMEM_TABLE_MAX)
    launch_apply_w<W, FUSE, true>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, nvec, fz);
  else
    launch_apply_w<W, FUSE, false>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, nvec, fz);
}

// ------------------------------------------------------------------ pack

template <int W>
__global__ void k_pack(const Key<W> *__restrict__ keys, const uint32_t *__restrict__ row_slot, int64_t n,
                       const double2 *__restrict__ x, int xs, const double *__restrict__ scale,
                       const double *__restrict__ thr2, double2 *own_out, Slot *slots) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double2 v = x[r * xs];
  if (scale) {
    double sc = *scale, t2 = *thr2;
    v.x *= sc;
    v.y *= sc;
    if (!(v.x * v.x + v.y * v.y > t2)) v = make_double2(0.0, 0.0);  // the reference keeps |a|^2 > eps^2
  }
  if (own_out) own_out[r * xs] = v;
  Key<W> k = keys[r];
  Slot s;
  s.k[0] = k.w[0];
  s.k[1] = (W == 1) ? 0ull : k.w[W - 1];
  s.vre = v.x;
  s.vim = v.y;
  slots[row_slot[r]] = s;
}

qg_status qg_pack(qg_context ctx, qg_basis b, const double *x, int xs, const double *scale, const double *thr2,
                  double *own_out) {
  if (!b->n) return QG_OK;
  if (b->W == 1)
    k_pack<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<1> *)b->d_keys, b->d_row_slot, b->n,
                                                            (const double2 *)x, xs, scale, thr2, (double2 *)own_out,
                                                            b->d_slots);
  else
    k_pack<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<2> *)b->d_keys, b->d_row_slot, b->n,
                                                            (const double2 *)x, xs, scale, thr2, (double2 *)own_out,
                                                            b->d_slots);
  ctx->launches++;
  return qg_check_launch(ctx, "pack");
}

// ------------------------------------------------------------------ diagonal

template <int W>
__global__ void k_diag(const Key<W> *__restrict__ rows, int64_t n, const GroupDev<W> *__restrict__ groups, int ngroups,
                       const TermDev<W> *__restrict__ terms, double2 *diag) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  Key<W> d = rows[r];
  double2 acc = make_double2(0.0, 0.0);
  for (int g = 0; g < ngroups; g++) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < W; i++) ok &= (d.w[i] & groups[g].need1[i]) == groups[g].need1[i];
    if (!ok) continue;
    for (int t = groups[g].begin; t < groups[g].end; t++) {
      bool app = true;
      int par = 0;
#pragma unroll
      for (int i = 0; i < W; i++) {
        app &= (d.w[i] & terms[t].need0[i]) == 0;
        par += __popcll(d.w[i] & terms[t].sgn[i]);
      }
      if (!app) continue;
      double s = (par & 1) ? -1.0 : 1.0;
      acc.x += s * terms[t].vre;
      acc.y += s * terms[t].vim;
    }
  }
  diag[r] = acc;
}

double *qg_basis_diag(qg_basis b, qg_operator op, qg_status *st) {
  *st = QG_OK;
  for (auto &c : b->diag)
    if (c.op_uid == op->uid) return c.d_diag;
  qg_context ctx = b->ctx;
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, std::max<int64_t>(b->n, 1) * 16);
  if (e != cudaSuccess) {
    *st = qg_cuda_fail(ctx, e, "diagonal");
    return nullptr;
  }
  if (b->n) {
    if (op->W == 1)
      k_diag<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<1> *)b->d_keys, b->n,
                                                              (const GroupDev<1> *)op->diag.d_groups, op->diag.ngroups,
                                                              (const TermDev<1> *)op->diag.d_terms, (double2 *)d);
    else
      k_diag<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<2> *)b->d_keys, b->n,
                                                              (const GroupDev<2> *)op->diag.d_groups, op->diag.ngroups,
                                                              (const TermDev<2> *)op->diag.d_terms, (double2 *)d);
    ctx->launches++;
  }
  if (b->diag.size() >= 4) {  // small cache: drop the oldest
    cudaStreamSynchronize(ctx->stream);
    cudaFree(b->diag.front().d_diag);
    b->diag.erase(b->diag.begin());
  }
  b->diag.push_back({op->uid, d});
  *st = qg_check_launch(ctx, "diagonal");
  return d;
}

// ------------------------------------------------------------------ entry points

qg_status qg_apply_strided(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                           double *y, int ys, int nvec, const ApplyFuse *fz, bool x_packed) {
  ApplyFuse none;
  const double2 *x2 = (const double2 *)x;
  double2 *y2 = (double2 *)y;
  qg_status st = QG_OK;
  const double2 *diag = nullptr;
  const HostTable *tab = &op->pull;
  if (dst == src) {
    diag = (const double2 *)qg_basis_diag(dst, op, &st);
    if (st != QG_OK) return st;
    tab = &op->pull_off;
  }
  int packed = 0;
  if (nvec == 1) {
    if (!x_packed) QG_TRY(qg_pack(ctx, src, x, xs, nullptr, nullptr, nullptr));
    packed = 1;
  }
  const ApplyFuse &f = fz ? *fz : none;
  if (op->W == 1) {
    if (fz)
      launch_apply_s<1, true>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f);
    else
      launch_apply_s<1, false>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f);
  } else {
    if (fz)
      launch_apply_s<2, true>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f);
    else
      launch_apply_s<2, false>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f);
  }
  return qg_check_launch(ctx, "qg_apply");
}

qg_status qg_apply_launch(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, double *y,
                          int nvec, const ApplyFuse *fz) {
  return qg_apply_strided(ctx, op, dst, src, x, nvec, y, nvec, nvec, fz, false);
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
                        int ngroups, const TermDev<W> *__restrict__ terms, const Slot *__restrict__ slots,
                        uint64_t hmask, int offdiag_only, unsigned long long *out, unsigned int *err) {
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
        bool app = true, dg = true;
        Key<W> s;
#pragma unroll
        for (int i = 0; i < W; i++) {
          app &= (d.w[i] & terms[t].need0[i]) == 0;
          s.w[i] = d.w[i] ^ terms[t].flip[i];
          dg &= terms[t].flip[i] == 0;
        }
        if (!app || (dg && offdiag_only)) continue;
        if (qg_find_slot<W>(slots, hmask, s, err) >= 0) c++;
      }
    }
  }
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

static qg_status count_nnz(qg_context ctx, qg_operator op, qg_basis b, int offdiag, int64_t *nnz) {
  *nnz = 0;
  if (!b->n) return QG_OK;
  unsigned long long *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, 8));
  QG_CUDA(ctx, cudaMemsetAsync(d, 0, 8, ctx->stream));
  if (op->W == 1)
    k_count<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>(
        (const Key<1> *)b->d_keys, b->n, (const GroupDev<1> *)op->pull.d_groups, op->pull.ngroups,
        (const TermDev<1> *)op->pull.d_terms, b->d_slots, b->hcap - 1, offdiag, d, ctx->d_err);
  else
    k_count<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>(
        (const Key<2> *)b->d_keys, b->n, (const GroupDev<2> *)op->pull.d_groups, op->pull.ngroups,
        (const TermDev<2> *)op->pull.d_terms, b->d_slots, b->hcap - 1, offdiag, d, ctx->d_err);
  ctx->launches++;
  unsigned long long h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_count_nnz");
  *nnz = (int64_t)h;
  return qg_check_device_error(ctx, "qg_count_nnz");
}

extern "C" qg_status qg_count_nnz(qg_context ctx, qg_operator op, qg_basis b, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf) return QG_ERR_ARG;
  return count_nnz(ctx, op, b, 0, nnz);
}

extern "C" qg_status qg_count_nnz_offdiag(qg_context ctx, qg_operator op, qg_basis b, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf) return QG_ERR_ARG;
  return count_nnz(ctx, op, b, 1, nnz);
}
