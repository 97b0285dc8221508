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
#include <cub/cub.cuh>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "qgpu_internal.cuh"

static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

#define QG_SMEM_TABLE_MAX (96 * 1024)
#define QG_MBAR_SPIN_LIMIT (1 << 24)
#ifndef QG_LOCAL_UNROLL
#define QG_LOCAL_UNROLL 1
#endif
static constexpr int kLocalUnroll = QG_LOCAL_UNROLL;  // local moves unrolled per iteration
#ifndef QG_APPLY_MIN_BLOCKS
#define QG_APPLY_MIN_BLOCKS 6  // resident blocks asked of the single-vector apply (caps registers)
#endif

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

// Local decomposition view (see OpBasisCache): rows of one local configuration form a block;
// entry e of block b moves a row to block ent[e].tblock at the same offset when the blocks
// list the same remaining (non-local) configurations, which a key comparison verifies.
struct LocalView {
  int on;
  int lo;          // device bit of the lowest local orbital
  uint32_t lmask;  // (1 << H) - 1
  const int32_t *cfg;
  const uint32_t *bstart, *eoff;
  const LocalEntry *ent;
  const uint32_t *etarget;
};

template <int W>
__device__ __forceinline__ uint32_t get_local(const Key<W> &d, int lo, uint32_t lmask) {
  if (W == 1) return (uint32_t)(d.w[0] >> lo) & lmask;
  if (lo >= 64) return (uint32_t)(d.w[W - 1] >> (lo - 64)) & lmask;
  uint64_t v = (d.w[0] >> lo) | (lo ? (d.w[W - 1] << (64 - lo)) : 0ull);
  return (uint32_t)v & lmask;
}

template <int W>
__device__ __forceinline__ Key<W> set_local(const Key<W> &d, int lo, uint32_t lmask, uint32_t c) {
  Key<W> o = d;
  if (W == 1) {
    o.w[0] = (d.w[0] & ~((uint64_t)lmask << lo)) | ((uint64_t)c << lo);
  } else if (lo >= 64) {
    o.w[W - 1] = (d.w[W - 1] & ~((uint64_t)lmask << (lo - 64))) | ((uint64_t)c << (lo - 64));
  } else {
    o.w[0] = (d.w[0] & ~((uint64_t)lmask << lo)) | ((uint64_t)c << lo);
    if (lo) o.w[W - 1] = (d.w[W - 1] & ~((uint64_t)lmask >> (64 - lo))) | ((uint64_t)c >> (64 - lo));
  }
  return o;
}

// Window bits of a row: bit 5q + (D + 2) is set when moving D in [-2, 2] electrons into window
// q keeps it inside [min_q, max_q]; a source the row reaches by a term whose window changes
// are D_q passes iff all its bits (the term's wreq) are set.
template <int W>
__device__ __forceinline__ uint64_t window_bits(const Key<W> &d, const SrcView &v) {
  uint64_t ok = 0;
  for (int q = 0; q < v.nres; q++) {
    int c = 0;
#pragma unroll
    for (int i = 0; i < W; i++) c += __popcll(d.w[i] & __ldg(v.rmask + q * W + i));
    int lo = __ldg(v.rmin + q), hi = __ldg(v.rmax + q);
#pragma unroll
    for (int D = -2; D <= 2; D++)
      if (c + D >= lo && c + D <= hi) ok |= 1ull << (5 * q + D + 2);
  }
  return ok;
}

// FP64 arithmetic on this GPU issues at 2 FMA per clock per SM, and the apply kernel spends
// most of its issue slots there, so FP64 work per connection is kept minimal: the parity sign
// is an integer flip of the sign bits, and a term with a real value (every hopping, Coulomb
// and one-body real term) costs two FMAs per vector instead of four.  A zero imaginary part
// contributes fma(-0, x, acc) == acc exactly, so both forms give the same bits.

// The fused Lanczos epilogue's per-block partial of a = Re <x|H x> for each of NV vectors (the
// Lanczos diagonal is real).  The apply kernels are bound by the FP64 pipe, so the reduction
// spends as few FP64 adds as it can: the rows' terms go to shared memory in row order (dvs of
// the row at block position me), eight threads per vector add 32 terms each and one thread adds
// their eight sums -- about one add per row, where a warp-shuffle tree costs five per row and
// vector.  Every apply kernel reduces in this order, so their Lanczos chains agree bitwise.
// Blocks of 256 threads; s_dot holds NV x 256 doubles (stride 256), s_red NV x 8.
// NS sums per row (NV, or 2 NV with PAIR: the two parts of each vector, written as .x and .y).
template <int NS, bool PAIR>
__device__ __forceinline__ void fused_dot_partials(const double *dvs, int me, double *s_dot, double *s_red,
                                                   double2 *part, int ys, int vec0) {
#pragma unroll
  for (int k = 0; k < NS; k++) s_dot[k * 256 + me] = dvs[k];
  __syncthreads();
  if (threadIdx.x < NS * 8) {
    const int k = threadIdx.x >> 3, seg = threadIdx.x & 7;
    double t = 0.0;
#pragma unroll 8
    for (int i = 0; i < 32; i++) t += s_dot[k * 256 + seg * 32 + i];
    s_red[k * 8 + seg] = t;
  }
  __syncthreads();
  if (!PAIR && threadIdx.x < NS) {
    double t = 0.0;
#pragma unroll
    for (int g = 0; g < 8; g++) t += s_red[threadIdx.x * 8 + g];
    part[blockIdx.x * ys + vec0 + threadIdx.x] = make_double2(t, 0.0);
  }
  if (PAIR && threadIdx.x < NS / 2) {
    double ta = 0.0, tb = 0.0;
#pragma unroll
    for (int g = 0; g < 8; g++) ta += s_red[2 * threadIdx.x * 8 + g];
#pragma unroll
    for (int g = 0; g < 8; g++) tb += s_red[(2 * threadIdx.x + 1) * 8 + g];
    part[blockIdx.x * ys + vec0 + threadIdx.x] = make_double2(ta, tb);
  }
}

template <int W, int NV, bool FUSE, bool SMEM>
__global__ void __launch_bounds__(256, NV == 1 ? QG_APPLY_MIN_BLOCKS : 1) k_apply(const Key<W> *__restrict__ rows, int64_t n_rows,
                                               const unsigned char *__restrict__ gtab, uint32_t tab_bytes,
                                               int ngroups, int nhop, uint64_t hop0, uint64_t hop1,
                                               const double2 *__restrict__ diag, SrcView src, int packed,
                                               int same_basis, const double2 *__restrict__ x, int xs,
                                               double2 *__restrict__ y, int ys, int vec0, ApplyFuse fz,
                                               LocalView lv, const uint64_t *__restrict__ wreq,
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
      const double2 dg = diag[r];
      const bool dgc = qg_is_nonzero(dg.y);  // Hermitian operators: real diagonal
#pragma unroll
      for (int k = 0; k < NV; k++) acc[k] = qg_diag_mul(dg, x[r * xs + vec0 + k], dgc);
    }
    uint64_t okm = 0;
    if (wreq && src.nres) okm = window_bits<W>(d, src);
    if (lv.on) {
      // local moves: the target sits in another block at the same offset; when the two blocks
      // list the same non-local configurations (flag bit 31 of tblock) that is certain,
      // otherwise a key comparison checks it and a miss falls back to the hash table
      int b = __ldg(lv.cfg + get_local<W>(d, lv.lo, lv.lmask));
      uint32_t rs = __ldg(lv.bstart + b);
      int64_t off = r - (int64_t)rs;
      uint32_t e1 = __ldg(lv.eoff + b + 1);
#pragma unroll (kLocalUnroll)
      for (uint32_t e = __ldg(lv.eoff + b); e < e1; e++) {
        const LocalEntry *E = lv.ent + e;
        uint32_t te = __ldg(&E->tend);
        int64_t j = (int64_t)__ldg(&E->tstart) + off;
        if (!(te >> 31)) {
          Key<W> s = set_local<W>(d, lv.lo, lv.lmask, __ldg(lv.etarget + e));
          bool hit = false;
          if (j < (int64_t)(te & 0x7FFFFFFFu)) {
            Key<W> kj = rows[j];
            hit = qg_eq<W>(kj, s);
          }
          if (!hit) {
            if (src.nres) {
              uint64_t req = __ldg(&E->wreq);
              if (wreq ? ((okm & req) != req) : !in_windows<W>(s, src)) continue;
            }
            int64_t h = qg_find_slot<W>(src.slots, src.hmask, s, err);
            if (h < 0) continue;
            j = (int64_t)__ldg(src.slot_row + h);
          }
        }
        double vr = __ldg(&E->vre), vi = __ldg(&E->vim);
        bool cplx = qg_is_nonzero(vi);
#pragma unroll
        for (int k = 0; k < NV; k++) qg_cmac(acc[k], vr, vi, cplx, __ldg(x + j * xs + vec0 + k));
      }
    }
    // one term of the table: source = row ^ flip, looked up, accumulated with its sign
    auto term = [&](int t, bool known_applicable) {
      const TermDev<W> &T = terms[t];
      if (!known_applicable) {
        bool app = true;
#pragma unroll
        for (int i = 0; i < W; i++) app &= (d.w[i] & T.need0[i]) == 0;
        if (!app) return;
      }
      Key<W> s;
      bool dg = true;
#pragma unroll
      for (int i = 0; i < W; i++) {
        uint64_t fl = T.flip[i];
        s.w[i] = d.w[i] ^ fl;
        dg &= fl == 0;
      }
      int64_t h = -1, j = -1;
      if (dg && same_basis) {
        j = r;
      } else {
        if (src.nres) {
          if (wreq) {
            uint64_t req = __ldg(wreq + t);
            if ((okm & req) != req) return;
          } else if (!in_windows<W>(s, src)) {
            return;
          }
        }
        h = qg_find_slot<W>(src.slots, src.hmask, s, err);
        if (h < 0) return;
        if (!(NV == 1 && packed)) j = (int64_t)__ldg(src.slot_row + h);
      }
      int par = 0;
#pragma unroll
      for (int i = 0; i < W; i++) par += __popcll(d.w[i] & T.sgn[i]);
      double vi = T.vim;
      bool cplx = qg_is_nonzero(vi);
      double vr = qg_flip_sign(T.vre, par);
      vi = qg_flip_sign(vi, par);
#pragma unroll
      for (int k = 0; k < NV; k++) {
        double2 xv;
        if (NV == 1 && packed && h >= 0)
          xv = __ldg(reinterpret_cast<const double2 *>(src.slots + h) + 1);
        else
          xv = __ldg(x + j * xs + vec0 + k);
        qg_cmac(acc[k], vr, vi, cplx, xv);
      }
    };
    // hop groups: each occupied orbital p with one-body moves, then each empty target q of it
    int gbase = 0;
#pragma unroll
    for (int i = 0; i < W; i++) {
      uint64_t hm = i == 0 ? hop0 : hop1;
      uint64_t m = d.w[i] & hm;
      while (m) {
        int bp = __ffsll((long long)m) - 1;
        m &= m - 1;
        const GroupDev<W> &G = groups[gbase + __popcll(hm & ((1ull << bp) - 1))];
        int tq = G.begin;
#pragma unroll
        for (int i2 = 0; i2 < W; i2++) {
          uint64_t qm = G.qmask[i2];
          uint64_t c = qm & ~d.w[i2];
          while (c) {
            int bq = __ffsll((long long)c) - 1;
            c &= c - 1;
            term(tq + __popcll(qm & ((1ull << bq) - 1)), true);
          }
          tq += __popcll(qm);
        }
      }
      gbase += __popcll(hm);
    }
    for (int g = nhop; g < ngroups; g++) {
      bool ok = true;
#pragma unroll
      for (int i = 0; i < W; i++) {
        uint64_t n1 = groups[g].need1[i];
        ok &= (d.w[i] & n1) == n1;
      }
      if (!ok) continue;
      int tb = groups[g].begin, te = groups[g].end;
      for (int t = tb; t < te; t++) term(t, false);
    }
  }
  if (!FUSE) {
    if (live) {
#pragma unroll
      for (int k = 0; k < NV; k++) y[r * ys + vec0 + k] = acc[k];
    }
  } else {
    // fused epilogue: y = H x - beta prev and the block's partial of Re <x|H x>
    __shared__ double s_dot[NV * 256], s_red[NV * 8];
    double dvs[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double dv = 0.0;
      if (live) {
        dv = qg_redot(x[r * xs + vec0 + k], acc[k]);
        y[r * ys + vec0 + k] = qg_axpy2(acc[k], fz.beta[vec0 + k], fz.prev[r * ys + vec0 + k]);
      }
      dvs[k] = dv;
    }
    fused_dot_partials<NV, false>(dvs, threadIdx.x, s_dot, s_red, fz.dot_part, ys, vec0);
  }
  if (SMEM && pending) mbar_wait_bounded(smem_addr(&s_bar), 0);  // never leave with a copy in flight
}

// ------------------------------------------------------------------ warp-per-row, lanes over vectors
//
// For many vectors (nvec >= 32) one warp takes one row at a time: its 32 lanes share the
// row's work out (local moves, terms of the table: one per lane per round), and every lane
// that found a connection appends (source row, signed value) to a per-warp list in shared
// memory in lane order (ballot + prefix popcount, so the order is fixed).  The list is then
// applied with lanes over vectors: lane l owns vectors vec0 + l + 32 m, so the amplitudes of
// one source row are one coalesced read and every FP64 lane is busy.  The list order is the
// thread-per-row kernel's order (diagonal, local moves in entry order, terms in table order),
// so each vector's sum runs in the same order and the output is bitwise the same.
#define QG_WARP_LIST 128

template <int W, int VPL, bool FUSE, bool SMEM>
__global__ void __launch_bounds__(256) k_apply_warp(const Key<W> *__restrict__ rows, int64_t n_rows,
                                                    const unsigned char *__restrict__ gtab, uint32_t tab_bytes,
                                                    int ngroups, int nterms, uint32_t tgrp_off,
                                                    const double2 *__restrict__ diag, SrcView src,
                                                    const double2 *__restrict__ x, int xs, double2 *__restrict__ y,
                                                    int ys, int vec0, int nv, ApplyFuse fz, LocalView lv,
                                                    const uint64_t *__restrict__ wreq, unsigned int *err) {
  extern __shared__ __align__(128) unsigned char s_tab[];
  __shared__ __align__(8) unsigned long long s_bar;
  __shared__ uint32_t s_j[8][QG_WARP_LIST];
  __shared__ double s_vr[8][QG_WARP_LIST], s_vi[8][QG_WARP_LIST];
  bool pending = false;
  const unsigned char *tab = gtab;
  if (SMEM) tab = stage_table(gtab, tab_bytes, s_tab, &s_bar, err, pending);
  const GroupDev<W> *groups = reinterpret_cast<const GroupDev<W> *>(tab);
  const TermDev<W> *terms = reinterpret_cast<const TermDev<W> *>(tab + (size_t)ngroups * sizeof(GroupDev<W>));
  const uint32_t *tgrp = reinterpret_cast<const uint32_t *>(tab + tgrp_off);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  uint32_t *lj = s_j[wid];
  double *lvr = s_vr[wid], *lvi = s_vi[wid];
  double2 dsum[VPL];
#pragma unroll
  for (int m = 0; m < VPL; m++) dsum[m] = make_double2(0.0, 0.0);
  const int64_t base = (int64_t)blockIdx.x * 256 + wid * 32;
  for (int it = 0; it < 32; it++) {
    const int64_t r = base + it;
    if (r >= n_rows) break;  // uniform across the warp
    const Key<W> d = rows[r];
    double2 acc[VPL];
    double2 dg = diag ? diag[r] : make_double2(0.0, 0.0);
    bool dgc = qg_is_nonzero(dg.y);
#pragma unroll
    for (int m = 0; m < VPL; m++) {
      int k = lane + 32 * m;
      acc[m] = make_double2(0.0, 0.0);
      if (diag && k < nv) acc[m] = qg_diag_mul(dg, x[r * xs + vec0 + k], dgc);
    }
    int cnt = 0;
    auto flush = [&]() {
      __syncwarp();
      for (int c = 0; c < cnt; c++) {
        int64_t j = lj[c];
        double vr = lvr[c], vi = lvi[c];
        bool cplx = qg_is_nonzero(vi);
#pragma unroll
        for (int m = 0; m < VPL; m++) {
          int k = lane + 32 * m;
          if (k < nv) qg_cmac(acc[m], vr, vi, cplx, __ldg(x + j * xs + vec0 + k));
        }
      }
      __syncwarp();
      cnt = 0;
    };
    auto append = [&](bool has, int64_t j, double vr, double vi) {
      unsigned msk = __ballot_sync(FULL, has);
      if (!msk) return;
      if (cnt + 32 > QG_WARP_LIST) flush();
      if (has) {
        int pos = cnt + __popc(msk & ((1u << lane) - 1u));
        lj[pos] = (uint32_t)j;
        lvr[pos] = vr;
        lvi[pos] = vi;
      }
      cnt += __popc(msk);
    };
    // window bits of the row, one window per lane
    uint64_t okm = 0;
    if (wreq && src.nres) {
      uint64_t mine = 0;
      if (lane < src.nres) {
        int c = 0;
#pragma unroll
        for (int i = 0; i < W; i++) c += __popcll(d.w[i] & __ldg(src.rmask + lane * W + i));
        int lo = __ldg(src.rmin + lane), hi = __ldg(src.rmax + lane);
#pragma unroll
        for (int D = -2; D <= 2; D++)
          if (c + D >= lo && c + D <= hi) mine |= 1ull << (5 * lane + D + 2);
      }
      uint32_t a = __reduce_or_sync(FULL, (uint32_t)mine), b = __reduce_or_sync(FULL, (uint32_t)(mine >> 32));
      okm = (uint64_t)a | ((uint64_t)b << 32);
    }
    if (lv.on) {
      int b = __ldg(lv.cfg + get_local<W>(d, lv.lo, lv.lmask));
      int64_t off = r - (int64_t)__ldg(lv.bstart + b);
      uint32_t e0 = __ldg(lv.eoff + b), e1 = __ldg(lv.eoff + b + 1);
      for (uint32_t e = e0; e < e1; e += 32) {
        uint32_t ee = e + lane;
        bool has = false;
        int64_t j = 0;
        double vr = 0.0, vi = 0.0;
        if (ee < e1) {
          const LocalEntry *E = lv.ent + ee;
          uint32_t te = __ldg(&E->tend);
          j = (int64_t)__ldg(&E->tstart) + off;
          if (te >> 31) {
            has = true;
          } else {
            Key<W> s = set_local<W>(d, lv.lo, lv.lmask, __ldg(lv.etarget + ee));
            if (j < (int64_t)(te & 0x7FFFFFFFu)) has = qg_eq<W>(rows[j], s);
            if (!has) {
              bool ok = true;
              if (src.nres) {
                uint64_t req = __ldg(&E->wreq);
                ok = wreq ? ((okm & req) == req) : in_windows<W>(s, src);
              }
              if (ok) {
                int64_t h = qg_find_slot<W>(src.slots, src.hmask, s, err);
                if (h >= 0) {
                  j = (int64_t)__ldg(src.slot_row + h);
                  has = true;
                }
              }
            }
          }
          if (has) {
            vr = __ldg(&E->vre);
            vi = __ldg(&E->vim);
          }
        }
        append(has, j, vr, vi);
      }
    }
    // table terms, one per lane per round, in table order
    for (int t0 = 0; t0 < nterms; t0 += 32) {
      int t = t0 + lane;
      bool has = false;
      int64_t j = 0;
      double vr = 0.0, vi = 0.0;
      if (t < nterms) {
        const GroupDev<W> &G = groups[tgrp[t]];
        const TermDev<W> &T = terms[t];
        bool app = true, dgt = true;
        Key<W> s;
#pragma unroll
        for (int i = 0; i < W; i++) {
          app &= (d.w[i] & G.need1[i]) == G.need1[i];
          app &= (d.w[i] & T.need0[i]) == 0;
          s.w[i] = d.w[i] ^ T.flip[i];
          dgt &= T.flip[i] == 0;
        }
        if (app) {
          if (dgt) {
            j = r;
            has = true;
          } else {
            bool ok = true;
            if (src.nres) {
              if (wreq) {
                uint64_t req = __ldg(wreq + t);
                ok = (okm & req) == req;
              } else {
                ok = in_windows<W>(s, src);
              }
            }
            if (ok) {
              int64_t h = qg_find_slot<W>(src.slots, src.hmask, s, err);
              if (h >= 0) {
                j = (int64_t)__ldg(src.slot_row + h);
                has = true;
              }
            }
          }
          if (has) {
            int par = 0;
#pragma unroll
            for (int i = 0; i < W; i++) par += __popcll(d.w[i] & T.sgn[i]);
            vr = qg_flip_sign(T.vre, par);
            vi = qg_flip_sign(T.vim, par);
          }
        }
      }
      append(has, j, vr, vi);
    }
    flush();
#pragma unroll
    for (int m = 0; m < VPL; m++) {
      int k = lane + 32 * m;
      if (k >= nv) continue;
      if (!FUSE) {
        y[r * ys + vec0 + k] = acc[m];
      } else {
        dsum[m].x += qg_redot(x[r * xs + vec0 + k], acc[m]);
        y[r * ys + vec0 + k] = qg_axpy2(acc[m], fz.beta[vec0 + k], fz.prev[r * ys + vec0 + k]);
      }
    }
  }
  if (FUSE) {
    __shared__ double2 red[8][32 * VPL];
#pragma unroll
    for (int m = 0; m < VPL; m++) red[wid][lane + 32 * m] = dsum[m];
    __syncthreads();
    for (int k = threadIdx.x; k < nv && k < 32 * VPL; k += blockDim.x) {
      double sacc = 0.0;
      for (int w = 0; w < 8; w++) sacc += red[w][k].x;
      fz.dot_part[blockIdx.x * ys + vec0 + k] = make_double2(sacc, 0.0);
    }
  }
  if (SMEM && pending) mbar_wait_bounded(smem_addr(&s_bar), 0);
}

// ------------------------------------------------------------------ connection lists
//
// k_apply resolves a connection that has no certain offset through the hash table on every
// H*psi: it hashes the source key, probes (one random 32-byte sector of a table twice the
// basis), and for several vectors reads the slot's row.  The sources do not change between
// the H*psi calls of a Lanczos run, so k_conn resolves them once per (operator, basis), in
// the order k_apply visits them, into per-row lists of (source row, meta); k_apply_list then
// gathers x[source] by row.  Rows of a warp are neighbours in the sorted basis and a term
// maps sorted sources monotonically to sorted targets, so their sources are neighbours too:
// the gathers share sectors and stay in L2, where hashed probes scatter over the table.
// Both kernels follow k_apply's visiting order exactly, so each row's sum is bitwise the same.

// One pass over a row's connections: FILL = false counts them into cnt[r], FILL = true
// writes them at cptr[r] (bounded by cptr[r + 1]).
template <int W, bool FILL>
__global__ void __launch_bounds__(256) k_conn(const Key<W> *__restrict__ rows, int64_t n_rows,
                                              const GroupDev<W> *__restrict__ groups, const TermDev<W> *__restrict__ terms,
                                              int ngroups, int nhop, uint64_t hop0, uint64_t hop1, SrcView src,
                                              LocalView lv, const uint64_t *__restrict__ wreq, int64_t *cptr,
                                              uint2 *conn, unsigned int *err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  const Key<W> d = rows[r];
  const int64_t p0 = FILL ? cptr[r] : 0, pend = FILL ? cptr[r + 1] : 0;
  int64_t c = 0;
  auto emit = [&](uint32_t j, uint32_t meta) {
    if (FILL) {
      if (p0 + c < pend)
        conn[p0 + c] = make_uint2(j, meta);
      else
        atomicOr(err, QG_DEVERR_OVERFLOW);
    }
    c++;
  };
  uint64_t okm = 0;
  if (wreq && src.nres) okm = window_bits<W>(d, src);
  if (lv.on) {
    int b = __ldg(lv.cfg + get_local<W>(d, lv.lo, lv.lmask));
    int64_t off = r - (int64_t)__ldg(lv.bstart + b);
    uint32_t e1 = __ldg(lv.eoff + b + 1);
    for (uint32_t e = __ldg(lv.eoff + b); e < e1; e++) {
      const LocalEntry *E = lv.ent + e;
      uint32_t te = __ldg(&E->tend);
      if (te >> 31) continue;  // certain offset: no list entry
      int64_t j = (int64_t)__ldg(&E->tstart) + off;
      Key<W> s = set_local<W>(d, lv.lo, lv.lmask, __ldg(lv.etarget + e));
      bool hit = false;
      if (j < (int64_t)(te & 0x7FFFFFFFu)) hit = qg_eq<W>(rows[j], s);
      if (!hit) {
        if (src.nres) {
          uint64_t req = __ldg(&E->wreq);
          if (wreq ? ((okm & req) != req) : !in_windows<W>(s, src)) {
            emit(QG_NO_INDEX, 0);
            continue;
          }
        }
        int64_t h = qg_find_slot<W>(src.slots, src.hmask, s, err);
        if (h < 0) {
          emit(QG_NO_INDEX, 0);
          continue;
        }
        j = (int64_t)__ldg(src.slot_row + h);
      }
      emit((uint32_t)j, 0);
    }
  }
  auto term = [&](int t, bool known_applicable) {
    const TermDev<W> &T = terms[t];
    if (!known_applicable) {
      bool app = true;
#pragma unroll
      for (int i = 0; i < W; i++) app &= (d.w[i] & T.need0[i]) == 0;
      if (!app) return;
    }
    Key<W> s;
    bool dg = true;
#pragma unroll
    for (int i = 0; i < W; i++) {
      uint64_t fl = T.flip[i];
      s.w[i] = d.w[i] ^ fl;
      dg &= fl == 0;
    }
    int64_t j = r;
    if (!dg) {
      if (src.nres) {
        if (wreq) {
          uint64_t req = __ldg(wreq + t);
          if ((okm & req) != req) return;
        } else if (!in_windows<W>(s, src)) {
          return;
        }
      }
      int64_t h = qg_find_slot<W>(src.slots, src.hmask, s, err);
      if (h < 0) return;
      j = (int64_t)__ldg(src.slot_row + h);
    }
    int par = 0;
#pragma unroll
    for (int i = 0; i < W; i++) par += __popcll(d.w[i] & T.sgn[i]);
    emit((uint32_t)j, (uint32_t)t | ((uint32_t)(par & 1) << 31));
  };
  int gbase = 0;
#pragma unroll
  for (int i = 0; i < W; i++) {
    uint64_t hm = i == 0 ? hop0 : hop1;
    uint64_t m = d.w[i] & hm;
    while (m) {
      int bp = __ffsll((long long)m) - 1;
      m &= m - 1;
      const GroupDev<W> &G = groups[gbase + __popcll(hm & ((1ull << bp) - 1))];
      int tq = G.begin;
#pragma unroll
      for (int i2 = 0; i2 < W; i2++) {
        uint64_t qm = G.qmask[i2];
        uint64_t cm = qm & ~d.w[i2];
        while (cm) {
          int bq = __ffsll((long long)cm) - 1;
          cm &= cm - 1;
          term(tq + __popcll(qm & ((1ull << bq) - 1)), true);
        }
        tq += __popcll(qm);
      }
    }
    gbase += __popcll(hm);
  }
  for (int g = nhop; g < ngroups; g++) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < W; i++) {
      uint64_t n1 = groups[g].need1[i];
      ok &= (d.w[i] & n1) == n1;
    }
    if (!ok) continue;
    int tb = groups[g].begin, te = groups[g].end;
    for (int t = tb; t < te; t++) term(t, false);
  }
  if (!FILL) cptr[r] = c;
}

// The apply over connection lists: diagonal, local moves (certain offsets inline, the others
// from the list), then the listed table connections; the arithmetic of each connection is
// k_apply's (qg_cmac with the parity-flipped value), in the same order.
//
// Rows of a warp share their local moves (one block of the sorted basis) but not the lengths
// of their lists, so a warp would run its list loop as long as its longest row with the other
// lanes idle -- on FP64 issue, the kernel's limit.  With REGROUP the block's 256 rows are
// dealt out again after the local moves, sorted by the length of what is left of their lists
// (a counting sort in shared memory), so each warp continues 32 rows of about equal length.
// Each row keeps its accumulator and its order of summation, so the output is bitwise the
// same; the fused epilogue's dot partials are reduced in the original row order.
// the list kernel reads (tstart, tend) and (vre, vim) of a LocalEntry as vector loads
static_assert(sizeof(LocalEntry) == 32 && offsetof(LocalEntry, tend) == 4 && offsetof(LocalEntry, vre) == 16 &&
                  offsetof(LocalEntry, vim) == 24,
              "LocalEntry layout");
#ifndef QG_LIST_REGROUP
#define QG_LIST_REGROUP 1
#endif
#define QG_REGROUP_BUCKETS 64

//
// REAL: every value of the operator is real (the diagonal, the local entries and the listed
// coefficients), so each connection is two FMAs and no imaginary part is read or tested.  The
// general form's per-connection test of the imaginary part compiles to predicated FMAs, which
// hold the FP64 pipe whether or not they take effect; a real operator would pay for all four.
// acc += v x[idx] for a real value v: RV, x holds one real number per row (a real vector; the
// products a complex vector with a zero imaginary part would form, without the zero half)
template <bool RV>
__device__ __forceinline__ void acc_real_term(double2 &acc, double v, const double2 *__restrict__ x, int64_t idx) {
  if (RV)
    acc.x = fma(v, __ldg(reinterpret_cast<const double *>(x) + idx), acc.x);
  else
    qg_cmac(acc, v, 0.0, false, __ldg(x + idx));
}

// ORD: y is host memory (see the store at the end).  SPLIT (with FUSE and REAL): each complex
// vector carries two real Lanczos chains, its real and imaginary parts.  RV (with FUSE, REAL
// and NV = 1): x, y and prev hold one real number per row.
template <int W, int NV, bool FUSE, bool REAL, bool ORD = false, bool SPLIT = false, bool RV = false>
__global__ void __launch_bounds__(256, NV == 1 ? QG_APPLY_MIN_BLOCKS : 1)
    k_apply_list(const Key<W> *__restrict__ rows, int64_t n_rows, const int64_t *__restrict__ cptr,
                 const uint2 *__restrict__ conn, const double2 *__restrict__ coef, const double2 *__restrict__ diag,
                 const double2 *__restrict__ x, int xs, double2 *__restrict__ y, int ys, int vec0, ApplyFuse fz,
                 LocalView lv) {
  vec0 += blockIdx.y * NV;  // passes of NV vectors side by side (gridDim.y of them)
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool live = r < n_rows;
  double2 acc[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) acc[k] = make_double2(0.0, 0.0);
  int64_t p = 0, pe = 0;
  if (live) {
    if (diag) {
      const double2 dg = diag[r];
      const bool dgc = !REAL && qg_is_nonzero(dg.y);
#pragma unroll
      for (int k = 0; k < NV; k++)
        acc[k] = RV ? make_double2(dg.x * reinterpret_cast<const double *>(x)[r], 0.0)
                    : qg_diag_mul(dg, x[r * xs + vec0 + k], dgc);
    }
    p = __ldg(cptr + r);
    pe = __ldg(cptr + r + 1);
    if (lv.on) {
      const Key<W> d = rows[r];
      int b = __ldg(lv.cfg + get_local<W>(d, lv.lo, lv.lmask));
      int64_t off = r - (int64_t)__ldg(lv.bstart + b);
      uint32_t e1 = __ldg(lv.eoff + b + 1);
#pragma unroll(kLocalUnroll)
      for (uint32_t e = __ldg(lv.eoff + b); e < e1; e++) {
        const LocalEntry *E = lv.ent + e;
        // (tstart, tend) and (vre, vim) as two vector loads (entries are 32-byte aligned)
        const uint2 tt = __ldg(reinterpret_cast<const uint2 *>(&E->tstart));
        int64_t j;
        if (tt.y >> 31) {
          j = (int64_t)tt.x + off;
        } else {
          uint32_t js = p < pe ? __ldg(&conn[p].x) : QG_NO_INDEX;
          p++;
          if (js == QG_NO_INDEX) continue;
          j = js;
        }
        if (REAL) {
          const double v = __ldg(&E->vre);
#pragma unroll
          for (int k = 0; k < NV; k++) acc_real_term<RV>(acc[k], v, x, j * xs + vec0 + k);
        } else {
          const double2 v = __ldg(reinterpret_cast<const double2 *>(&E->vre));
          bool cplx = qg_is_nonzero(v.y);
#pragma unroll
          for (int k = 0; k < NV; k++) qg_cmac(acc[k], v.x, v.y, cplx, __ldg(x + j * xs + vec0 + k));
        }
      }
    }
  }
  int me = threadIdx.x;  // the block position of the row this thread finishes
  // regrouped accumulators, then (FUSE) the rows' dot terms in their original order
  __shared__ double2 s_acc[QG_LIST_REGROUP || FUSE ? NV : 1][QG_LIST_REGROUP || FUSE ? 256 : 1];
  if (QG_LIST_REGROUP) {
    __shared__ int s_cnt[QG_REGROUP_BUCKETS];
    __shared__ int64_t s_p[256], s_pe[256];
    __shared__ int s_me[256];
    if (threadIdx.x < QG_REGROUP_BUCKETS) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    int64_t left = live && pe > p ? pe - p : 0;
    int bucket = (int)(left < QG_REGROUP_BUCKETS - 1 ? left : QG_REGROUP_BUCKETS - 1);
    atomicAdd(&s_cnt[bucket], 1);
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of the bucket counts, longest lists first
      int lane = threadIdx.x;
      int c0 = s_cnt[QG_REGROUP_BUCKETS - 1 - 2 * lane], c1 = s_cnt[QG_REGROUP_BUCKETS - 2 - 2 * lane];
      int v = c0 + c1, incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      int excl = incl - v;
      s_cnt[QG_REGROUP_BUCKETS - 1 - 2 * lane] = excl;
      s_cnt[QG_REGROUP_BUCKETS - 2 - 2 * lane] = excl + c0;
    }
    __syncthreads();
    int slot = atomicAdd(&s_cnt[bucket], 1);
    s_p[slot] = p;
    s_pe[slot] = live ? pe : p;
    s_me[slot] = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; k++) s_acc[k][slot] = acc[k];
    __syncthreads();
    p = s_p[threadIdx.x];
    pe = s_pe[threadIdx.x];
    me = s_me[threadIdx.x];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = s_acc[k][threadIdx.x];
    r = blockIdx.x * (int64_t)blockDim.x + me;
    live = r < n_rows;
  }
  if (live) {
    for (; p < pe; p++) {
      uint2 cn = __ldg(conn + p);
      int par = (int)(cn.y >> 31);
      int64_t j = cn.x;
      if (REAL) {
        double vr = qg_flip_sign(__ldg(&coef[cn.y & 0x7FFFFFFFu].x), par);
#pragma unroll
        for (int k = 0; k < NV; k++) acc_real_term<RV>(acc[k], vr, x, j * xs + vec0 + k);
      } else {
        double2 cf = __ldg(coef + (cn.y & 0x7FFFFFFFu));
        bool cplx = qg_is_nonzero(cf.y);
        double vr = qg_flip_sign(cf.x, par), vi = qg_flip_sign(cf.y, par);
#pragma unroll
        for (int k = 0; k < NV; k++) qg_cmac(acc[k], vr, vi, cplx, __ldg(x + j * xs + vec0 + k));
      }
    }
  }
  if (!FUSE) {
    if (QG_LIST_REGROUP && ORD) {
      // y in host memory (qg_apply_host): back to the original row order, so a warp stores 32
      // consecutive rows and the host link carries whole lines instead of 16-byte pieces (in
      // device memory the scattered stores of a block merge in L2 and cost nothing extra)
      __syncthreads();  // every regrouped accumulator has been read
#pragma unroll
      for (int k = 0; k < NV; k++) s_acc[k][me] = acc[k];
      __syncthreads();
      const int64_t r0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
      if (r0 < n_rows) {
#pragma unroll
        for (int k = 0; k < NV; k++) y[r0 * ys + vec0 + k] = s_acc[k][threadIdx.x];
      }
    } else if (live) {
#pragma unroll
      for (int k = 0; k < NV; k++) y[r * ys + vec0 + k] = acc[k];
    }
  } else if (RV) {
    // one real chain: y = H x - beta prev and the partial of <x|H x>, the arithmetic of the
    // real part of a complex chain whose imaginary part is zero
    __shared__ double s_red[8];
    double dvs[1] = {0.0};
    if (live) {
      const double xv = reinterpret_cast<const double *>(x)[r], pv = reinterpret_cast<const double *>(fz.prev)[r];
      dvs[0] = __dmul_rn(xv, acc[0].x);
      reinterpret_cast<double *>(y)[r] = fma(-fz.beta[0], pv, acc[0].x);
    }
    if (QG_LIST_REGROUP) __syncthreads();  // every regrouped accumulator has been read
    fused_dot_partials<1, false>(dvs, me, reinterpret_cast<double *>(&s_acc[0][0]), s_red, fz.dot_part, ys, vec0);
  } else if (SPLIT) {
    // two real chains per vector: the real operator keeps the parts apart, so each part is
    // updated and reduced with exactly the arithmetic of its chain run alone (a zero
    // imaginary part adds nothing to the real one): y = H x - beta prev per part with its
    // own beta, the partials of <x|H x> per part as .x and .y
    __shared__ double s_red[2 * NV * 8];
    double dvs[2 * NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double da = 0.0, db = 0.0;
      if (live) {
        const double2 xv = x[r * xs + vec0 + k], pv = fz.prev[r * ys + vec0 + k];
        da = __dmul_rn(xv.x, acc[k].x);
        db = __dmul_rn(xv.y, acc[k].y);
        y[r * ys + vec0 + k] = make_double2(fma(-fz.beta[2 * (vec0 + k)], pv.x, acc[k].x),
                                            fma(-fz.beta[2 * (vec0 + k) + 1], pv.y, acc[k].y));
      }
      dvs[2 * k] = da;
      dvs[2 * k + 1] = db;
    }
    if (QG_LIST_REGROUP) __syncthreads();  // every regrouped accumulator has been read
    fused_dot_partials<2 * NV, true>(dvs, me, reinterpret_cast<double *>(&s_acc[0][0]), s_red, fz.dot_part, ys,
                                     vec0);
  } else {
    // y = H x - beta prev and the block's partial of Re <x|H x>, reduced in the original row
    // order (the regrouped accumulators' storage holds the rows' terms)
    __shared__ double s_red[NV * 8];
    double dvs[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double dv = 0.0;
      if (live) {
        dv = qg_redot(x[r * xs + vec0 + k], acc[k]);
        y[r * ys + vec0 + k] = qg_axpy2(acc[k], fz.beta[vec0 + k], fz.prev[r * ys + vec0 + k]);
      }
      dvs[k] = dv;
    }
    if (QG_LIST_REGROUP) __syncthreads();  // every regrouped accumulator has been read
    fused_dot_partials<NV, false>(dvs, me, reinterpret_cast<double *>(&s_acc[0][0]), s_red, fz.dot_part, ys, vec0);
  }
}

// FP64 operations of one single-vector k_apply_list launch, counted per row as the kernel
// issues them: the diagonal 2 multiplies (real) or 4 (complex), each connection 2 FMAs (real
// value) or 4 (complex).  The exact work behind the FP64 ceiling of the roofline.
template <int W>
__global__ void k_count_fp64(const Key<W> *__restrict__ rows, int64_t n_rows, const int64_t *__restrict__ cptr,
                             const uint2 *__restrict__ conn, const double2 *__restrict__ coef,
                             const double2 *__restrict__ diag, LocalView lv, unsigned long long *out) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (r < n_rows) {
    if (diag) c += qg_is_nonzero(diag[r].y) ? 4 : 2;
    int64_t p = cptr[r];
    const int64_t pe = cptr[r + 1];
    if (lv.on) {
      const Key<W> d = rows[r];
      int b = lv.cfg[get_local<W>(d, lv.lo, lv.lmask)];
      uint32_t e1 = lv.eoff[b + 1];
      for (uint32_t e = lv.eoff[b]; e < e1; e++) {
        const LocalEntry *E = lv.ent + e;
        if (!(E->tend >> 31)) {
          uint32_t js = p < pe ? conn[p].x : QG_NO_INDEX;
          p++;
          if (js == QG_NO_INDEX) continue;
        }
        c += qg_is_nonzero(E->vim) ? 4 : 2;
      }
    }
    for (; p < pe; p++) c += qg_is_nonzero(coef[conn[p].y & 0x7FFFFFFFu].y) ? 4 : 2;
  }
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

int qg_apply_grid(qg_basis dst) { return (int)std::max<int64_t>(1, (dst->n + 255) / 256); }

template <int W, int NV, bool FUSE, bool SMEM>
static void launch_apply_t(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int vec0, const ApplyFuse &fz,
                           const LocalView &lv, const uint64_t *wreq) {
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
      (const Key<W> *)dst->d_keys, dst->n, (const unsigned char *)tab.d_blob, (uint32_t)tab.bytes, tab.ngroups,
      tab.nhop, tab.hopmask[0], tab.hopmask[1], diag, sv, packed, dst == src, x, xs, y, ys, vec0, fz, lv, wreq,
      ctx->d_err);
  ctx->launches++;
}

template <int W, int VPL, bool FUSE, bool SMEM>
static void launch_apply_warp_t(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst,
                                qg_basis src, const double2 *x, int xs, double2 *y, int ys, int vec0, int nv,
                                const ApplyFuse &fz, const LocalView &lv, const uint64_t *wreq) {
  size_t smem = SMEM ? tab.bytes : 0;
  if (SMEM) {
    static bool attr_done = false;
    if (!attr_done) {
      cudaFuncSetAttribute(k_apply_warp<W, VPL, FUSE, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           QG_SMEM_TABLE_MAX);
      attr_done = true;
    }
  }
  SrcView sv{src->d_slots, src->d_slot_row, (uint64_t)(src->hcap - 1), src->nres, src->d_rmask, src->d_rmin,
             src->d_rmax};
  k_apply_warp<W, VPL, FUSE, SMEM><<<qg_apply_grid(dst), 256, smem, ctx->stream>>>(
      (const Key<W> *)dst->d_keys, dst->n, (const unsigned char *)tab.d_blob, (uint32_t)tab.bytes, tab.ngroups,
      tab.nterms, (uint32_t)tab.tgrp_off, diag, sv, x, xs, y, ys, vec0, nv, fz, lv, wreq, ctx->d_err);
  ctx->launches++;
}

template <int W, bool FUSE, bool SMEM>
static void launch_apply_w(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int nvec, const ApplyFuse &fz,
                           const LocalView &lv, const uint64_t *wreq, int chunk) {
  if (chunk < 0 && dst == src) {
    // warp per row with lanes over vectors: passes of 32 or 64 vectors
    int per = -chunk;
    for (int v = 0; v < nvec; v += per) {
      int nv = std::min(per, nvec - v);
      if (per > 32)
        launch_apply_warp_t<W, 2, FUSE, SMEM>(ctx, tab, diag, dst, src, x, xs, y, ys, v, nv, fz, lv, wreq);
      else
        launch_apply_warp_t<W, 1, FUSE, SMEM>(ctx, tab, diag, dst, src, x, xs, y, ys, v, nv, fz, lv, wreq);
    }
    return;
  }
  if (chunk < 0) chunk = 8;
  int v = 0;
  while (v < nvec) {
    int left = std::min(nvec - v, chunk);
    if (left >= 8) {
      launch_apply_t<W, 8, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz, lv, wreq);
      v += 8;
    } else if (left >= 4) {
      launch_apply_t<W, 4, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz, lv, wreq);
      v += 4;
    } else if (left >= 2) {
      launch_apply_t<W, 2, FUSE, SMEM>(ctx, tab, diag, dst, src, 0, x, xs, y, ys, v, fz, lv, wreq);
      v += 2;
    } else {
      launch_apply_t<W, 1, FUSE, SMEM>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, v, fz, lv, wreq);
      v += 1;
    }
  }
}

template <int W, bool FUSE>
static void launch_apply_s(qg_context ctx, const HostTable &tab, const double2 *diag, qg_basis dst, qg_basis src,
                           int packed, const double2 *x, int xs, double2 *y, int ys, int nvec, const ApplyFuse &fz,
                           const LocalView &lv, const uint64_t *wreq, int chunk) {
  if (tab.bytes <= QG_SMEM_TABLE_MAX)
    launch_apply_w<W, FUSE, true>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, nvec, fz, lv, wreq, chunk);
  else
    launch_apply_w<W, FUSE, false>(ctx, tab, diag, dst, src, packed, x, xs, y, ys, nvec, fz, lv, wreq, chunk);
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
    if (!(qg_norm2(v) > t2)) v = make_double2(0.0, 0.0);  // the reference keeps |a|^2 > eps^2
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

template <int W>
__global__ void k_local_cfg(const Key<W> *keys, int64_t n, int lo, uint32_t lmask, uint32_t *cfg, uint32_t *flag) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint32_t c = get_local<W>(keys[r], lo, lmask);
  cfg[r] = c;
  flag[r] = (r == 0) ? 1u : (get_local<W>(keys[r - 1], lo, lmask) != c ? 1u : 0u);
}

__global__ void k_block_scatter(const uint32_t *cfg, const uint32_t *flag, const uint32_t *pos, int64_t n,
                                uint32_t *bstart, uint32_t *bcfg) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  if (flag[r]) {
    bstart[pos[r] - 1] = (uint32_t)r;
    bcfg[pos[r] - 1] = cfg[r];
  }
}

// Block classes: two blocks whose rows list the same non-local configurations (same count,
// same sorted non-local parts) align row by row, so a local move between them needs no check.
// A per-block fingerprint (two sums of mixed non-local parts) proposes the classes; an exact
// row-by-row comparison with the class representative confirms each member.

template <int W>
__device__ __forceinline__ Key<W> nonlocal_part(const Key<W> &d, int lo, uint32_t lmask) {
  return set_local<W>(d, lo, lmask, 0u);
}

// one CTA per block of rows: the sums of two mixes of the rows' non-local parts (modulo 2^64,
// so the order of summation does not matter)
template <int W>
__global__ void k_block_fp(const Key<W> *keys, const uint32_t *bstart, int lo, uint32_t lmask,
                           unsigned long long *fp) {
  __shared__ unsigned long long sa[256], sb[256];
  int blk = blockIdx.x;
  uint32_t r0 = bstart[blk], r1 = bstart[blk + 1];
  unsigned long long a = 0, b = 0;
  for (uint32_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    Key<W> k = nonlocal_part<W>(keys[r], lo, lmask);
    uint64_t x = k.w[0], y = W == 2 ? k.w[W - 1] : 0x9e3779b97f4a7c15ull;
    a += qg_mix64(x ^ qg_mix64(y + 0x632be59bd9b4e019ull));
    b += qg_mix64(y ^ qg_mix64(x + 0x8cb92ba72f3d8dd7ull));
  }
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sa[threadIdx.x] += sa[threadIdx.x + o];
      sb[threadIdx.x] += sb[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    fp[2 * (size_t)blk] = sa[0];
    fp[2 * (size_t)blk + 1] = sb[0];
  }
}

template <int W>
__global__ void k_block_verify(const Key<W> *keys, int64_t n, int lo, uint32_t lmask, const uint32_t *pos,
                               const uint32_t *bstart, const uint32_t *rep, uint32_t *mismatch) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint32_t blk = pos[r] - 1, rp = rep[blk];
  if (rp == blk) return;
  int64_t j = (int64_t)bstart[rp] + (r - (int64_t)bstart[blk]);
  Key<W> a = nonlocal_part<W>(keys[r], lo, lmask), b = nonlocal_part<W>(keys[j], lo, lmask);
  if (!qg_eq<W>(a, b)) mismatch[blk] = 1u;
}

void qg_cache_free(OpBasisCache &c) {
  cudaFree(c.d_diag);
  cudaFree(c.d_wreq);
  cudaFree(c.d_bstart);
  cudaFree(c.d_cfg);
  cudaFree(c.d_eoff);
  cudaFree(c.d_ent);
  cudaFree(c.d_ent_target);
  cudaFree(c.d_cptr);
  cudaFree(c.d_conn);
  cudaFree(c.d_coef);
  c = OpBasisCache();
}

namespace {

inline int popc2(const uint64_t *a, const uint64_t *b, const uint64_t *c, int W) {
  int n = 0;
  for (int i = 0; i < W; i++) n += __builtin_popcountll(a[i] & b[i] & c[i]);
  return n;
}

// window bits a move needs: D_q = (bits turned on) - (bits turned off) inside window q;
// returns false when some |D_q| > 2 (the encoding cannot express it)
bool move_bits(const qg_basis b, const uint64_t *on, const uint64_t *offb, uint64_t &req) {
  req = 0;
  uint64_t ones[2] = {~0ull, ~0ull};
  for (int q = 0; q < b->nres; q++) {
    const uint64_t *m = &b->h_rmask[(size_t)q * b->W];
    int D = popc2(on, m, ones, b->W) - popc2(offb, m, ones, b->W);
    if (D == 0) continue;
    if (D < -2 || D > 2) return false;
    req |= 1ull << (5 * q + D + 2);
  }
  return true;
}

// local-bit masks (bits lo.. of a W-word key) -> H-bit integer
uint32_t to_local(const uint64_t *m, int lo, int W) {
  if (W == 1) return (uint32_t)(m[0] >> lo);
  if (lo >= 64) return (uint32_t)(m[1] >> (lo - 64));
  return (uint32_t)((m[0] >> lo) | (lo ? (m[1] << (64 - lo)) : 0ull));
}

void from_local(uint32_t c, int lo, int W, uint64_t *out) {
  out[0] = out[1] = 0;
  if (W == 1) {
    out[0] = (uint64_t)c << lo;
  } else if (lo >= 64) {
    out[1] = (uint64_t)c << (lo - 64);
  } else {
    out[0] = (uint64_t)c << lo;
    if (lo) out[1] = (uint64_t)c >> (64 - lo);
  }
}

}  // namespace

static qg_status build_local(qg_basis bs, qg_operator op, OpBasisCache &c) {
  qg_context ctx = bs->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = bs->n;
  int H = op->H, lo = bs->nf - H, W = bs->W;
  uint32_t lmask = (H >= 32) ? 0xFFFFFFFFu : ((1u << H) - 1);
  uint32_t *cfg = nullptr, *flag = nullptr, *pos = nullptr, *bst = nullptr, *bcf = nullptr;
  void *tmp = nullptr;
  size_t tb = 0;
  cudaError_t e = cudaMalloc(&cfg, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&flag, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&pos, n * 4);
  if (e == cudaSuccess) e = cub::DeviceScan::InclusiveSum(nullptr, tb, flag, pos, (int)n, s);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, tb);
  if (e == cudaSuccess) {
    if (W == 1)
      k_local_cfg<1><<<grid_for(n, 256), 256, 0, s>>>((const Key<1> *)bs->d_keys, n, lo, lmask, cfg, flag);
    else
      k_local_cfg<2><<<grid_for(n, 256), 256, 0, s>>>((const Key<2> *)bs->d_keys, n, lo, lmask, cfg, flag);
    ctx->launches++;
    e = cub::DeviceScan::InclusiveSum(tmp, tb, flag, pos, (int)n, s);
    ctx->launches += 2;
  }
  uint32_t nb = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nb, pos + n - 1, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMalloc(&bst, (size_t)(nb + 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&bcf, (size_t)nb * 4 + 4);
  if (e == cudaSuccess) {
    k_block_scatter<<<grid_for(n, 256), 256, 0, s>>>(cfg, flag, pos, n, bst, bcf);
    ctx->launches++;
  }
  std::vector<uint32_t> hstart(nb + 1), hcfg(nb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hstart.data(), bst, (size_t)nb * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hcfg.data(), bcf, (size_t)nb * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  hstart[nb] = (uint32_t)n;
  if (e == cudaSuccess) e = cudaMemcpyAsync(bst + nb, &hstart[nb], 4, cudaMemcpyHostToDevice, s);
  // block classes (rows of blocks in one class align)
  std::vector<uint32_t> cls(nb);
  for (uint32_t k = 0; k < nb; k++) cls[k] = k;
  {
    unsigned long long *fp = nullptr;
    uint32_t *rep = nullptr, *mis = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&fp, (size_t)nb * 16 + 16);
    if (e == cudaSuccess) e = cudaMalloc(&rep, (size_t)nb * 4 + 4);
    if (e == cudaSuccess) e = cudaMalloc(&mis, (size_t)nb * 4 + 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(mis, 0, (size_t)nb * 4 + 4, s);
    if (e == cudaSuccess) {
      if (W == 1)
        k_block_fp<1><<<nb, 256, 0, s>>>((const Key<1> *)bs->d_keys, bst, lo, lmask, fp);
      else
        k_block_fp<2><<<nb, 256, 0, s>>>((const Key<2> *)bs->d_keys, bst, lo, lmask, fp);
      ctx->launches++;
    }
    std::vector<unsigned long long> hfp((size_t)2 * nb);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hfp.data(), fp, (size_t)nb * 16, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    std::vector<uint32_t> hrep(nb);
    if (e == cudaSuccess) {
      std::map<std::tuple<uint32_t, unsigned long long, unsigned long long>, uint32_t> first;
      for (uint32_t k = 0; k < nb; k++) {
        auto key = std::make_tuple(hstart[k + 1] - hstart[k], hfp[2 * k], hfp[2 * k + 1]);
        auto it = first.find(key);
        hrep[k] = it == first.end() ? (first[key] = k) : it->second;
      }
      e = cudaMemcpyAsync(rep, hrep.data(), (size_t)nb * 4, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess) {
      if (W == 1)
        k_block_verify<1><<<grid_for(n, 256), 256, 0, s>>>((const Key<1> *)bs->d_keys, n, lo, lmask, pos, bst, rep,
                                                           mis);
      else
        k_block_verify<2><<<grid_for(n, 256), 256, 0, s>>>((const Key<2> *)bs->d_keys, n, lo, lmask, pos, bst, rep,
                                                           mis);
      ctx->launches++;
    }
    std::vector<uint32_t> hmis(nb);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hmis.data(), mis, (size_t)nb * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess)
      for (uint32_t k = 0; k < nb; k++) cls[k] = hmis[k] ? k : hrep[k];
    cudaFree(fp);
    cudaFree(rep);
    cudaFree(mis);
  }
  cudaFree(cfg);
  cudaFree(flag);
  cudaFree(pos);
  cudaFree(tmp);
  cudaFree(bcf);
  if (e != cudaSuccess) {
    cudaFree(bst);
    return qg_cuda_fail(ctx, e, "local blocks");
  }
  // configuration -> block
  std::vector<int32_t> table((size_t)1 << H, -1);
  for (uint32_t k = 0; k < nb; k++) table[hcfg[k]] = (int32_t)k;
  // local terms in H-bit form
  struct LT {
    uint32_t n1, n0, fl, sg;
    double re, im;
  };
  std::vector<LT> lt;
  for (auto &t : op->local_off)
    lt.push_back({to_local(t.n1, lo, W), to_local(t.n0, lo, W), to_local(t.fl, lo, W), to_local(t.sg, lo, W), t.re,
                  t.im});
  std::vector<uint32_t> eoff(nb + 1, 0);
  std::vector<LocalEntry> ent;
  std::vector<uint32_t> etarget;
  bool exact = true;
  for (uint32_t k = 0; k < nb; k++) {
    uint32_t cc = hcfg[k];
    std::map<uint32_t, std::pair<double, double>> acc;
    for (auto &t : lt) {
      if ((cc & t.n1) != t.n1 || (cc & t.n0)) continue;
      uint32_t tg = cc ^ t.fl;
      double sg = (__builtin_popcount(cc & t.sg) & 1) ? -1.0 : 1.0;
      auto &v = acc[tg];
      v.first += sg * t.re;
      v.second += sg * t.im;
    }
    eoff[k] = (uint32_t)ent.size();
    for (auto &kv : acc) {
      int32_t tbk = table[kv.first];
      if (tbk < 0 || (!op->keep_zero && kv.second.first == 0.0 && kv.second.second == 0.0)) continue;
      LocalEntry le;
      le.tstart = hstart[tbk];
      le.tend = hstart[tbk + 1] | (cls[k] == cls[tbk] ? 0x80000000u : 0u);
      etarget.push_back(kv.first);
      le.vre = kv.second.first;
      le.vim = kv.second.second;
      le.wreq = 0;
      if (bs->nres) {
        uint64_t on[2], offb[2];
        from_local(kv.first & ~cc, lo, W, on);
        from_local(cc & ~kv.first, lo, W, offb);
        exact &= move_bits(bs, on, offb, le.wreq);
      }
      ent.push_back(le);
    }
  }
  eoff[nb] = (uint32_t)ent.size();
  c.nblocks = (int)nb;
  c.nent = (int64_t)ent.size();
  c.h_bcfg = hcfg;
  c.h_eoff = eoff;
  c.h_etarget = etarget;
  c.h_ent = ent;
  c.d_bstart = bst;
  e = cudaMalloc(&c.d_cfg, table.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(c.d_cfg, table.data(), table.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c.d_eoff, eoff.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(c.d_eoff, eoff.data(), eoff.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c.d_ent, std::max<size_t>(ent.size(), 1) * sizeof(LocalEntry));
  if (e == cudaSuccess && !ent.empty())
    e = cudaMemcpy(c.d_ent, ent.data(), ent.size() * sizeof(LocalEntry), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c.d_ent_target, std::max<size_t>(etarget.size(), 1) * 4);
  if (e == cudaSuccess && !etarget.empty())
    e = cudaMemcpy(c.d_ent_target, etarget.data(), etarget.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "local entries");
  if (!exact) c.wreq_exact = false;
  return QG_OK;
}

// New values of a sum operator's local entries on the blocks of a cache (same entries, same
// order: the entry set of a sum operator does not depend on its values).
static qg_status refresh_local(qg_basis bs, qg_operator op, OpBasisCache &c) {
  if (c.nent == 0) return QG_OK;
  int H = op->H, lo = bs->nf - H, W = bs->W;
  struct LT {
    uint32_t n1, n0, fl, sg;
    double re, im;
  };
  std::vector<LT> lt;
  for (auto &t : op->local_off)
    lt.push_back({to_local(t.n1, lo, W), to_local(t.n0, lo, W), to_local(t.fl, lo, W), to_local(t.sg, lo, W), t.re,
                  t.im});
  for (size_t k = 0; k + 1 < c.h_eoff.size(); k++) {
    uint32_t cc = c.h_bcfg[k];
    std::map<uint32_t, std::pair<double, double>> acc;
    for (auto &t : lt) {
      if ((cc & t.n1) != t.n1 || (cc & t.n0)) continue;
      double sg = (__builtin_popcount(cc & t.sg) & 1) ? -1.0 : 1.0;
      auto &v = acc[cc ^ t.fl];
      v.first += sg * t.re;
      v.second += sg * t.im;
    }
    for (uint32_t e = c.h_eoff[k]; e < c.h_eoff[k + 1]; e++) {
      auto &v = acc[c.h_etarget[e]];
      c.h_ent[e].vre = v.first;
      c.h_ent[e].vim = v.second;
    }
  }
  QG_CUDA(bs->ctx, cudaMemcpyAsync(c.d_ent, c.h_ent.data(), c.h_ent.size() * sizeof(LocalEntry),
                                   cudaMemcpyHostToDevice, bs->ctx->stream));
  return QG_OK;
}

static void launch_diag(qg_context ctx, qg_operator op, qg_basis b, double *d_diag);
template <int W>
__global__ void k_term_coef(const TermDev<W> *__restrict__ terms, int nterms, double2 *coef);

// A sum operator was rescaled since this cache was built: recompute what depends on values
// (the diagonal, the local entries' values, the list coefficients); the structure -- blocks,
// entries, window bits, connection lists -- stays.
static qg_status refresh_values(qg_basis b, qg_operator op, OpBasisCache &c) {
  qg_context ctx = b->ctx;
  // the refresh must run now, not be recorded into a graph being captured
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    ctx->last_error = "a rescaled operator was first used on this basis under stream capture";
    return QG_ERR_ARG;
  }
  if (b->n) launch_diag(ctx, op, b, c.d_diag);
  if (op->H > 0) QG_TRY(refresh_local(b, op, c));
  if (c.conn_state == 1) {
    const HostTable &tab = op->H > 0 ? op->pull_nl : op->pull_off;
    if (tab.nterms > 0) {
      if (b->W == 1)
        k_term_coef<1><<<(tab.nterms + 255) / 256, 256, 0, ctx->stream>>>((const TermDev<1> *)tab.d_terms, tab.nterms,
                                                                          c.d_coef);
      else
        k_term_coef<2><<<(tab.nterms + 255) / 256, 256, 0, ctx->stream>>>((const TermDev<2> *)tab.d_terms, tab.nterms,
                                                                          c.d_coef);
      ctx->launches++;
    }
  }
  c.op_version = op->version;
  return qg_check_launch(ctx, "value refresh");
}

// the diagonal of op on every row of b (all flip == 0 terms), into d_diag
static void launch_diag(qg_context ctx, qg_operator op, qg_basis b, double *d_diag) {
  if (op->W == 1)
    k_diag<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<1> *)b->d_keys, b->n,
                                                            (const GroupDev<1> *)op->diag.d_groups, op->diag.ngroups,
                                                            (const TermDev<1> *)op->diag.d_terms, (double2 *)d_diag);
  else
    k_diag<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<2> *)b->d_keys, b->n,
                                                            (const GroupDev<2> *)op->diag.d_groups, op->diag.ngroups,
                                                            (const TermDev<2> *)op->diag.d_terms, (double2 *)d_diag);
  ctx->launches++;
}

OpBasisCache *qg_basis_cache(qg_basis b, qg_operator op, qg_status *st) {
  *st = QG_OK;
  for (auto &c : b->caches)
    if (c.op_uid == op->uid) {
      if (c.op_version != op->version) {
        *st = refresh_values(b, op, c);
        if (*st != QG_OK) return nullptr;
      }
      return &c;
    }
  qg_context ctx = b->ctx;
  if (b->caches.size() >= 4) {  // small cache: drop the oldest
    cudaStreamSynchronize(ctx->stream);
    qg_cache_free(b->caches.front());
    b->caches.erase(b->caches.begin());
  }
  OpBasisCache c;
  c.op_uid = op->uid;
  c.op_version = op->version;
  cudaError_t e = cudaMalloc(&c.d_diag, std::max<int64_t>(b->n, 1) * 16);
  if (e != cudaSuccess) {
    *st = qg_cuda_fail(ctx, e, "diagonal");
    return nullptr;
  }
  if (b->n) launch_diag(ctx, op, b, c.d_diag);
  // window bits of the non-local terms (encoding: 5 bits per window, moves of up to 2)
  c.wreq_exact = b->nres > 0 && b->nres <= 12;
  if (c.wreq_exact) {
    std::vector<uint64_t> wr(std::max<size_t>(op->nl_host.size(), 1), 0);
    for (size_t t = 0; t < op->nl_host.size() && c.wreq_exact; t++) {
      const HostTerm &h = op->nl_host[t];
      uint64_t on[2] = {h.fl[0] & h.n0[0], h.fl[1] & h.n0[1]}, offb[2] = {h.fl[0] & h.n1[0], h.fl[1] & h.n1[1]};
      c.wreq_exact = move_bits(b, on, offb, wr[t]);
    }
    if (c.wreq_exact) {
      e = cudaMalloc(&c.d_wreq, wr.size() * 8);
      if (e == cudaSuccess) e = cudaMemcpy(c.d_wreq, wr.data(), wr.size() * 8, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        qg_cache_free(c);
        *st = qg_cuda_fail(ctx, e, "window bits");
        return nullptr;
      }
    }
  }
  if (op->H > 0 && b->n > 0) {
    bool keep_exact = c.wreq_exact;
    *st = build_local(b, op, c);
    if (*st != QG_OK) {
      qg_cache_free(c);
      return nullptr;
    }
    if (keep_exact && !c.wreq_exact) {  // a local move outside the encoding: full checks
      cudaFree(c.d_wreq);
      c.d_wreq = nullptr;
    }
  }
  b->caches.push_back(c);
  *st = qg_check_launch(ctx, "operator-basis cache");
  return &b->caches.back();
}

// ------------------------------------------------------------------ connection lists (host)

// The table and local view the same-basis apply scans (also used by the list build).
static void same_basis_view(qg_operator op, qg_basis b, const OpBasisCache *c, const HostTable **tab, LocalView *lv,
                            const uint64_t **wreq) {
  *lv = LocalView{};
  lv->on = 0;
  *tab = &op->pull_off;
  *wreq = nullptr;
  if (op->H > 0) {
    *tab = &op->pull_nl;
    lv->on = 1;
    lv->lo = b->nf - op->H;
    lv->lmask = (1u << op->H) - 1;
    lv->cfg = c->d_cfg;
    lv->bstart = c->d_bstart;
    lv->eoff = c->d_eoff;
    lv->ent = c->d_ent;
    lv->etarget = c->d_ent_target;
    if (c->wreq_exact && c->d_wreq) *wreq = c->d_wreq;
  }
}

template <int W>
__global__ void k_term_coef(const TermDev<W> *__restrict__ terms, int nterms, double2 *coef) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nterms) coef[t] = make_double2(terms[t].vre, terms[t].vim);
}

template <int W>
static void launch_conn(qg_context ctx, qg_basis b, const HostTable &tab, const LocalView &lv, const uint64_t *wreq,
                        int64_t *cptr, uint2 *conn, bool fill) {
  SrcView sv{b->d_slots, b->d_slot_row, (uint64_t)(b->hcap - 1), b->nres, b->d_rmask, b->d_rmin, b->d_rmax};
  const GroupDev<W> *g = (const GroupDev<W> *)tab.d_groups;
  const TermDev<W> *t = (const TermDev<W> *)tab.d_terms;
  if (fill)
    k_conn<W, true><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<W> *)b->d_keys, b->n, g, t, tab.ngroups,
                                                                  tab.nhop, tab.hopmask[0], tab.hopmask[1], sv, lv,
                                                                  wreq, cptr, conn, ctx->d_err);
  else
    k_conn<W, false><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<W> *)b->d_keys, b->n, g, t,
                                                                   tab.ngroups, tab.nhop, tab.hopmask[0],
                                                                   tab.hopmask[1], sv, lv, wreq, cptr, conn,
                                                                   ctx->d_err);
  ctx->launches++;
}

// Build the connection lists of (op, b) into c.  Leaves conn_state = -1 (and the apply on the
// hash path) when the basis is too large for 32-bit rows, when the lists would take more than
// a quarter of the free device memory, or while the stream is being captured (then it is
// tried again on a later apply).
static qg_status build_conn(qg_context ctx, qg_operator op, qg_basis b, OpBasisCache &c) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return QG_OK;
  }
  c.conn_state = -1;
  const int64_t n = b->n;
  if (n <= 0 || n >= (int64_t)QG_NO_INDEX) return QG_OK;
  const HostTable *tab;
  LocalView lv;
  const uint64_t *wreq;
  same_basis_view(op, b, &c, &tab, &lv, &wreq);
  cudaStream_t s = ctx->stream;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return QG_OK;
  }
  const size_t ptr_bytes = (size_t)(n + 1) * 8;
  if (4 * 2 * ptr_bytes > fr) return QG_OK;
  int64_t *cnt = nullptr, *cptr = nullptr;
  void *tmp = nullptr;
  size_t tb = 0;
  cudaError_t e = cudaMalloc(&cnt, ptr_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&cptr, ptr_bytes);
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, cptr, n + 1, s);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, std::max<size_t>(tb, 16));
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt + n, 0, 8, s);
  if (e == cudaSuccess) {
    if (b->W == 1)
      launch_conn<1>(ctx, b, *tab, lv, wreq, cnt, nullptr, false);
    else
      launch_conn<2>(ctx, b, *tab, lv, wreq, cnt, nullptr, false);
    e = cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, cptr, n + 1, s);
    ctx->launches += 2;
  }
  int64_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, cptr + n, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(cnt);
  cudaFree(tmp);
  if (e != cudaSuccess) {
    cudaFree(cptr);
    return qg_cuda_fail(ctx, e, "connection counts");
  }
  QG_TRY(qg_check_device_error(ctx, "connection counts"));
  size_t conn_bytes = (size_t)std::max<int64_t>(total, 1) * sizeof(uint2);
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || 4 * conn_bytes > fr) {
    cudaGetLastError();
    cudaFree(cptr);
    return QG_OK;
  }
  uint2 *conn = nullptr;
  double2 *coef = nullptr;
  e = cudaMalloc(&conn, conn_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&coef, (size_t)std::max(tab->nterms, 1) * 16);
  if (e != cudaSuccess) {
    cudaFree(cptr);
    cudaFree(conn);
    cudaFree(coef);
    cudaGetLastError();
    return QG_OK;  // no room: the hash path stays
  }
  if (tab->nterms > 0) {
    if (b->W == 1)
      k_term_coef<1><<<(tab->nterms + 255) / 256, 256, 0, s>>>((const TermDev<1> *)tab->d_terms, tab->nterms, coef);
    else
      k_term_coef<2><<<(tab->nterms + 255) / 256, 256, 0, s>>>((const TermDev<2> *)tab->d_terms, tab->nterms, coef);
    ctx->launches++;
  }
  if (b->W == 1)
    launch_conn<1>(ctx, b, *tab, lv, wreq, cptr, conn, true);
  else
    launch_conn<2>(ctx, b, *tab, lv, wreq, cptr, conn, true);
  qg_status st = qg_check_launch(ctx, "connection lists");
  if (st == QG_OK) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "connection lists");
  }
  if (st == QG_OK) st = qg_check_device_error(ctx, "connection lists");
  if (st != QG_OK) {
    cudaFree(cptr);
    cudaFree(conn);
    cudaFree(coef);
    return st;
  }
  c.d_cptr = cptr;
  c.d_conn = conn;
  c.d_coef = coef;
  c.nconn = total;
  c.conn_state = 1;
  return QG_OK;
}

static qg_status ensure_conn(qg_context ctx, qg_operator op, qg_basis b, OpBasisCache *c) {
  if (!ctx->conn_lists || c->conn_state != 0) return QG_OK;
  return build_conn(ctx, op, b, *c);
}

bool qg_apply_uses_lists(qg_operator op, qg_basis b) {
  qg_context ctx = b->ctx;
  if (!ctx->conn_lists || op->nf != b->nf || b->n <= 0) return false;
  qg_status st = QG_OK;
  OpBasisCache *c = qg_basis_cache(b, op, &st);
  if (st != QG_OK || !c) return false;
  if (ensure_conn(ctx, op, b, c) != QG_OK) return false;
  return c->conn_state == 1;
}

template <int W, int NV, bool FUSE>
static void launch_apply_list_t(qg_context ctx, const OpBasisCache *c, const double2 *diag, qg_basis dst,
                                const double2 *x, int xs, double2 *y, int ys, int vec0, int npass,
                                const ApplyFuse &fz, const LocalView &lv, bool real) {
  dim3 grid((unsigned)qg_apply_grid(dst), (unsigned)npass);
  const Key<W> *keys = (const Key<W> *)dst->d_keys;
  if (NV == 1 && !FUSE && ctx->y_host) {  // one vector into host memory: rows stored in order
    if (real)
      k_apply_list<W, 1, false, true, true><<<grid, 256, 0, ctx->stream>>>(keys, dst->n, c->d_cptr, c->d_conn,
                                                                        c->d_coef, diag, x, xs, y, ys, vec0, fz, lv);
    else
      k_apply_list<W, 1, false, false, true><<<grid, 256, 0, ctx->stream>>>(keys, dst->n, c->d_cptr, c->d_conn,
                                                                         c->d_coef, diag, x, xs, y, ys, vec0, fz, lv);
  } else if (NV == 1 && FUSE && fz.real_vector) {  // real operators only (the caller checks)
    k_apply_list<W, 1, true, true, false, false, true><<<grid, 256, 0, ctx->stream>>>(
        keys, dst->n, c->d_cptr, c->d_conn, c->d_coef, diag, x, xs, y, ys, vec0, fz, lv);
  } else if (FUSE && fz.split) {  // real operators only (the caller checks)
    k_apply_list<W, NV, true, true, false, true><<<grid, 256, 0, ctx->stream>>>(
        keys, dst->n, c->d_cptr, c->d_conn, c->d_coef, diag, x, xs, y, ys, vec0, fz, lv);
  } else if (real) {
    k_apply_list<W, NV, FUSE, true><<<grid, 256, 0, ctx->stream>>>(keys, dst->n, c->d_cptr, c->d_conn, c->d_coef,
                                                                   diag, x, xs, y, ys, vec0, fz, lv);
  } else {
    k_apply_list<W, NV, FUSE, false><<<grid, 256, 0, ctx->stream>>>(keys, dst->n, c->d_cptr, c->d_conn, c->d_coef,
                                                                    diag, x, xs, y, ys, vec0, fz, lv);
  }
  ctx->launches++;
}

// Passes of 8, 4, 3, 2 or 1 vectors (at most `chunk` per pass); all passes of one width run as
// one launch with a pass per blockIdx.y, so a small basis still spreads its vectors over the
// SMs.  Three vectors (the x, y, z polarisations) get a width of their own: as 2 + 1 passes
// each pass would gather 32 or 16 of every 48 bytes of a row.
template <int W, bool FUSE>
static void launch_apply_list(qg_context ctx, const OpBasisCache *c, const double2 *diag, qg_basis dst,
                              const double2 *x, int xs, double2 *y, int ys, int nvec, const ApplyFuse &fz,
                              const LocalView &lv, int chunk, bool real) {
  if (chunk <= 0) chunk = 8;
  int v = 0;
  while (v < nvec) {
    int left = std::min(nvec - v, chunk);
    int per = left >= 8 ? 8 : left >= 4 ? 4 : left == 3 ? 3 : left >= 2 ? 2 : 1;
    int np = std::min((nvec - v) / per, 65535);
    if (per == 8)
      launch_apply_list_t<W, 8, FUSE>(ctx, c, diag, dst, x, xs, y, ys, v, np, fz, lv, real);
    else if (per == 4)
      launch_apply_list_t<W, 4, FUSE>(ctx, c, diag, dst, x, xs, y, ys, v, np, fz, lv, real);
    else if (per == 3)
      launch_apply_list_t<W, 3, FUSE>(ctx, c, diag, dst, x, xs, y, ys, v, np, fz, lv, real);
    else if (per == 2)
      launch_apply_list_t<W, 2, FUSE>(ctx, c, diag, dst, x, xs, y, ys, v, np, fz, lv, real);
    else
      launch_apply_list_t<W, 1, FUSE>(ctx, c, diag, dst, x, xs, y, ys, v, np, fz, lv, real);
    v += per * np;
  }
}

// ------------------------------------------------------------------ small bases as explicit rows

static bool op_values_real(qg_operator op);

// The rows of the same-basis list apply (k_apply_list) as CSR: per row the diagonal, every local
// move (certain offset or listed source) and every listed connection, in that kernel's order,
// each with its source row and the value and form (kind) it multiplies with.  Count pass
// (FILL false: cnt[r]) and fill pass (FILL true, rowptr given).
template <int W, bool FILL, bool REAL>
__global__ void k_small_csr(const Key<W> *__restrict__ rows, int64_t n, const int64_t *__restrict__ cptr,
                            const uint2 *__restrict__ conn, const double2 *__restrict__ coef,
                            const double2 *__restrict__ diag, LocalView lv, int *__restrict__ cnt,
                            const int *__restrict__ rowptr, int *__restrict__ col, double2 *__restrict__ val,
                            unsigned char *__restrict__ kind) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int c = 0;
  int64_t o = FILL ? rowptr[r] : 0;
  auto emit = [&](int64_t j, double2 v, unsigned char kd) {
    if (FILL) {
      col[o] = (int)j;
      val[o] = v;
      kind[o] = kd;
      o++;
    }
    c++;
  };
  if (diag) {
    const double2 dg = diag[r];
    emit(r, dg, (!REAL && qg_is_nonzero(dg.y)) ? 1 : 0);
  }
  int64_t p = cptr[r];
  const int64_t pe = cptr[r + 1];
  if (lv.on) {
    const Key<W> d = rows[r];
    const int b = lv.cfg[get_local<W>(d, lv.lo, lv.lmask)];
    const int64_t off = r - (int64_t)lv.bstart[b];
    const uint32_t e1 = lv.eoff[b + 1];
    for (uint32_t e = lv.eoff[b]; e < e1; e++) {
      const LocalEntry *E = lv.ent + e;
      int64_t j;
      if (E->tend >> 31) {
        j = (int64_t)E->tstart + off;
      } else {
        const uint32_t js = p < pe ? conn[p].x : QG_NO_INDEX;
        p++;
        if (js == QG_NO_INDEX) continue;
        j = js;
      }
      if (REAL)
        emit(j, make_double2(E->vre, 0.0), 2);
      else
        emit(j, make_double2(E->vre, E->vim), qg_is_nonzero(E->vim) ? 3 : 2);
    }
  }
  for (; p < pe; p++) {
    const uint2 cn = conn[p];
    const int par = (int)(cn.y >> 31);
    const double2 cf = coef[cn.y & 0x7FFFFFFFu];
    if (REAL)
      emit(cn.x, make_double2(qg_flip_sign(cf.x, par), 0.0), 2);
    else
      emit(cn.x, make_double2(qg_flip_sign(cf.x, par), qg_flip_sign(cf.y, par)), qg_is_nonzero(cf.y) ? 3 : 2);
  }
  if (!FILL) cnt[r] = c;
}

template <int W, bool FILL>
static void launch_small_csr(qg_context ctx, qg_basis b, const OpBasisCache *c, const LocalView &lv, bool real,
                             int *cnt, const int *rowptr, int *col, double2 *val, unsigned char *kind) {
  const Key<W> *keys = (const Key<W> *)b->d_keys;
  const unsigned g = (unsigned)((b->n + 255) / 256);
  if (real)
    k_small_csr<W, FILL, true><<<g, 256, 0, ctx->stream>>>(keys, b->n, c->d_cptr, c->d_conn, c->d_coef,
                                                            (const double2 *)c->d_diag, lv, cnt, rowptr, col,
                                                            val, kind);
  else
    k_small_csr<W, FILL, false><<<g, 256, 0, ctx->stream>>>(keys, b->n, c->d_cptr, c->d_conn, c->d_coef,
                                                             (const double2 *)c->d_diag, lv, cnt, rowptr, col,
                                                             val, kind);
  ctx->launches++;
}

void qg_small_csr_free(SmallCsr &c) {
  cudaFree(c.rowptr);
  cudaFree(c.col);
  cudaFree(c.val);
  cudaFree(c.kind);
  c = SmallCsr();
}

qg_status qg_small_csr(qg_context ctx, qg_operator op, qg_basis b, int64_t max_nnz, SmallCsr *out) {
  *out = SmallCsr();
  if (!qg_apply_uses_lists(op, b) || b->n > (1 << 30)) return QG_OK;
  qg_status st = QG_OK;
  OpBasisCache *c = qg_basis_cache(b, op, &st);
  if (st != QG_OK) return st;
  const HostTable *tab;
  LocalView lv;
  const uint64_t *wreq;
  same_basis_view(op, b, c, &tab, &lv, &wreq);
  const bool real = op_values_real(op);
  const int n = (int)b->n;
  SmallCsr s;
  s.n = n;
  int *cnt = nullptr;
  cudaError_t e = cudaMalloc(&cnt, (size_t)n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s.rowptr, (size_t)(n + 1) * sizeof(int));
  if (e == cudaSuccess) {
    if (b->W == 1)
      launch_small_csr<1, false>(ctx, b, c, lv, real, cnt, nullptr, nullptr, nullptr, nullptr);
    else
      launch_small_csr<2, false>(ctx, b, c, lv, real, cnt, nullptr, nullptr, nullptr, nullptr);
    e = cudaGetLastError();
  }
  std::vector<int> hc(n), hp(n + 1, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), cnt, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(cnt);
  if (e != cudaSuccess) {
    qg_small_csr_free(s);
    return qg_cuda_fail(ctx, e, "small-basis rows");
  }
  int64_t tot = 0;
  for (int r = 0; r < n; r++) {
    hp[r] = (int)tot;
    tot += hc[r];
  }
  hp[n] = (int)std::min<int64_t>(tot, INT32_MAX);
  s.nnz = tot;
  if (tot > max_nnz) {  // too many terms for one block per chain: the caller takes the general path
    cudaFree(s.rowptr);
    out->n = n;
    out->nnz = tot;
    return QG_OK;
  }
  e = cudaMemcpyAsync(s.rowptr, hp.data(), (size_t)(n + 1) * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMalloc(&s.col, (size_t)std::max<int64_t>(tot, 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&s.val, (size_t)std::max<int64_t>(tot, 1) * sizeof(double2));
  if (e == cudaSuccess) e = cudaMalloc(&s.kind, (size_t)std::max<int64_t>(tot, 1));
  if (e == cudaSuccess) {
    if (b->W == 1)
      launch_small_csr<1, true>(ctx, b, c, lv, real, nullptr, s.rowptr, s.col, s.val, s.kind);
    else
      launch_small_csr<2, true>(ctx, b, c, lv, real, nullptr, s.rowptr, s.col, s.val, s.kind);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    qg_small_csr_free(s);
    return qg_cuda_fail(ctx, e, "small-basis rows");
  }
  *out = s;
  return QG_OK;
}

// ------------------------------------------------------------------ entry points

// Every value of the operator is real (its current values, after any rescale of a sum
// operator): then the diagonal, the merged local entries and the listed coefficients are real.
static bool op_values_real(qg_operator op) {
  for (const HostTerm &h : op->fwd_host)
    if (h.im != 0.0) return false;
  return true;
}

bool qg_operator_values_real(qg_operator op) { return op_values_real(op); }

static int tuned_chunk(const OpBasisCache *c, int nvec) {
  if (c)
    for (auto &p : c->chunk)
      if (p.first == nvec) return p.second;
  return 0;
}

static qg_status apply_chunked(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                               double *y, int ys, int nvec, const ApplyFuse *fz, bool x_packed, int chunk);

// The autotuner: the first multi-vector apply of an operator on a basis (outside stream
// capture) times one plain apply per candidate number of vectors per pass (8, 4, 3, 2, 1) and
// keeps the fastest for that vector count.  The candidates compute bitwise the same result
// (each vector's sum runs in the same order), so the choice changes only the speed.
static qg_status autotune(qg_context ctx, qg_operator op, qg_basis b, OpBasisCache *c, const double *x, int xs,
                          double *y, int ys, int nvec) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return QG_OK;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    cudaGetLastError();
    return QG_OK;  // untuned: the default chunk stays
  }
  int best = 8;
  float best_ms = 0;
  // thread per row with 8, 4, 3, 2 or 1 vectors per pass; warp per row with 32 or 64
  const int cand[7] = {8, 4, 3, 2, 1, -32, -64};
  qg_status st = QG_OK;
  for (int i = 0; i < 7 && st == QG_OK; i++) {
    int ch = cand[i];
    if (ch > nvec && ch != 8) continue;
    if (ch < 0 && (nvec < 16 || (ch == -64 && nvec <= 32))) continue;
    if (i == 0) st = apply_chunked(ctx, op, b, b, x, xs, y, ys, nvec, nullptr, false, ch);  // warm
    cudaEventRecord(e0, ctx->stream);
    if (st == QG_OK) st = apply_chunked(ctx, op, b, b, x, xs, y, ys, nvec, nullptr, false, ch);
    cudaEventRecord(e1, ctx->stream);
    float ms = 0;
    if (st == QG_OK && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
      if (i == 0 || ms < best_ms) {
        best = ch;
        best_ms = ms;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
  if (st == QG_OK) c->chunk.push_back({nvec, best});
  return st;
}

qg_status qg_apply_strided(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                           double *y, int ys, int nvec, const ApplyFuse *fz, bool x_packed) {
  int chunk = 8;
  if (dst == src && nvec >= 2) {
    qg_status st = QG_OK;
    OpBasisCache *c = qg_basis_cache(dst, op, &st);
    if (st != QG_OK) return st;
    chunk = tuned_chunk(c, nvec);
    if (!chunk && ctx->autotune) {
      QG_TRY(autotune(ctx, op, dst, c, x, xs, y, ys, nvec));
      chunk = tuned_chunk(c, nvec);
    }
    if (!chunk) chunk = 8;
  }
  return apply_chunked(ctx, op, dst, src, x, xs, y, ys, nvec, fz, x_packed, chunk);
}

static qg_status apply_chunked(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                               double *y, int ys, int nvec, const ApplyFuse *fz, bool x_packed, int chunk) {
  ApplyFuse none;
  const double2 *x2 = (const double2 *)x;
  double2 *y2 = (double2 *)y;
  qg_status st = QG_OK;
  const double2 *diag = nullptr;
  const HostTable *tab = &op->pull;
  const uint64_t *wreq = nullptr;
  LocalView lv{};
  lv.on = 0;
  if (dst == src) {
    OpBasisCache *c = qg_basis_cache(dst, op, &st);
    if (st != QG_OK) return st;
    diag = (const double2 *)c->d_diag;
    if (op->H > 0) {
      tab = &op->pull_nl;
      lv.on = 1;
      lv.lo = dst->nf - op->H;
      lv.lmask = (1u << op->H) - 1;
      lv.cfg = c->d_cfg;
      lv.bstart = c->d_bstart;
      lv.eoff = c->d_eoff;
      lv.ent = c->d_ent;
      lv.etarget = c->d_ent_target;
    } else {
      tab = &op->pull_off;
    }
    if (c->wreq_exact && c->d_wreq && tab == &op->pull_nl) wreq = c->d_wreq;
    if (chunk > 0) {  // thread per row: gather through the connection lists when built
      QG_TRY(ensure_conn(ctx, op, dst, c));
      if (c->conn_state == 1) {
        const ApplyFuse &f = fz ? *fz : none;
        const bool real = op_values_real(op);
        if (op->W == 1) {
          if (fz)
            launch_apply_list<1, true>(ctx, c, diag, dst, x2, xs, y2, ys, nvec, f, lv, chunk, real);
          else
            launch_apply_list<1, false>(ctx, c, diag, dst, x2, xs, y2, ys, nvec, f, lv, chunk, real);
        } else {
          if (fz)
            launch_apply_list<2, true>(ctx, c, diag, dst, x2, xs, y2, ys, nvec, f, lv, chunk, real);
          else
            launch_apply_list<2, false>(ctx, c, diag, dst, x2, xs, y2, ys, nvec, f, lv, chunk, real);
        }
        return qg_check_launch(ctx, "qg_apply");
      }
    }
  }
  int packed = 0;
  if (nvec == 1) {
    if (!x_packed) QG_TRY(qg_pack(ctx, src, x, xs, nullptr, nullptr, nullptr));
    packed = 1;
  }
  const ApplyFuse &f = fz ? *fz : none;
  if (op->W == 1) {
    if (fz)
      launch_apply_s<1, true>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f, lv, wreq, chunk);
    else
      launch_apply_s<1, false>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f, lv, wreq, chunk);
  } else {
    if (fz)
      launch_apply_s<2, true>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f, lv, wreq, chunk);
    else
      launch_apply_s<2, false>(ctx, *tab, diag, dst, src, packed, x2, xs, y2, ys, nvec, f, lv, wreq, chunk);
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

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister memory is
// mapped into the device's address space), or nullptr for pageable memory.
static void *mapped_host(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Streams a page-locked host buffer into device memory with the SMs (16-byte loads, grid
// stride).  On GB300 this, the copy engine, and both together all run at the host link's
// ~211 GB/s (measured), so the simplest form is kept.
__global__ void k_pull_host(const double2 *__restrict__ src, double2 *__restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

extern "C" qg_status qg_apply_host(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x_host,
                                   double *y_host, int32_t nvec) {
  if (!ctx || !op || !dst || !src || nvec <= 0 || !x_host || !y_host || op->nf != dst->nf || op->nf != src->nf)
    return QG_ERR_ARG;
  size_t xb = (size_t)src->n * nvec * 16, yb = (size_t)dst->n * nvec * 16;
  if (!dst->n) return QG_OK;
  if (!src->n) {
    QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    memset(y_host, 0, yb);
    return QG_OK;
  }
  // page-locked buffers: x is pulled by the SMs, y is written by the apply kernel straight
  // into host memory (the copy back overlaps the gather); pageable ones go through staging
  const double2 *xmap = (const double2 *)mapped_host(x_host);
  double *ymap = (double *)mapped_host(y_host);
  size_t need = xb + (ymap ? 0 : yb);
  if (ctx->io_bytes < need) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_io);
    ctx->d_io = nullptr;
    ctx->io_bytes = 0;
    QG_CUDA(ctx, cudaMalloc(&ctx->d_io, need));
    ctx->io_bytes = need;
  }
  double *dx = ctx->d_io, *dy = ymap ? ymap : ctx->d_io + xb / 8;
  if (xmap) {
    int64_t n2 = (int64_t)(xb / 16);
    unsigned g = (unsigned)std::min<int64_t>((n2 + 255) / 256, (int64_t)ctx->num_sms * 8);
    k_pull_host<<<g, 256, 0, ctx->stream>>>(xmap, (double2 *)dx, n2);
    ctx->launches++;
    QG_TRY(qg_check_launch(ctx, "qg_apply_host pull"));
  } else {
    QG_CUDA(ctx, cudaMemcpyAsync(dx, x_host, xb, cudaMemcpyHostToDevice, ctx->stream));
  }
  ctx->y_host = ymap != nullptr;
  qg_status st = qg_apply(ctx, op, dst, src, dx, dy, nvec);
  ctx->y_host = false;
  if (st != QG_OK) return st;
  if (!ymap) QG_CUDA(ctx, cudaMemcpyAsync(y_host, dy, yb, cudaMemcpyDeviceToHost, ctx->stream));
  QG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return qg_check_device_error(ctx, "qg_apply_host");
}

// ------------------------------------------------------------------ nnz count

// Connections into rows row0, row0 + stride, ... (cnt of them): per row the (row, term) pairs
// with a non-zero sign whose source lies in the basis.
template <int W>
__global__ void k_count(const Key<W> *__restrict__ rows, int64_t row0, int64_t stride, int64_t cnt,
                        const GroupDev<W> *__restrict__ groups, int ngroups, const TermDev<W> *__restrict__ terms,
                        const Slot *__restrict__ slots, uint64_t hmask, int offdiag_only, unsigned long long *out,
                        unsigned int *err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (i < cnt) {
    Key<W> d = rows[row0 + i * stride];
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

static qg_status count_nnz(qg_context ctx, qg_operator op, qg_basis b, int offdiag, int64_t row0, int64_t stride,
                           int64_t *nnz) {
  *nnz = 0;
  if (row0 >= b->n) return QG_OK;
  const int64_t cnt = (b->n - row0 + stride - 1) / stride;
  unsigned long long *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, 8));
  cudaError_t e = cudaMemsetAsync(d, 0, 8, ctx->stream);
  if (e == cudaSuccess) {
    if (op->W == 1)
      k_count<1><<<grid_for(cnt, 256), 256, 0, ctx->stream>>>(
          (const Key<1> *)b->d_keys, row0, stride, cnt, (const GroupDev<1> *)op->pull.d_groups, op->pull.ngroups,
          (const TermDev<1> *)op->pull.d_terms, b->d_slots, b->hcap - 1, offdiag, d, ctx->d_err);
    else
      k_count<2><<<grid_for(cnt, 256), 256, 0, ctx->stream>>>(
          (const Key<2> *)b->d_keys, row0, stride, cnt, (const GroupDev<2> *)op->pull.d_groups, op->pull.ngroups,
          (const TermDev<2> *)op->pull.d_terms, b->d_slots, b->hcap - 1, offdiag, d, ctx->d_err);
    ctx->launches++;
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_count_nnz");
  *nnz = (int64_t)h;
  return qg_check_device_error(ctx, "qg_count_nnz");
}

extern "C" qg_status qg_count_nnz(qg_context ctx, qg_operator op, qg_basis b, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf) return QG_ERR_ARG;
  return count_nnz(ctx, op, b, 0, 0, 1, nnz);
}

extern "C" qg_status qg_count_nnz_rows(qg_context ctx, qg_operator op, qg_basis b, int64_t row0, int64_t stride,
                                       int32_t offdiag, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf || row0 < 0 || stride < 1) return QG_ERR_ARG;
  return count_nnz(ctx, op, b, offdiag != 0, row0, stride, nnz);
}

extern "C" qg_status qg_set_autotune(qg_context ctx, int32_t on) {
  if (!ctx) return QG_ERR_ARG;
  ctx->autotune = on != 0;
  return QG_OK;
}

extern "C" qg_status qg_apply_set_chunk(qg_context ctx, qg_operator op, qg_basis b, int32_t nvec, int32_t chunk) {
  if (!ctx || !op || !b || nvec <= 0) return QG_ERR_ARG;
  if (!(chunk == 1 || chunk == 2 || chunk == 3 || chunk == 4 || chunk == 8 || chunk == -32 || chunk == -64))
    return QG_ERR_ARG;
  qg_status st = QG_OK;
  OpBasisCache *c = qg_basis_cache(b, op, &st);
  if (st != QG_OK) return st;
  for (auto &p : c->chunk)
    if (p.first == nvec) {
      p.second = chunk;
      return QG_OK;
    }
  c->chunk.push_back({nvec, chunk});
  return QG_OK;
}

extern "C" qg_status qg_set_connection_lists(qg_context ctx, int32_t on) {
  if (!ctx) return QG_ERR_ARG;
  ctx->conn_lists = on != 0;
  return QG_OK;
}

extern "C" qg_status qg_apply_list_info(qg_context ctx, qg_operator op, qg_basis b, int32_t *built, int64_t *nconn) {
  if (!ctx || !op || !b || !built || !nconn || op->nf != b->nf) return QG_ERR_ARG;
  *built = 0;
  *nconn = 0;
  for (auto &c : b->caches)
    if (c.op_uid == op->uid && c.conn_state == 1) {
      *built = 1;
      *nconn = c.nconn;
    }
  return QG_OK;
}

extern "C" qg_status qg_apply_fp64_ops(qg_context ctx, qg_operator op, qg_basis b, int64_t *ops) {
  if (!ctx || !op || !b || !ops || op->nf != b->nf) return QG_ERR_ARG;
  *ops = 0;
  if (!b->n) return QG_OK;
  if (!qg_apply_uses_lists(op, b)) {
    ctx->last_error = "qg_apply_fp64_ops: no connection lists for this operator and basis";
    return QG_ERR_ARG;
  }
  qg_status st = QG_OK;
  OpBasisCache *c = qg_basis_cache(b, op, &st);
  if (st != QG_OK) return st;
  const HostTable *tab;
  LocalView lv;
  const uint64_t *wreq;
  same_basis_view(op, b, c, &tab, &lv, &wreq);
  unsigned long long *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, 8));
  cudaError_t e = cudaMemsetAsync(d, 0, 8, ctx->stream);
  if (e == cudaSuccess) {
    if (b->W == 1)
      k_count_fp64<1><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<1> *)b->d_keys, b->n, c->d_cptr,
                                                                      c->d_conn, c->d_coef,
                                                                      (const double2 *)c->d_diag, lv, d);
    else
      k_count_fp64<2><<<grid_for(b->n, 256), 256, 0, ctx->stream>>>((const Key<2> *)b->d_keys, b->n, c->d_cptr,
                                                                      c->d_conn, c->d_coef,
                                                                      (const double2 *)c->d_diag, lv, d);
    ctx->launches++;
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_apply_fp64_ops");
  *ops = (int64_t)h;
  return QG_OK;
}

extern "C" qg_status qg_apply_chunk(qg_context ctx, qg_operator op, qg_basis b, int32_t nvec, int32_t *chunk) {
  if (!ctx || !op || !b || !chunk || nvec <= 0) return QG_ERR_ARG;
  *chunk = 0;
  for (auto &c : b->caches)
    if (c.op_uid == op->uid) *chunk = tuned_chunk(&c, nvec);
  return QG_OK;
}

extern "C" qg_status qg_count_nnz_offdiag(qg_context ctx, qg_operator op, qg_basis b, int64_t *nnz) {
  if (!ctx || !op || !b || !nnz || op->nf != b->nf) return QG_ERR_ARG;
  return count_nnz(ctx, op, b, 1, 0, 1, nnz);
}
