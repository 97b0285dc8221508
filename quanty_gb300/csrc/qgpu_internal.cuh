// Internal definitions shared by the qgpu translation units.
//
// Device determinant layout: a Key<W> of W 64-bit words; reference orbital i lives at device
// bit p = nf-1-i (word p>>6, bit p&63).  With this reversal the numeric order of keys (word
// W-1 most significant) is the lexicographic order of the reference's determinant strings,
// orbital 0 first, so the low-index "impurity" orbitals of a Quanty model are the most
// significant bits and rows of one impurity configuration are contiguous in a sorted basis.
//
// An operator term is pre-digested on the host into masks (see qgpu_operator.cu):
//   applicable on det d  <=>  (d & need1) == need1  and  (d & need0) == 0
//   target               =    d ^ flip
//   sign                 =    (-1)^(popcount(d & sgn) + const)   (const folded into the value)
// which is exact for any ladder string: the fermion sign of each ladder step is the parity
// of the occupied orbitals below it in the intermediate determinant, and that intermediate
// differs from d only by bits the string has already toggled, a term-constant.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/qgpu.h"

#define QG_MAXW 2
#define QG_EMPTY_WORD 0xFFFFFFFFFFFFFFFFull
#define QG_NO_INDEX 0xFFFFFFFFu
#define QG_PROBE_LIMIT (1 << 20)

// Error bits a kernel may raise in the context's device error word.
#define QG_DEVERR_PROBE 1u      // a hash probe exceeded QG_PROBE_LIMIT
#define QG_DEVERR_TABLE_FULL 2u // an insert found the table over its load limit
#define QG_DEVERR_OVERFLOW 4u   // an output list overflowed its capacity
#define QG_DEVERR_TIMEOUT 8u    // a bounded wait on an asynchronous copy gave up

template <int W>
struct __align__(8 * W) Key {
  uint64_t w[W];
};

// Per-term masks for W words and the signed value, padded to a multiple of 16 bytes so a
// table can be moved with one bulk copy.
template <int W>
struct __align__(16) TermDev {
  uint64_t need0[W];
  uint64_t flip[W];
  uint64_t sgn[W];
  uint64_t pad[W == 1 ? 1 : 0];
  double vre, vim;
};
template <>
struct __align__(16) TermDev<2> {
  uint64_t need0[2];
  uint64_t flip[2];
  uint64_t sgn[2];
  double vre, vim;
};

// Terms sharing one need1 mask; terms[begin, end).  48 bytes.
// A hop group holds one-body moves only: need1 is one orbital p, every term empties p and
// fills one orbital q (need0 = {q}, flip = {p, q}), the terms in ascending order of q; qmask
// is the set of those q.  Such a group's applicable terms are the set bits of qmask & ~row,
// so no term is tested.
template <int W>
struct __align__(16) GroupDev {
  uint64_t need1[2];  // words >= W are zero
  int32_t begin, end;
  int32_t diag;  // all terms of the group have flip == 0
  int32_t hop;   // a hop group (see above)
  uint64_t qmask[2];
};

// Hash slot, one 32-byte DRAM sector: the key and the current source amplitude (written by
// the pack step that precedes an H*psi), so a connection costs one sector.  The row a slot
// belongs to is kept in a separate array.  For W = 1 the second key word is zero.
struct __align__(32) Slot {
  uint64_t k[2];
  double vre, vim;
};

struct qg_context_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;
  int64_t launches = 0;
  unsigned int *d_err = nullptr;      // device error word
  double *d_scratch = nullptr;        // reduction scratch
  size_t scratch_bytes = 0;
  double *h_pinned = nullptr;         // pinned host staging for small results
  size_t pinned_bytes = 0;
  int num_sms = 148;
  double *d_io = nullptr;             // staging for host-buffer entry points
  size_t io_bytes = 0;
  bool use_graphs = true;             // capture Lanczos step sequences into CUDA graphs
  bool y_host = false;                // the apply being launched writes y into host memory
  bool autotune = true;               // time the vectors-per-pass choices of multi-vector applies
  bool conn_lists = true;             // resolve hashed connections once per (operator, basis)
  bool small_lanczos = true;          // persistent one-block-per-chain Lanczos on small bases
  bool split_chains = true;           // real Lanczos chains of a real operator two per vector
};

// A term table in one device allocation: ngroups GroupDev followed by nterms TermDev.
// Hop groups come first, in ascending order of their orbital p (word 0 bits, then word 1);
// hopmask holds those orbitals, so the hop group of an occupied p is found by a popcount.
struct HostTable {
  void *d_blob = nullptr;
  void *d_groups = nullptr;  // = d_blob
  void *d_terms = nullptr;   // = d_blob + ngroups * sizeof(GroupDev)
  size_t bytes = 0;          // multiple of 16
  int ngroups = 0, nterms = 0;
  int nhop = 0;              // leading hop groups
  uint64_t hopmask[2] = {0, 0};
  size_t tgrp_off = 0;       // byte offset of the uint32 group index of each term (after the terms)
  // host copy of the blob and, per term slot, the forward term it came from and the sign
  // its value carries (adjoint tables): what a rescale of a sum operator patches
  std::vector<unsigned char> h_blob;
  std::vector<std::pair<int, int>> slot_src;
};

// A digested term on the host (canonical masks in device bit positions, signed value).
struct HostTerm {
  uint64_t n1[2], n0[2], fl[2], sg[2];
  double re, im;
  int src = -1, sgn = 1;  // forward term it came from, sign its value carries
};

struct qg_operator_s {
  qg_context ctx = nullptr;
  int nf = 0, W = 1;
  int nterms_in = 0, nterms = 0;
  int hermitian = 0;
  HostTable pull;      // adjoint action grouped by need1: rows gather their sources
  HostTable pull_off;  // the same without diagonal terms (diagonal precomputed per basis)
  HostTable diag;      // diagonal terms only (flip == 0)
  HostTable push;      // forward action grouped by need1: sources emit their targets
  int max_len = 0;
  uint64_t uid = 0;    // unique per operator, keys the per-basis caches
  // local decomposition: the H leading orbitals (device bits nf-H .. nf-1) hold every
  // many-body term; off-diagonal terms confined to them are precomputed per local
  // configuration of a basis; the rest (pull_nl, host copy nl_host in table order) is scanned
  int H = 0;
  std::vector<HostTerm> local_off;
  HostTable pull_nl;
  std::vector<HostTerm> nl_host;
  // forward terms in creation order (masks and values)
  std::vector<HostTerm> fwd_host;
  // sum operators (parameter scans, qg_operator_create_sum): the union of the components'
  // terms, zero values kept, so the structure never depends on the coefficients; comp holds
  // each term's contribution per component ([ncomp][fwd] complex); a rescale rewrites the
  // values and bumps `version`, and per-basis caches refresh their values when they see it
  int ncomp = 0;
  bool keep_zero = false;
  std::vector<double> comp_re, comp_im;
  uint64_t version = 0;
};

// Per-(operator, basis) precomputed data for the same-basis H*psi.
struct LocalEntry {
  uint32_t tstart;   // first row of the target local configuration's block
  uint32_t tend;     // one past its last row; bit 31: both blocks list the same non-local
                     // configurations, so the target row is at the same offset
  uint64_t wreq;     // window bits the target needs (see qgpu_apply.cu)
  double vre, vim;   // merged, signed coefficient
};

struct OpBasisCache {
  uint64_t op_uid = 0;
  uint64_t op_version = 0;        // the operator's value version the cached values belong to
  // host copies for a value refresh (sum operators): configuration of each block, entries
  std::vector<uint32_t> h_bcfg, h_eoff, h_etarget;
  std::vector<LocalEntry> h_ent;
  double *d_diag = nullptr;       // complex per row: all diagonal terms
  uint64_t *d_wreq = nullptr;     // per term of op->pull_nl: window bits its source needs
  bool wreq_exact = false;        // every term's window change fits the bit encoding
  // local blocks (op->H > 0): rows sharing a local configuration are contiguous
  int nblocks = 0;
  uint32_t *d_bstart = nullptr;   // [nblocks + 1]
  int32_t *d_cfg = nullptr;       // [2^H] local configuration -> block, -1 if absent
  uint32_t *d_eoff = nullptr;     // [nblocks + 1]
  LocalEntry *d_ent = nullptr;
  uint32_t *d_ent_target = nullptr;  // target local configuration of each entry
  int64_t nent = 0;
  // connection lists: per row, in the order the thread-per-row apply visits them, the
  // connections it would otherwise resolve through the hash table (local moves without a
  // certain offset, hit or miss; hits of the scanned table), each as (source row, meta):
  // meta = term index in the scanned table | parity sign << 31, QG_NO_INDEX rows mark a
  // local move whose source is absent.  Built once per (operator, basis); every later H*psi
  // gathers x[source] by row, so neighbouring rows read neighbouring sources.
  int conn_state = 0;             // 0 not tried, 1 built, -1 not built (size, memory, capture)
  int64_t nconn = 0;
  int64_t *d_cptr = nullptr;      // [n + 1] list offsets
  uint2 *d_conn = nullptr;        // [nconn]
  double2 *d_coef = nullptr;      // [terms of the scanned table] (vre, vim)
  // autotuned vectors per pass of the apply kernel, per number of vectors (pairs nvec, chunk)
  std::vector<std::pair<int, int>> chunk;
};

struct qg_basis_s {
  qg_context ctx = nullptr;
  int nf = 0, W = 1;
  int64_t n = 0;
  void *d_keys = nullptr;         // Key<W>[n], sorted ascending
  Slot *d_slots = nullptr;        // [hcap]
  uint32_t *d_slot_row = nullptr; // [hcap] row of the slot's key
  uint32_t *d_row_slot = nullptr; // [n] slot of the row's key
  int64_t hcap = 0;               // power of two, >= 2n
  // occupation windows every determinant of the basis satisfies (the closure's
  // restrictions): a source outside them cannot be in the basis, so no lookup is made
  int nres = 0;
  uint64_t *d_rmask = nullptr;    // [nres][W]
  int32_t *d_rmin = nullptr, *d_rmax = nullptr;
  std::vector<uint64_t> h_rmask;
  std::vector<int32_t> h_rmin, h_rmax;
  std::vector<OpBasisCache> caches;
};

// ------------------------------------------------------------------ device helpers

__host__ __device__ inline uint64_t qg_mix64(uint64_t h) {
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

template <int W>
__host__ __device__ inline uint64_t qg_hash(const Key<W> &k) {
  uint64_t h = 0x9e3779b97f4a7c15ull;
#pragma unroll
  for (int i = 0; i < W; i++) h = qg_mix64(h ^ k.w[i]) + 0x632be59bd9b4e019ull * (i + 1);
  return qg_mix64(h);
}

template <int W>
__host__ __device__ inline bool qg_eq(const Key<W> &a, const Key<W> &b) {
  bool e = true;
#pragma unroll
  for (int i = 0; i < W; i++) e &= (a.w[i] == b.w[i]);
  return e;
}

template <int W>
__host__ __device__ inline bool qg_less(const Key<W> &a, const Key<W> &b) {
#pragma unroll
  for (int i = W - 1; i >= 0; i--) {
    if (a.w[i] != b.w[i]) return a.w[i] < b.w[i];
  }
  return false;
}

// Linear probe for key k starting at slot h; returns the slot index or -1.  Probes are bounded.
// A slot is empty when its second word is all ones: an occupied slot holds 0 there (W = 1) or
// the key's top word, which never has all 64 bits set (at most 63 orbitals live in it since
// nf <= 127).  The low word can be all ones for a resident key (W = 2, orbitals nf-64..nf-1
// all occupied), so it cannot mark an empty slot.
template <int W>
__device__ __forceinline__ int64_t qg_find_slot_at(const Slot *__restrict__ slots, uint64_t hmask, const Key<W> &k,
                                                   uint64_t h, unsigned int *err) {
  for (int p = 0; p < QG_PROBE_LIMIT; p++) {
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(slots + h));
    if (v.x == k.w[0] && (W == 1 || v.y == k.w[W - 1])) return (int64_t)h;
    if (v.y == QG_EMPTY_WORD) return -1;  // the key's top word is never all ones (nf <= 127)
    h = (h + 1) & hmask;
  }
  atomicOr(err, QG_DEVERR_PROBE);
  return -1;
}

template <int W>
__device__ __forceinline__ int64_t qg_find_slot(const Slot *__restrict__ slots, uint64_t hmask, const Key<W> &k,
                                                unsigned int *err) {
  uint64_t h = qg_hash<W>(k) & hmask;
  for (int p = 0; p < QG_PROBE_LIMIT; p++) {
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(slots + h));
    if (v.x == k.w[0] && (W == 1 || v.y == k.w[W - 1])) return (int64_t)h;
    if (v.y == QG_EMPTY_WORD) return -1;  // the key's top word is never all ones (nf <= 127)
    h = (h + 1) & hmask;
  }
  atomicOr(err, QG_DEVERR_PROBE);
  return -1;
}

// Row of a key, or -1.
template <int W>
__device__ __forceinline__ int64_t qg_lookup(const Slot *__restrict__ slots, const uint32_t *__restrict__ slot_row,
                                             uint64_t hmask, const Key<W> &k, unsigned int *err) {
  int64_t h = qg_find_slot<W>(slots, hmask, k, err);
  return h < 0 ? -1 : (int64_t)__ldg(slot_row + h);
}

template <int W>
__device__ __forceinline__ int qg_parity_and(const Key<W> &d, const uint64_t *m) {
  int c = 0;
#pragma unroll
  for (int i = 0; i < W; i++) c += __popcll(d.w[i] & m[i]);
  return c & 1;
}

// ------------------------------------------------------------------ host helpers

#define QG_TRY(expr)                   \
  do {                                 \
    qg_status _s = (expr);             \
    if (_s != QG_OK) return _s;        \
  } while (0)

qg_status qg_cuda_fail(qg_context ctx, cudaError_t e, const char *what);
#define QG_CUDA(ctx, expr)                                     \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return qg_cuda_fail(ctx, _e, #expr); \
  } while (0)

qg_status qg_check_launch(qg_context ctx, const char *what);
qg_status qg_check_device_error(qg_context ctx, const char *what);
qg_status qg_ensure_scratch(qg_context ctx, size_t bytes);
qg_status qg_ensure_pinned(qg_context ctx, size_t bytes);

inline int qg_words_for(int nf) { return nf / 64 + 1; }  // nf <= 63 -> 1, <= 127 -> 2

// basis helpers (qgpu_basis.cu)
qg_status qg_basis_from_device_keys(qg_context ctx, int nf, int W, void *d_keys_unsorted, int64_t n,
                                    qg_basis *out, int64_t *d_perm /* optional, size n */);
qg_status qg_basis_build_hash(qg_basis b);
qg_status qg_basis_set_windows(qg_basis b, int nres, const uint64_t *mask_host, const int32_t *min_host,
                               const int32_t *max_host);
// per-(operator, basis) cache (diagonal, window bits, local blocks); nullptr on failure
OpBasisCache *qg_basis_cache(qg_basis b, qg_operator op, qg_status *st);
void qg_cache_free(OpBasisCache &c);

// Epilogue options for the fused Lanczos step (see qgpu_krylov.cu):
//   prev/beta:  y = H x - beta[k] * prev;
//   dot_part:   per-block partial sums of conj(x_r) * (H x)_r.
struct ApplyFuse {
  const double2 *prev = nullptr;
  const double *beta = nullptr;  // [nvec], or [2 nvec] when split
  double2 *dot_part = nullptr;   // [gridDim.x * nvec]
  // two real Lanczos chains per complex vector (real and imaginary parts, a real operator):
  // each part has its own beta and its own dot partial (.x and .y of dot_part)
  int split = 0;
  // one real chain (a real operator, nvec 1): x, y and prev hold one real number per row
  int real_vector = 0;
};
qg_status qg_apply_launch(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, double *y,
                          int nvec, const ApplyFuse *fz);
// x row stride xs, y row stride ys (complex entries), nvec columns from the given pointers.
// x_packed: for nvec == 1 the caller has already written x into the source basis' slots.
qg_status qg_apply_strided(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                           double *y, int ys, int nvec, const ApplyFuse *fz, bool x_packed = false);
// write x (one column, stride xs) into the slots of basis b; with scale/thr2 (device, one
// value each) the entries are scaled and truncated first and also stored to own_out
qg_status qg_pack(qg_context ctx, qg_basis b, const double *x, int xs, const double *scale, const double *thr2,
                  double *own_out);
int qg_apply_grid(qg_basis dst);
// True when the same-basis apply of op on b gathers through connection lists (builds the
// per-(operator, basis) cache first), so a caller need not pack x into the hash slots.
bool qg_apply_uses_lists(qg_operator op, qg_basis b);
// every current value of the operator is real
bool qg_operator_values_real(qg_operator op);

// Hermitian eigenproblems on the device (qgpu_jacobi.cu): A (k x k row-major, device,
// overwritten) -> eigenvalues ascending (w_dev, k) and the lowest nv eigenvectors as the columns
// of V_dev (k x nv row-major); the host-buffer form copies in and out.
qg_status qg_eigh_device(qg_context ctx, int k, double2 *A, double *w_dev, double2 *V_dev, int nv);
// the same for k > 1 by Householder reduction, bisection and inverse iteration (qgpu_hermitian.cu)
qg_status qg_eigh_tridiag(qg_context ctx, int k, double2 *A, double *w_dev, double2 *V_dev, int nv);
qg_status qg_eigh_host_io(qg_context ctx, int k, const double *a_host, double *w_host, double *v_host, int nv);
int qg_partial_blocks(qg_context ctx, int64_t n);

// dense complex block products (qgpu_blocks.cu); row-major n x k blocks
//   C (ka x kb row-major) = A^H B, with a work buffer of work_elems complex entries for the
//   partial sums;   X = beta X + alpha A M  (M ka x kb row-major)
//   real: every value of A, B (and M) is real: one FMA per term instead of four
qg_status qg_block_gram(qg_context ctx, const double2 *A, int lda, int ka, const double2 *B, int ldb, int kb,
                        int64_t n, double2 *C, double2 *work, int64_t work_elems, bool real = false);
qg_status qg_block_update(qg_context ctx, const double2 *A, int lda, int ka, const double2 *M, double2 *X, int ldx,
                          int kb, int64_t n, double alpha, double beta, bool real = false);
// out (n x np row-major) = sum_i K_i C[i][:], K vector-major (K[i * n + r])
qg_status qg_block_combine(qg_context ctx, const double2 *K, int64_t n, int ntri, const double2 *C, int np,
                           double2 *out);

// reductions (qgpu_krylov.cu)
qg_status qg_dot_dev(qg_context ctx, int64_t n, int nvec, const double *x, const double *y, double *out_dev);

__device__ __forceinline__ double qg_flip_sign(double v, int par) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(par & 1) << 63));
}

__device__ __forceinline__ bool qg_is_nonzero(double v) { return (__double_as_longlong(v) << 1) != 0; }

// acc += (vr + i vi) xv, in the operation order of the complex form
__device__ __forceinline__ void qg_cmac(double2 &acc, double vr, double vi, bool cplx, double2 xv) {
  if (cplx) {
    acc.x = fma(-vi, xv.y, acc.x);
    acc.y = fma(vi, xv.x, acc.y);
  }
  acc.x = fma(vr, xv.x, acc.x);
  acc.y = fma(vr, xv.y, acc.y);
}

// Per-element arithmetic of the Lanczos kernels with every fused multiply-add written out, so
// the general path and the persistent small-basis kernel round alike.
__device__ __forceinline__ double qg_norm2(double2 v) { return fma(v.x, v.x, v.y * v.y); }
// Re(conj(x) y)
__device__ __forceinline__ double qg_redot(double2 x, double2 y) { return fma(x.x, y.x, x.y * y.y); }
// w - a p
__device__ __forceinline__ double2 qg_axpy2(double2 w, double a, double2 p) {
  return make_double2(fma(-a, p.x, w.x), fma(-a, p.y, w.y));
}
// the diagonal term dg * x: real dg (two products) or complex
__device__ __forceinline__ double2 qg_diag_mul(double2 dg, double2 xv, bool cplx) {
  if (cplx) return make_double2(fma(dg.x, xv.x, -(dg.y * xv.y)), fma(dg.x, xv.y, dg.y * xv.x));
  return make_double2(dg.x * xv.x, dg.x * xv.y);
}
// after a Lanczos norm t = |v|^2: b = sqrt(t), scale = 1/b (0 for an empty vector), truncation
// threshold (eps/err)^2 with the err before this step, err *= b^2/(b^2 + 4 gamma^2)
__device__ __forceinline__ void qg_lanczos_norm_scalars(double t, bool first, double eps, double gamma, double &b,
                                                        double &scale, double &thr2, double &err) {
  b = sqrt(t);
  scale = (b > 0.0) ? 1.0 / b : 0.0;
  const double e = first ? 1.0 : err;
  const double th = eps / e;
  thr2 = __dmul_rn(th, th);
  const double b2 = __dmul_rn(b, b), g4 = __dmul_rn(__dmul_rn(4.0, gamma), gamma);
  err = first ? 1.0 : e * (b2 / (b2 + g4));
}

// The same-basis apply of op on b as explicit rows (CSR) for the persistent Lanczos kernel of
// small bases (qgpu_apply.cu): per row, in the list kernel's order, its terms with the source
// row and the value that kernel multiplies by; kind 0 / 1 a real / complex diagonal product,
// 2 / 3 a real / complex multiply-add.  Arrays stay null when the connection lists are not
// built or the rows hold more than max_nnz terms (nnz then says how many).
struct SmallCsr {
  int n = 0;
  int64_t nnz = 0;
  int *rowptr = nullptr;
  int *col = nullptr;
  double2 *val = nullptr;
  unsigned char *kind = nullptr;
};
qg_status qg_small_csr(qg_context ctx, qg_operator op, qg_basis b, int64_t max_nnz, SmallCsr *out);
void qg_small_csr_free(SmallCsr &c);
