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

template <int W>
struct __align__(8 * W) Key {
  uint64_t w[W];
};

// Per-term masks for W words and the signed value.
template <int W>
struct TermDev {
  uint64_t need0[W];
  uint64_t flip[W];
  uint64_t sgn[W];
  double vre, vim;
};

// Terms sharing one need1 mask; terms[begin, end).
template <int W>
struct GroupDev {
  uint64_t need1[W];
  int32_t begin, end;
  int32_t diag;  // all terms of the group have flip == 0
  int32_t pad;
};

// Hash slot: key + basis index.  W=1: 16 bytes, W=2: 32 bytes (one DRAM sector).
template <int W>
struct __align__(16 * W) Slot {
  uint64_t k[W];
  uint32_t idx;
  uint32_t pad[2 * W - 1];
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
};

struct HostTable {
  // device arrays
  void *d_groups = nullptr;
  void *d_terms = nullptr;
  int ngroups = 0, nterms = 0;
};

struct qg_operator_s {
  qg_context ctx = nullptr;
  int nf = 0, W = 1;
  int nterms_in = 0, nterms = 0;
  int hermitian = 0;
  HostTable pull;  // adjoint strings grouped by need1: rows gather their sources
  HostTable push;  // forward strings grouped by need1: sources emit their targets
  int max_len = 0;
};

struct qg_basis_s {
  qg_context ctx = nullptr;
  int nf = 0, W = 1;
  int64_t n = 0;
  void *d_keys = nullptr;   // Key<W>[n], sorted ascending
  void *d_slots = nullptr;  // Slot<W>[hcap]
  int64_t hcap = 0;         // power of two, >= 2n
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

// Look up a key; returns the basis index or -1.  Probes are bounded.
template <int W>
__device__ __forceinline__ int64_t qg_lookup(const Slot<W> *__restrict__ slots, uint64_t hmask,
                                             const Key<W> &k, unsigned int *err) {
  uint64_t h = qg_hash<W>(k) & hmask;
  for (int p = 0; p < QG_PROBE_LIMIT; p++) {
    const Slot<W> *s = slots + h;
    Key<W> sk;
    if (W == 1) {
      ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(s));
      sk.w[0] = v.x;
      if (sk.w[0] == k.w[0]) return (int64_t)(uint32_t)v.y;
      if (sk.w[0] == QG_EMPTY_WORD) return -1;
    } else {
      ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(s));
      if (v.x == k.w[0] && v.y == k.w[1]) {
        uint32_t idx = __ldg(reinterpret_cast<const uint32_t *>(s) + 4);
        return (int64_t)idx;
      }
      if (v.x == QG_EMPTY_WORD && v.y == QG_EMPTY_WORD) return -1;
    }
    h = (h + 1) & hmask;
  }
  atomicOr(err, QG_DEVERR_PROBE);
  return -1;
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

// Epilogue options for the fused Lanczos step (see qgpu_krylov.cu):
//   src_scale:  x is used as x * src_scale[k] with entries |x*scale| <= thr[k] read as zero
//               (normalisation and truncation of the Krylov vector folded into the gather);
//   own_out:    row r of the scaled/truncated x written back (the stored Krylov vector);
//   prev/beta:  y = H x - beta[k] * prev;
//   dot:        per-block partial sums of conj(x_r) * (H x)_r written to dot_part.
struct ApplyFuse {
  const double *src_scale = nullptr;  // [nvec]
  const double *thr2 = nullptr;       // [nvec] squared truncation threshold, after scaling
  double2 *own_out = nullptr;
  const double2 *prev = nullptr;
  const double *beta = nullptr;  // [nvec]
  double2 *dot_part = nullptr;   // [gridDim.x * nvec]
};
qg_status qg_apply_launch(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, double *y,
                          int nvec, const ApplyFuse *fz);
// x row stride xs, y row stride ys (complex entries), nvec columns from the given pointers
qg_status qg_apply_strided(qg_context ctx, qg_operator op, qg_basis dst, qg_basis src, const double *x, int xs,
                           double *y, int ys, int nvec, const ApplyFuse *fz);

// reductions (qgpu_krylov.cu)
qg_status qg_dot_dev(qg_context ctx, int64_t n, int nvec, const double *x, const double *y, double *out_dev);
