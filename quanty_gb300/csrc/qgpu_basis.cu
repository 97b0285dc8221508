// Determinant bases on the device: conversion from the reference byte layout, sorting,
// the lookup hash, and basis growth (targets of an operator, closure, union) through an
// open-addressing hash with atomicCAS insert.
//
// The reference stores a basis as blocked byte arrays with a chained hash
// (Core/StructDef.cpp:188-206, Core/Hash.cpp:163) and grows it one element at a time under
// an OpenMP critical section (ComplexWaveFunctionAddElementOMPMiniFlush,
// Core/ComplexWaveFunctionArithmetic.cpp:453-473).  Here a basis is a sorted array of W-word
// keys plus an open-addressing table (linear probing, load <= 1/2) mapping key -> row.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>

#include "qgpu_internal.cuh"

// ------------------------------------------------------------------ small device pieces

__device__ __forceinline__ void qg_cas128(unsigned long long *addr, unsigned long long clo,
                                          unsigned long long chi, unsigned long long nlo,
                                          unsigned long long nhi, unsigned long long &olo,
                                          unsigned long long &ohi) {
  asm volatile(
      "{\n\t.reg .b128 c, n, o;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 n, {%4, %5};\n\t"
      "atom.global.cas.b128 o, [%6], c, n;\n\t"
      "mov.b128 {%0, %1}, o;\n\t}"
      : "=l"(olo), "=l"(ohi)
      : "l"(clo), "l"(chi), "l"(nlo), "l"(nhi), "l"(addr)
      : "memory");
}

// Insert a key into the set; returns 1 if this call inserted it, 0 if it was present, -1 if the probe limit was hit.  The slot index
// is stored to *slot_out.
// Each probe reads the slot first (at L2, bypassing L1, which may hold an old copy) and takes
// the atomic only where that read cannot settle it.  A slot changes once, from empty (both
// words all ones) to a whole key, so a read with neither word all ones is that key even if the
// two words were read apart; a read with an all-ones word (an empty slot, one being filled, or
// a key whose low word is all ones) goes to the CAS, which returns the slot's true contents.
// Most inserts of a closure find their key already present, so they cost loads, not atomics.
template <int W>
__device__ __forceinline__ int qg_set_insert(Slot *slots, uint64_t hmask, const Key<W> &k, int64_t *slot_out) {
  uint64_t h = qg_hash<W>(k) & hmask;
  uint64_t k1 = (W == 1) ? 0ull : k.w[W - 1];
  for (int p = 0; p < QG_PROBE_LIMIT; p++) {
    unsigned long long *a = reinterpret_cast<unsigned long long *>(slots + h);
    ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(a));
    if (v.x != QG_EMPTY_WORD && v.y != QG_EMPTY_WORD) {
      if (v.x == k.w[0] && v.y == k1) {
        *slot_out = (int64_t)h;
        return 0;
      }
      h = (h + 1) & hmask;
      continue;
    }
    unsigned long long olo, ohi;
    qg_cas128(a, QG_EMPTY_WORD, QG_EMPTY_WORD, k.w[0], k1, olo, ohi);
    if (olo == QG_EMPTY_WORD && ohi == QG_EMPTY_WORD) {
      *slot_out = (int64_t)h;
      return 1;
    }
    if (olo == k.w[0] && ohi == k1) {
      *slot_out = (int64_t)h;
      return 0;
    }
    h = (h + 1) & hmask;
  }
  return -1;
}

__global__ void k_slots_clear(Slot *slots, uint32_t *slot_row, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Slot s;
  s.k[0] = QG_EMPTY_WORD;
  s.k[1] = QG_EMPTY_WORD;
  s.vre = 0.0;
  s.vim = 0.0;
  slots[i] = s;
  if (slot_row) slot_row[i] = QG_NO_INDEX;
}

// Unique keys -> table rows (full-key CAS claims the slot), plus both index maps.
template <int W>
__global__ void k_hash_build(Slot *slots, uint32_t *slot_row, uint32_t *row_slot, uint64_t hmask, const Key<W> *keys,
                             int64_t n, unsigned int *err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t h = -1;
  if (qg_set_insert<W>(slots, hmask, keys[i], &h) < 0) {
    atomicOr(err, QG_DEVERR_PROBE);
    return;
  }
  slot_row[h] = (uint32_t)i;
  row_slot[i] = (uint32_t)h;
}

// Reference bytes (orbital i in byte i>>3, mask 128>>(i&7)) -> key (orbital i at bit nf-1-i).
template <int W>
__global__ void k_bytes_to_keys(const uint8_t *bytes, int nf, int nword, int64_t n, Key<W> *keys) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  Key<W> k;
  for (int j = 0; j < W; j++) k.w[j] = 0;
  const uint8_t *b = bytes + r * nword;
  for (int i = 0; i < nf; i++) {
    if (b[i >> 3] & (128 >> (i & 7))) {
      int p = nf - 1 - i;
      k.w[p >> 6] |= 1ull << (p & 63);
    }
  }
  keys[r] = k;
}

template <int W>
__global__ void k_keys_to_bytes(const Key<W> *keys, int nf, int nword, int64_t n, uint8_t *bytes) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  Key<W> k = keys[r];
  uint8_t *b = bytes + r * nword;
  for (int j = 0; j < nword; j++) b[j] = 0;
  for (int i = 0; i < nf; i++) {
    int p = nf - 1 - i;
    if ((k.w[p >> 6] >> (p & 63)) & 1ull) b[i >> 3] |= (uint8_t)(128 >> (i & 7));
  }
}

template <int W>
__global__ void k_extract_word(const Key<W> *keys, const uint32_t *idx, int64_t n, int w, uint64_t *out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = keys[idx ? idx[i] : i].w[w];
}

__global__ void k_iota(uint32_t *v, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

template <int W>
__global__ void k_gather_keys(const Key<W> *in, const uint32_t *idx, int64_t n, Key<W> *out, uint32_t *flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Key<W> k = in[idx[i]];
  out[i] = k;
  uint32_t f = 1;
  if (i > 0) f = qg_eq<W>(k, in[idx[i - 1]]) ? 0u : 1u;
  flag[i] = f;
}

template <int W>
__global__ void k_compact_unique(const Key<W> *sorted, const uint32_t *flag, const uint32_t *pos_incl,
                                 const uint32_t *idx, int64_t n, Key<W> *uniq, int64_t *perm) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t u = pos_incl[i] - 1;
  if (flag[i]) uniq[u] = sorted[i];
  if (perm) perm[idx[i]] = (int64_t)u;
}

static inline unsigned grid_for(int64_t n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

static int64_t hcap_for(int64_t n) {
  int64_t c = 64;
  while (c < 2 * n) c <<= 1;
  return c;
}

template <int W>
static qg_status build_hash_t(qg_basis b) {
  qg_context ctx = b->ctx;
  int64_t hcap = hcap_for(b->n);
  if (b->d_slots && b->hcap != hcap) {
    cudaFree(b->d_slots);
    cudaFree(b->d_slot_row);
    b->d_slots = nullptr;
    b->d_slot_row = nullptr;
  }
  cudaError_t e = cudaSuccess;
  if (!b->d_slots) {
    e = cudaMalloc(&b->d_slots, hcap * sizeof(Slot));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_slot_row, hcap * sizeof(uint32_t));
  }
  if (e == cudaSuccess && !b->d_row_slot) e = cudaMalloc(&b->d_row_slot, std::max<int64_t>(b->n, 1) * sizeof(uint32_t));
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "hash table");
  b->hcap = hcap;
  k_slots_clear<<<grid_for(hcap), 256, 0, ctx->stream>>>(b->d_slots, b->d_slot_row, hcap);
  ctx->launches++;
  if (b->n) {
    k_hash_build<W><<<grid_for(b->n), 256, 0, ctx->stream>>>(b->d_slots, b->d_slot_row, b->d_row_slot,
                                                             (uint64_t)(hcap - 1), (const Key<W> *)b->d_keys, b->n,
                                                             ctx->d_err);
    ctx->launches++;
  }
  return qg_check_launch(ctx, "hash build");
}

qg_status qg_basis_build_hash(qg_basis b) { return b->W == 1 ? build_hash_t<1>(b) : build_hash_t<2>(b); }

// Sort device keys, merge duplicates, build the basis.  d_perm (optional) receives for each
// input key its row in the basis.
template <int W>
static qg_status from_keys_t(qg_context ctx, int nf, void *d_keys_in, int64_t n, qg_basis *out, int64_t *d_perm) {
  cudaStream_t s = ctx->stream;
  qg_basis b = new qg_basis_s();
  b->ctx = ctx;
  b->nf = nf;
  b->W = W;
  if (n > (int64_t)0xFFFFFFF0) {
    delete b;
    ctx->last_error = "basis larger than 2^32 determinants";
    return QG_ERR_ARG;
  }
  const Key<W> *keys = (const Key<W> *)d_keys_in;
  uint32_t *idx = nullptr, *idx2 = nullptr, *flag = nullptr, *pos = nullptr;
  uint64_t *w = nullptr, *w2 = nullptr;
  Key<W> *sorted = nullptr;
  void *tmp = nullptr;
  size_t tmpb = 0, need = 0;
  cudaError_t e = cudaSuccess;
  int64_t nn = std::max<int64_t>(n, 1);
#define ALLOC(p, bytes) \
  if (e == cudaSuccess) e = cudaMalloc((void **)&p, bytes)
  ALLOC(idx, nn * 4);
  ALLOC(idx2, nn * 4);
  ALLOC(flag, nn * 4);
  ALLOC(pos, nn * 4);
  ALLOC(w, nn * 8);
  ALLOC(w2, nn * 8);
  ALLOC(sorted, nn * sizeof(Key<W>));
  if (e == cudaSuccess) {
    cub::DeviceRadixSort::SortPairs(nullptr, need, w, w2, idx, idx2, (int)nn, 0, 64, s);
    tmpb = need;
    cub::DeviceScan::InclusiveSum(nullptr, need, flag, pos, (int)nn, s);
    tmpb = std::max(tmpb, need);
    ALLOC(tmp, tmpb);
  }
#undef ALLOC
  int64_t nuniq = 0;
  if (e == cudaSuccess && n > 0) {
    k_iota<<<grid_for(n), 256, 0, s>>>(idx, n);
    ctx->launches++;
    // LSD over words: low word first, then (stable) the higher ones
    for (int wd = 0; wd < W; wd++) {
      int lo_bit = 64 * wd, hi_bit = std::min(nf, 64 * (wd + 1));
      if (hi_bit <= lo_bit) continue;
      k_extract_word<W><<<grid_for(n), 256, 0, s>>>(keys, idx, n, wd, w);
      ctx->launches++;
      size_t tb = tmpb;
      e = cub::DeviceRadixSort::SortPairs(tmp, tb, w, w2, idx, idx2, (int)n, 0, hi_bit - lo_bit, s);
      ctx->launches += 4;
      if (e != cudaSuccess) break;
      std::swap(idx, idx2);
    }
    if (e == cudaSuccess) {
      k_gather_keys<W><<<grid_for(n), 256, 0, s>>>(keys, idx, n, sorted, flag);
      ctx->launches++;
      size_t tb = tmpb;
      e = cub::DeviceScan::InclusiveSum(tmp, tb, flag, pos, (int)n, s);
      ctx->launches += 2;
    }
    if (e == cudaSuccess) {
      uint32_t last = 0;
      e = cudaMemcpyAsync(&last, pos + (n - 1), 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      nuniq = last;
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_keys, std::max<int64_t>(nuniq, 1) * sizeof(Key<W>));
    if (e == cudaSuccess) {
      k_compact_unique<W><<<grid_for(n), 256, 0, s>>>(sorted, flag, pos, idx, n, (Key<W> *)b->d_keys, d_perm);
      ctx->launches++;
    }
  } else if (e == cudaSuccess) {
    e = cudaMalloc(&b->d_keys, sizeof(Key<W>));
  }
  cudaStreamSynchronize(s);
  cudaFree(idx);
  cudaFree(idx2);
  cudaFree(flag);
  cudaFree(pos);
  cudaFree(w);
  cudaFree(w2);
  cudaFree(sorted);
  cudaFree(tmp);
  if (e != cudaSuccess) {
    qg_basis_destroy(b);
    return qg_cuda_fail(ctx, e, "basis sort");
  }
  b->n = nuniq;
  qg_status st = qg_basis_build_hash(b);
  if (st != QG_OK) {
    qg_basis_destroy(b);
    return st;
  }
  *out = b;
  return QG_OK;
}

qg_status qg_basis_from_device_keys(qg_context ctx, int nf, int W, void *d_keys, int64_t n, qg_basis *out,
                                    int64_t *d_perm) {
  return W == 1 ? from_keys_t<1>(ctx, nf, d_keys, n, out, d_perm) : from_keys_t<2>(ctx, nf, d_keys, n, out, d_perm);
}

extern "C" qg_status qg_basis_create(qg_context ctx, int32_t nf, int64_t n, const uint8_t *dets_host, qg_basis *basis,
                                     int64_t *perm_host) {
  if (!ctx || !basis || nf <= 0 || nf > 127 || n < 0 || (n > 0 && !dets_host)) {
    if (ctx) ctx->last_error = "qg_basis_create: bad argument (need 0 < nf <= 127)";
    return QG_ERR_ARG;
  }
  int W = qg_words_for(nf), nword = (nf + 7) / 8;
  cudaStream_t s = ctx->stream;
  uint8_t *d_bytes = nullptr;
  void *d_keys = nullptr;
  int64_t *d_perm = nullptr;
  int64_t nn = std::max<int64_t>(n, 1);
  QG_CUDA(ctx, cudaMalloc(&d_bytes, nn * nword));
  QG_CUDA(ctx, cudaMalloc(&d_keys, nn * 8 * W));
  if (perm_host) QG_CUDA(ctx, cudaMalloc(&d_perm, nn * 8));
  if (n) QG_CUDA(ctx, cudaMemcpyAsync(d_bytes, dets_host, n * nword, cudaMemcpyHostToDevice, s));
  if (n) {
    if (W == 1)
      k_bytes_to_keys<1><<<grid_for(n), 256, 0, s>>>(d_bytes, nf, nword, n, (Key<1> *)d_keys);
    else
      k_bytes_to_keys<2><<<grid_for(n), 256, 0, s>>>(d_bytes, nf, nword, n, (Key<2> *)d_keys);
    ctx->launches++;
  }
  qg_status st = qg_basis_from_device_keys(ctx, nf, W, d_keys, n, basis, d_perm);
  if (st == QG_OK && perm_host && n) {
    cudaError_t e = cudaMemcpyAsync(perm_host, d_perm, n * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = qg_cuda_fail(ctx, e, "perm copy");
  }
  cudaStreamSynchronize(s);
  cudaFree(d_bytes);
  cudaFree(d_keys);
  cudaFree(d_perm);
  if (st == QG_OK) st = qg_check_device_error(ctx, "qg_basis_create");
  return st;
}

extern "C" qg_status qg_basis_destroy(qg_basis b) {
  if (!b) return QG_OK;
  cudaFree(b->d_keys);
  cudaFree(b->d_slots);
  cudaFree(b->d_slot_row);
  cudaFree(b->d_row_slot);
  cudaFree(b->d_rmask);
  cudaFree(b->d_rmin);
  cudaFree(b->d_rmax);
  for (auto &c : b->caches) qg_cache_free(c);
  delete b;
  return QG_OK;
}

qg_status qg_basis_set_windows(qg_basis b, int nres, const uint64_t *mask_host, const int32_t *min_host,
                               const int32_t *max_host) {
  qg_context ctx = b->ctx;
  cudaFree(b->d_rmask);
  cudaFree(b->d_rmin);
  cudaFree(b->d_rmax);
  b->d_rmask = nullptr;
  b->d_rmin = b->d_rmax = nullptr;
  b->nres = 0;
  if (nres <= 0) return QG_OK;
  QG_CUDA(ctx, cudaMalloc(&b->d_rmask, (size_t)nres * b->W * 8));
  QG_CUDA(ctx, cudaMalloc(&b->d_rmin, nres * 4));
  QG_CUDA(ctx, cudaMalloc(&b->d_rmax, nres * 4));
  QG_CUDA(ctx, cudaMemcpy(b->d_rmask, mask_host, (size_t)nres * b->W * 8, cudaMemcpyHostToDevice));
  QG_CUDA(ctx, cudaMemcpy(b->d_rmin, min_host, nres * 4, cudaMemcpyHostToDevice));
  QG_CUDA(ctx, cudaMemcpy(b->d_rmax, max_host, nres * 4, cudaMemcpyHostToDevice));
  b->nres = nres;
  b->h_rmask.assign(mask_host, mask_host + (size_t)nres * b->W);
  b->h_rmin.assign(min_host, min_host + nres);
  b->h_rmax.assign(max_host, max_host + nres);
  return QG_OK;
}

extern "C" int64_t qg_basis_size(qg_basis b) { return b ? b->n : -1; }

extern "C" qg_status qg_basis_get_dets(qg_basis b, uint8_t *dets_host) {
  if (!b || (!dets_host && b->n)) return QG_ERR_ARG;
  qg_context ctx = b->ctx;
  int nword = (b->nf + 7) / 8;
  if (!b->n) return QG_OK;
  uint8_t *d = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d, b->n * nword));
  if (b->W == 1)
    k_keys_to_bytes<1><<<grid_for(b->n), 256, 0, ctx->stream>>>((const Key<1> *)b->d_keys, b->nf, nword, b->n, d);
  else
    k_keys_to_bytes<2><<<grid_for(b->n), 256, 0, ctx->stream>>>((const Key<2> *)b->d_keys, b->nf, nword, b->n, d);
  ctx->launches++;
  cudaError_t e = cudaMemcpyAsync(dets_host, d, b->n * nword, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_basis_get_dets");
  return QG_OK;
}

template <int W>
__global__ void k_find(const Slot *slots, const uint32_t *slot_row, uint64_t hmask, const Key<W> *q, int64_t n,
                       int64_t *out, unsigned int *err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = qg_lookup<W>(slots, slot_row, hmask, q[i], err);
}

extern "C" qg_status qg_basis_find(qg_basis b, int64_t n, const uint8_t *dets_host, int64_t *index_host) {
  if (!b || n < 0 || (n && (!dets_host || !index_host))) return QG_ERR_ARG;
  if (!n) return QG_OK;
  qg_context ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  int nword = (b->nf + 7) / 8;
  uint8_t *d_bytes = nullptr;
  void *d_keys = nullptr;
  int64_t *d_out = nullptr;
  QG_CUDA(ctx, cudaMalloc(&d_bytes, n * nword));
  QG_CUDA(ctx, cudaMalloc(&d_keys, n * 8 * b->W));
  QG_CUDA(ctx, cudaMalloc(&d_out, n * 8));
  QG_CUDA(ctx, cudaMemcpyAsync(d_bytes, dets_host, n * nword, cudaMemcpyHostToDevice, s));
  if (b->W == 1) {
    k_bytes_to_keys<1><<<grid_for(n), 256, 0, s>>>(d_bytes, b->nf, nword, n, (Key<1> *)d_keys);
    k_find<1><<<grid_for(n), 256, 0, s>>>(b->d_slots, b->d_slot_row, b->hcap - 1, (const Key<1> *)d_keys, n, d_out,
                                          ctx->d_err);
  } else {
    k_bytes_to_keys<2><<<grid_for(n), 256, 0, s>>>(d_bytes, b->nf, nword, n, (Key<2> *)d_keys);
    k_find<2><<<grid_for(n), 256, 0, s>>>(b->d_slots, b->d_slot_row, b->hcap - 1, (const Key<2> *)d_keys, n, d_out,
                                          ctx->d_err);
  }
  ctx->launches += 2;
  cudaError_t e = cudaMemcpyAsync(index_host, d_out, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_bytes);
  cudaFree(d_keys);
  cudaFree(d_out);
  if (e != cudaSuccess) return qg_cuda_fail(ctx, e, "qg_basis_find");
  return qg_check_device_error(ctx, "qg_basis_find");
}

// ------------------------------------------------------------------ growth

// Insert the n keys of a warp's queue, 32 at a time (one per lane, independent probes);
// true on every lane if any insert hit the probe limit or found the list full.
template <int W>
__device__ __forceinline__ bool expand_flush(const Key<W> *q, int n, int lane, Slot *slots, uint64_t hmask,
                                             Key<W> *list, unsigned long long *count, unsigned long long limit,
                                             unsigned int *err) {
  bool bad = false;
  for (int i = lane; i < n; i += 32) {
    int64_t hs;
    int ins = qg_set_insert<W>(slots, hmask, q[i], &hs);
    if (ins < 0) {
      atomicOr(err, QG_DEVERR_PROBE);
      bad = true;
      break;
    }
    if (ins == 1) {
      unsigned long long pos = atomicAdd(count, 1ull);
      if (pos >= limit) {
        atomicOr(err, QG_DEVERR_TABLE_FULL);
        bad = true;
        break;
      }
      list[pos] = q[i];
    }
  }
  return __any_sync(0xffffffffu, bad);
}

#define QG_XQ 128  // entries of a warp's insert queue

// Expand the rows [r0, r1) of a key list through the forward (push) table: each applicable
// term's target that passes the restrictions is inserted into the set; new keys are appended
// to the list.  Lane per source determinant; the warp walks the groups and terms together
// (a group is skipped when no lane's source has its need1 bits) and queues the targets of all
// 32 lanes in shared memory, compacted by ballot; a full queue is inserted 32 keys at a time,
// one independent probe per lane, so inserts neither diverge nor wait on one another.  In a
// closure (skip_diag) the sources are members of the set already, so the terms that leave a
// determinant unchanged -- the densities and Coulomb direct terms, most of a Hamiltonian's
// applicable terms -- are skipped, a whole group at a time where the group holds only those.
// A round stops early once an insert has found the list full (the host grows the set and
// repeats the round): a thread checks the error word when it starts and stops at its first
// new key past the limit, so the set exceeds the list capacity by at most one key per
// resident thread.
// With twreq (one 64-bit word per term) the occupation windows are tested with one AND: bit
// 5q + D + 2 of a source's mask says its count in window q plus D, D in [-2, 2], stays inside
// the window, and a term's word holds the bit of its change D_q for every window (D_q = 0
// included, so a source outside a window passes none of its terms).
template <int W>
__global__ void __launch_bounds__(256) k_expand(const Key<W> *src, int64_t r0, int64_t r1,
                                                const GroupDev<W> *__restrict__ groups, int ngroups,
                                                const TermDev<W> *__restrict__ terms, int nres,
                                                const uint64_t *__restrict__ rmask, const int32_t *__restrict__ rmin,
                                                const int32_t *__restrict__ rmax, const uint64_t *__restrict__ twreq,
                                                Slot *slots, uint64_t hmask, Key<W> *list, unsigned long long *count,
                                                unsigned long long limit, unsigned int *err, int skip_diag) {
  __shared__ Key<W> queue[8][QG_XQ];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  Key<W> *q = queue[wid];
  int64_t r = r0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool live = r < r1 && !(*(volatile unsigned int *)err & (QG_DEVERR_TABLE_FULL | QG_DEVERR_PROBE));
  Key<W> d;
#pragma unroll
  for (int i = 0; i < W; i++) d.w[i] = live ? src[r].w[i] : 0ull;
  if (!__any_sync(0xffffffffu, live)) return;  // warp-uniform
  uint64_t okm = 0;
  if (twreq) {
    for (int c = 0; c < nres; c++) {
      int n = 0;
#pragma unroll
      for (int i = 0; i < W; i++) n += __popcll(d.w[i] & rmask[c * W + i]);
#pragma unroll
      for (int D = -2; D <= 2; D++)
        if (n + D >= rmin[c] && n + D <= rmax[c]) okm |= 1ull << (5 * c + D + 2);
    }
  }
  int qn = 0;
  bool halt = false;
  for (int g = 0; g < ngroups && !halt; g++) {
    const GroupDev<W> &G = groups[g];
    if (skip_diag && G.diag) continue;
    bool ok = live;
#pragma unroll
    for (int i = 0; i < W; i++) ok &= (d.w[i] & G.need1[i]) == G.need1[i];
    if (!__any_sync(0xffffffffu, ok)) continue;
    const int tb = G.begin, te = G.end;
    for (int t = tb; t < te; t++) {
      const TermDev<W> &T = terms[t];
      bool has = ok, moved = false;
#pragma unroll
      for (int i = 0; i < W; i++) {
        has &= (d.w[i] & T.need0[i]) == 0;
        moved |= T.flip[i] != 0;
      }
      // a term whose value is zero (a sum operator's component scaled to 0) reaches nothing,
      // as in the reference, whose operators hold no zero terms
      has &= !(T.vre == 0.0 && T.vim == 0.0) && !(skip_diag && !moved);
      Key<W> tg;
#pragma unroll
      for (int i = 0; i < W; i++) tg.w[i] = d.w[i] ^ T.flip[i];
      if (twreq) {
        const uint64_t req = twreq[t];
        has &= (okm & req) == req;
      } else {
        for (int c = 0; c < nres && has; c++) {
          int n = 0;
#pragma unroll
          for (int i = 0; i < W; i++) n += __popcll(tg.w[i] & rmask[c * W + i]);
          has = (n >= rmin[c]) && (n <= rmax[c]);
        }
      }
      unsigned m = __ballot_sync(0xffffffffu, has);
      if (has) q[qn + __popc(m & below)] = tg;
      qn += __popc(m);
      if (qn > QG_XQ - 32) {
        __syncwarp();
        halt = expand_flush<W>(q, qn, lane, slots, hmask, list, count, limit, err);
        qn = 0;
        __syncwarp();
        if (halt) break;
      }
    }
  }
  __syncwarp();
  if (!halt && qn) expand_flush<W>(q, qn, lane, slots, hmask, list, count, limit, err);
}

template <int W>
__global__ void k_count_outside(const Key<W> *keys, int64_t n, int nres, const uint64_t *rmask, const int32_t *rmin,
                                const int32_t *rmax, unsigned long long *bad) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Key<W> k = keys[i];
  for (int q = 0; q < nres; q++) {
    int c = 0;
    for (int j = 0; j < W; j++) c += __popcll(k.w[j] & rmask[q * W + j]);
    if (c < rmin[q] || c > rmax[q]) {
      atomicAdd(bad, 1ull);
      return;
    }
  }
}

template <int W>
__global__ void k_set_insert_list(Slot *slots, uint64_t hmask, const Key<W> *list, int64_t n, unsigned int *err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t h;
  if (qg_set_insert<W>(slots, hmask, list[i], &h) < 0) atomicOr(err, QG_DEVERR_PROBE);
}

namespace {

struct Restrictions {
  std::vector<uint64_t> mask;
  std::vector<int32_t> mn, mx;
  int n = 0;
};

// reference byte masks -> device key masks
bool convert_restrictions(int nf, int W, const qg_restrictions *res, Restrictions &out) {
  out.n = 0;
  if (!res || res->n <= 0) return true;
  if (!res->masks || !res->min || !res->max) return false;
  int nword = (nf + 7) / 8;
  out.n = res->n;
  out.mask.assign((size_t)res->n * W, 0);
  for (int q = 0; q < res->n; q++) {
    for (int i = 0; i < nf; i++) {
      if (res->masks[q * nword + (i >> 3)] & (128 >> (i & 7))) {
        int p = nf - 1 - i;
        out.mask[q * W + (p >> 6)] |= 1ull << (p & 63);
      }
    }
    out.mn.push_back(res->min[q]);
    out.mx.push_back(res->max[q]);
  }
  return true;
}

}  // namespace

// Grow a key set through the push table.  Starts from `seed_keys` (n_seed keys, inserted
// first when include_seed) and expands for up to max_rounds rounds (-1: until no new key).
// When include_seed is false only one round is made and the result is the target set.
template <int W>
static qg_status grow_t(qg_context ctx, qg_operator op, const Key<W> *seed_keys, int64_t n_seed, bool include_seed,
                        const qg_restrictions *res, int max_rounds, qg_basis *out, int *rounds_done) {
  cudaStream_t s = ctx->stream;
  Restrictions R;
  if (!convert_restrictions(op->nf, W, res, R)) return QG_ERR_ARG;
  uint64_t *d_rmask = nullptr, *d_twreq = nullptr;
  int32_t *d_rmin = nullptr, *d_rmax = nullptr;
  // per push term, the window bits its target needs (when every window change fits the code)
  std::vector<uint64_t> twreq;
  if (R.n > 0 && R.n <= 12 && op->push.nterms > 0) {
    const GroupDev<W> *hg = (const GroupDev<W> *)op->push.h_blob.data();
    const TermDev<W> *ht = (const TermDev<W> *)(op->push.h_blob.data() + op->push.ngroups * sizeof(GroupDev<W>));
    twreq.assign(op->push.nterms, 0);
    bool exact = true;
    for (int g = 0; g < op->push.ngroups && exact; g++)
      for (int t = hg[g].begin; t < hg[g].end && exact; t++)
        for (int q = 0; q < R.n && exact; q++) {
          int D = 0;
          for (int i = 0; i < W; i++) {
            // every flipped orbital has a fixed state in the source (need0 or need1), so the
            // window change is a term constant; otherwise fall back to counting the target
            if (ht[t].flip[i] & ~(ht[t].need0[i] | hg[g].need1[i])) exact = false;
            const uint64_t m = R.mask[(size_t)q * W + i];
            D += __builtin_popcountll(ht[t].flip[i] & ht[t].need0[i] & m) -
                 __builtin_popcountll(ht[t].flip[i] & hg[g].need1[i] & m);
          }
          if (D < -2 || D > 2)
            exact = false;
          else
            twreq[t] |= 1ull << (5 * q + D + 2);
        }
    if (!exact) twreq.clear();
  }
  if (R.n) {
    QG_CUDA(ctx, cudaMalloc(&d_rmask, R.mask.size() * 8));
    QG_CUDA(ctx, cudaMalloc(&d_rmin, R.n * 4));
    QG_CUDA(ctx, cudaMalloc(&d_rmax, R.n * 4));
    QG_CUDA(ctx, cudaMemcpy(d_rmask, R.mask.data(), R.mask.size() * 8, cudaMemcpyHostToDevice));
    QG_CUDA(ctx, cudaMemcpy(d_rmin, R.mn.data(), R.n * 4, cudaMemcpyHostToDevice));
    QG_CUDA(ctx, cudaMemcpy(d_rmax, R.mx.data(), R.n * 4, cudaMemcpyHostToDevice));
    if (!twreq.empty()) {
      QG_CUDA(ctx, cudaMalloc(&d_twreq, twreq.size() * 8));
      QG_CUDA(ctx, cudaMemcpy(d_twreq, twreq.data(), twreq.size() * 8, cudaMemcpyHostToDevice));
    }
  }
  // list capacity; the set has 2*cap slots.  An expansion stops inserting once the list is
  // full; each thread resident at that moment can add at most one key past it (well under
  // 2^20 in all), so the set stays below 2/3 load.
  int64_t cap = 1 << 20;
  while (cap < 4 * (n_seed + 1)) cap <<= 1;
  Key<W> *list = nullptr;
  Slot *slots = nullptr;
  unsigned long long *d_count = nullptr;
  qg_status st = QG_OK;
  cudaError_t e = cudaMalloc(&d_count, 8);
  auto alloc_table = [&](int64_t c) -> cudaError_t {
    cudaFree(slots);
    slots = nullptr;
    cudaError_t ee = cudaMalloc(&slots, 2 * c * sizeof(Slot));
    if (ee != cudaSuccess) return ee;
    k_slots_clear<<<grid_for(2 * c), 256, 0, s>>>(slots, nullptr, 2 * c);
    ctx->launches++;
    return cudaGetLastError();
  };
  if (e == cudaSuccess) e = cudaMalloc(&list, cap * sizeof(Key<W>));
  if (e == cudaSuccess) e = alloc_table(cap);
  unsigned long long count = 0;
  if (e == cudaSuccess && include_seed && n_seed) {
    // seed keys are unique (a basis): copy them to the list and the set
    e = cudaMemcpyAsync(list, seed_keys, n_seed * sizeof(Key<W>), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
      k_set_insert_list<W><<<grid_for(n_seed), 256, 0, s>>>(slots, (uint64_t)(2 * cap - 1), list, n_seed, ctx->d_err);
      ctx->launches++;
    }
    count = n_seed;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_count, &count, 8, cudaMemcpyHostToDevice, s);
  int rounds = 0;
  int64_t f0 = 0, f1 = include_seed ? count : 0;
  const Key<W> *front = include_seed ? list : seed_keys;
  if (!include_seed) {
    f1 = n_seed;
    max_rounds = 1;
  }
  while (e == cudaSuccess && st == QG_OK && f1 > f0 && (max_rounds < 0 || rounds < max_rounds)) {
    unsigned int zero = 0;
    e = cudaMemcpyAsync(ctx->d_err, &zero, 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) break;
    k_expand<W><<<grid_for(f1 - f0), 256, 0, s>>>(
        front, f0, f1, (const GroupDev<W> *)op->push.d_groups, op->push.ngroups, (const TermDev<W> *)op->push.d_terms,
        R.n, d_rmask, d_rmin, d_rmax, d_twreq, slots, (uint64_t)(2 * cap - 1), list, d_count,
        (unsigned long long)cap, ctx->d_err, include_seed ? 1 : 0);
    ctx->launches++;
    unsigned int herr = 0;
    e = cudaMemcpyAsync(&count, d_count, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, ctx->d_err, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) break;
    if (herr & QG_DEVERR_PROBE) {
      st = QG_ERR_TIMEOUT;
      ctx->last_error = "hash probe limit reached during basis growth";
      break;
    }
    if ((herr & QG_DEVERR_TABLE_FULL) || count > (unsigned long long)cap) {
      // grow: keep the keys that made it into the list, rebuild the set, redo the round
      int64_t kept = std::min<int64_t>((int64_t)count, cap);
      int64_t ncap = cap;
      while (ncap < 2 * (int64_t)count + 1024) ncap <<= 1;
      Key<W> *nlist = nullptr;
      e = cudaMalloc(&nlist, ncap * sizeof(Key<W>));
      if (e != cudaSuccess) break;
      e = cudaMemcpyAsync(nlist, list, kept * sizeof(Key<W>), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) break;
      cudaStreamSynchronize(s);
      cudaFree(list);
      list = nlist;
      if (include_seed) front = list;
      cap = ncap;
      e = alloc_table(cap);
      if (e != cudaSuccess) break;
      k_set_insert_list<W><<<grid_for(kept), 256, 0, s>>>(slots, (uint64_t)(2 * cap - 1), list, kept, ctx->d_err);
      ctx->launches++;
      count = kept;
      e = cudaMemcpyAsync(d_count, &count, 8, cudaMemcpyHostToDevice, s);
      continue;  // same frontier again
    }
    rounds++;
    if (include_seed) {
      f0 = f1;
      f1 = (int64_t)count;
    } else {
      break;
    }
  }
  if (e != cudaSuccess && st == QG_OK) st = qg_cuda_fail(ctx, e, "basis growth");
  if (st == QG_OK) st = qg_basis_from_device_keys(ctx, op->nf, W, list, (int64_t)count, out, nullptr);
  // the grown basis satisfies the windows when its seeds do (targets are filtered): record
  // them so H*psi skips sources that cannot be in it
  if (st == QG_OK && R.n) {
    bool seeds_ok = true;
    if (include_seed && n_seed) {
      unsigned long long *d_bad = nullptr;
      unsigned long long bad = 0;
      if (cudaMalloc(&d_bad, 8) == cudaSuccess) {
        cudaMemsetAsync(d_bad, 0, 8, s);
        k_count_outside<W><<<grid_for(n_seed), 256, 0, s>>>(seed_keys, n_seed, R.n, d_rmask, d_rmin, d_rmax, d_bad);
        ctx->launches++;
        cudaMemcpyAsync(&bad, d_bad, 8, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        cudaFree(d_bad);
        seeds_ok = (bad == 0);
      } else {
        seeds_ok = false;
      }
    }
    if (seeds_ok) st = qg_basis_set_windows(*out, R.n, R.mask.data(), R.mn.data(), R.mx.data());
  }
  cudaStreamSynchronize(s);
  cudaFree(list);
  cudaFree(slots);
  cudaFree(d_count);
  cudaFree(d_rmask);
  cudaFree(d_rmin);
  cudaFree(d_rmax);
  cudaFree(d_twreq);
  if (rounds_done) *rounds_done = rounds;
  return st;
}

extern "C" qg_status qg_operator_psi_basis(qg_context ctx, qg_operator op, qg_basis in, const qg_restrictions *res,
                                           qg_basis *out) {
  if (!ctx || !op || !in || !out || op->nf != in->nf) return QG_ERR_ARG;
  if (op->W == 1) return grow_t<1>(ctx, op, (const Key<1> *)in->d_keys, in->n, false, res, 1, out, nullptr);
  return grow_t<2>(ctx, op, (const Key<2> *)in->d_keys, in->n, false, res, 1, out, nullptr);
}

extern "C" qg_status qg_basis_closure(qg_context ctx, qg_operator op, qg_basis seed, const qg_restrictions *res,
                                      int32_t max_rounds, qg_basis *closed, int32_t *rounds_done) {
  if (!ctx || !op || !seed || !closed || op->nf != seed->nf) return QG_ERR_ARG;
  int r = 0;
  qg_status st;
  if (op->W == 1)
    st = grow_t<1>(ctx, op, (const Key<1> *)seed->d_keys, seed->n, true, res, max_rounds, closed, &r);
  else
    st = grow_t<2>(ctx, op, (const Key<2> *)seed->d_keys, seed->n, true, res, max_rounds, closed, &r);
  if (rounds_done) *rounds_done = r;
  return st;
}

extern "C" qg_status qg_basis_union(qg_context ctx, qg_basis a, qg_basis b, qg_basis *out) {
  if (!ctx || !a || !b || !out || a->nf != b->nf) return QG_ERR_ARG;
  int W = a->W;
  void *d = nullptr;
  int64_t n = a->n + b->n;
  QG_CUDA(ctx, cudaMalloc(&d, std::max<int64_t>(n, 1) * 8 * W));
  QG_CUDA(ctx, cudaMemcpyAsync(d, a->d_keys, a->n * 8 * W, cudaMemcpyDeviceToDevice, ctx->stream));
  QG_CUDA(ctx, cudaMemcpyAsync((char *)d + a->n * 8 * W, b->d_keys, b->n * 8 * W, cudaMemcpyDeviceToDevice, ctx->stream));
  qg_status st = qg_basis_from_device_keys(ctx, a->nf, W, d, n, out, nullptr);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  return st;
}

template <int W>
__global__ void k_map(const Key<W> *dst_keys, int64_t n, const Slot *src_slots, const uint32_t *src_slot_row,
                      uint64_t hmask, const double2 *x, double2 *y, int nvec, unsigned int *err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int64_t j = qg_lookup<W>(src_slots, src_slot_row, hmask, dst_keys[r], err);
  for (int k = 0; k < nvec; k++) y[r * nvec + k] = (j >= 0) ? x[j * nvec + k] : make_double2(0.0, 0.0);
}

extern "C" qg_status qg_basis_map(qg_context ctx, qg_basis src, const double *x_dev, qg_basis dst, double *y_dev,
                                  int32_t nvec) {
  if (!ctx || !src || !dst || src->nf != dst->nf || nvec <= 0) return QG_ERR_ARG;
  if (!dst->n) return QG_OK;
  if (src->W == 1)
    k_map<1><<<grid_for(dst->n), 256, 0, ctx->stream>>>((const Key<1> *)dst->d_keys, dst->n, src->d_slots,
                                                        src->d_slot_row, src->hcap - 1, (const double2 *)x_dev, (double2 *)y_dev, nvec,
                                                        ctx->d_err);
  else
    k_map<2><<<grid_for(dst->n), 256, 0, ctx->stream>>>((const Key<2> *)dst->d_keys, dst->n, src->d_slots,
                                                        src->d_slot_row, src->hcap - 1, (const double2 *)x_dev, (double2 *)y_dev, nvec,
                                                        ctx->d_err);
  ctx->launches++;
  return qg_check_launch(ctx, "qg_basis_map");
}
