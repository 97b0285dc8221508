// Operator upload: ladder strings -> canonical masks -> grouped device term tables.
//
// The reference keeps an operator as strings of ladder codes per length
// (OperatorFixedLengthType, Core/StructDef.cpp:223-236) and evaluates each string on each
// determinant with a byte loop (OperatorCr/OperatorAn/OperatorLader,
// Core/OperatorWaveFunction.cpp:7-115).  Here each string is evaluated once, symbolically,
// into the masks described in qgpu_internal.cuh, strings with identical action are merged,
// and two tables are uploaded:
//   push: forward action grouped by need1 -- a source determinant emits its targets
//         (basis closure);
//   pull: adjoint action grouped by need1 -- a row determinant finds its sources
//         (H*psi without atomics: y_i = sum_t V_t <i|t|j> x_j and <i|t|j> = sign(t^dag, i)).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "qgpu_internal.cuh"

namespace {

struct Masks {
  uint64_t n1[QG_MAXW] = {0, 0}, n0[QG_MAXW] = {0, 0}, fl[QG_MAXW] = {0, 0}, sg[QG_MAXW] = {0, 0};
  bool operator<(const Masks &o) const {
    for (int i = 0; i < QG_MAXW; i++) {
      if (n1[i] != o.n1[i]) return n1[i] < o.n1[i];
      if (n0[i] != o.n0[i]) return n0[i] < o.n0[i];
      if (fl[i] != o.fl[i]) return fl[i] < o.fl[i];
      if (sg[i] != o.sg[i]) return sg[i] < o.sg[i];
    }
    return false;
  }
};

inline void setbit(uint64_t *m, int p) { m[p >> 6] |= 1ull << (p & 63); }
inline int parity_and(const uint64_t *a, const uint64_t *b) {
  int c = 0;
  for (int i = 0; i < QG_MAXW; i++) c += __builtin_popcountll(a[i] & b[i]);
  return c & 1;
}
inline int devbit(int nf, int orb) { return nf - 1 - orb; }

// Symbolic evaluation of one ladder string (o[0] acts first).  Returns false if the string
// vanishes on every determinant.  sign = (-1)^(parity(d & sg) + c).
bool digest(int nf, int len, const uint16_t *o, Masks &m, int &c) {
  std::vector<int> init(nf, -1), tog(nf, 0);
  c = 0;
  for (int t = 0; t < len; t++) {
    int q = o[t] & 0x7FFF;
    bool cr = (o[t] & 0x8000) != 0;
    if (q >= nf) return false;
    int cur_needed = cr ? 0 : 1;  // occupation required before this step
    if (init[q] < 0) {
      init[q] = cur_needed ^ tog[q];
    } else if ((init[q] ^ tog[q]) != cur_needed) {
      return false;
    }
    // parity of occupied orbitals j < q in the intermediate determinant
    //   = parity(d & below(q)) ^ parity(toggled-so-far & below(q))
    int tp = 0;
    for (int j = 0; j < q; j++) tp ^= tog[j];
    c ^= tp;
    tog[q] ^= 1;
  }
  // rebuild sg as the xor of the below-sets of all steps: orbital j is in it iff an odd
  // number of steps act on an orbital above j
  std::memset(m.sg, 0, sizeof(m.sg));
  std::vector<int> cnt(nf + 1, 0);
  for (int t = 0; t < len; t++) cnt[(o[t] & 0x7FFF)]++;
  int above = 0;  // number of steps on orbitals > j, mod 2
  for (int j = nf - 1; j >= 0; j--) {
    if (above & 1) setbit(m.sg, devbit(nf, j));
    above += cnt[j];
  }
  for (int q = 0; q < nf; q++) {
    if (init[q] == 1) setbit(m.n1, devbit(nf, q));
    if (init[q] == 0) setbit(m.n0, devbit(nf, q));
    if (tog[q]) setbit(m.fl, devbit(nf, q));
  }
  // canonical form: sign bits on orbitals whose value is fixed on the domain fold into c
  uint64_t fixed[QG_MAXW];
  for (int i = 0; i < QG_MAXW; i++) fixed[i] = m.n1[i] | m.n0[i];
  c ^= parity_and(m.sg, m.n1);
  for (int i = 0; i < QG_MAXW; i++) m.sg[i] &= ~fixed[i];
  return true;
}

// Adjoint action: applicable on d' = d ^ fl; needs swap on flipped bits; same sg;
// const changes by parity(fl & sg).
Masks adjoint(const Masks &m, int &cflip) {
  Masks a;
  for (int i = 0; i < QG_MAXW; i++) {
    a.n1[i] = (m.n1[i] & ~m.fl[i]) | (m.n0[i] & m.fl[i]);
    a.n0[i] = (m.n0[i] & ~m.fl[i]) | (m.n1[i] & m.fl[i]);
    a.fl[i] = m.fl[i];
    a.sg[i] = m.sg[i];
  }
  cflip = parity_and(m.fl, m.sg);
  // re-canonicalise: sg has no bits on n1|n0 of m; on the adjoint domain the fixed bits are
  // the same set, so sg stays canonical.
  return a;
}

struct Entry {
  Masks m;
  double re, im;
  int src = -1;  // forward term it came from
  int sgn = 1;   // sign its value carries relative to that term's value
};

template <int W>
void build_table(qg_context ctx, const std::vector<Entry> &terms, HostTable &tab, qg_status &st,
                 std::vector<HostTerm> *order = nullptr) {
  // group by need1; inside a group diagonal terms first
  std::map<std::vector<uint64_t>, std::vector<int>> groups;
  for (int t = 0; t < (int)terms.size(); t++) {
    std::vector<uint64_t> key(terms[t].m.n1, terms[t].m.n1 + W);
    groups[key].push_back(t);
  }
  // hop groups (one-body moves out of a single orbital p) first, by p; then the rest
  auto popc2 = [&](const uint64_t *m) {
    int c = 0;
    for (int i = 0; i < W; i++) c += __builtin_popcountll(m[i]);
    return c;
  };
  auto bitpos = [&](const uint64_t *m) {  // position of the lowest set bit, word-major
    for (int i = 0; i < W; i++)
      if (m[i]) return 64 * i + __builtin_ctzll(m[i]);
    return -1;
  };
  auto is_hop = [&](const std::vector<int> &idx) {
    uint64_t qs[2] = {0, 0};
    for (int t : idx)
      for (int i = 0; i < W; i++) qs[i] |= terms[t].m.n0[i];
    if (popc2(qs) != (int)idx.size()) return false;  // one term per target orbital q
    for (int t : idx) {
      const Masks &m = terms[t].m;
      if (popc2(m.n1) != 1 || popc2(m.fl) != 2 || popc2(m.n0) != 1) return false;
      for (int i = 0; i < W; i++)
        if ((m.fl[i] & m.n1[i]) != m.n1[i] || (m.fl[i] & ~m.n1[i]) != m.n0[i]) return false;
    }
    return !idx.empty();
  };
  std::vector<std::pair<std::vector<uint64_t>, std::vector<int>>> order_g;
  std::vector<std::pair<std::vector<uint64_t>, std::vector<int>>> rest_g;
  for (auto &kv : groups) (is_hop(kv.second) ? order_g : rest_g).push_back(kv);
  std::sort(order_g.begin(), order_g.end(),
            [&](const auto &a, const auto &b) { return bitpos(a.first.data()) < bitpos(b.first.data()); });
  tab.nhop = (int)order_g.size();
  tab.hopmask[0] = tab.hopmask[1] = 0;
  for (auto &kv : order_g)
    for (int i = 0; i < W; i++) tab.hopmask[i] |= kv.first[i];
  for (auto &kv : order_g) {
    std::vector<int> &idx = kv.second;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return bitpos(terms[a].m.n0) < bitpos(terms[b].m.n0); });
  }
  for (auto &kv : rest_g) order_g.push_back(kv);
  std::vector<GroupDev<W>> g;
  std::vector<TermDev<W>> tt;
  for (auto &kv : order_g) {
    GroupDev<W> gd;
    std::memset(&gd, 0, sizeof(gd));
    for (int i = 0; i < W; i++) gd.need1[i] = kv.first[i];
    gd.begin = (int)tt.size();
    gd.diag = 1;
    gd.hop = (int)g.size() < tab.nhop;
    std::vector<int> idx = kv.second;
    if (gd.hop)
      for (int t : idx)
        for (int i = 0; i < W; i++) gd.qmask[i] |= terms[t].m.n0[i];
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
      bool da = true, db = true;
      for (int i = 0; i < W; i++) {
        da &= terms[a].m.fl[i] == 0;
        db &= terms[b].m.fl[i] == 0;
      }
      return da && !db;
    });
    for (int t : idx) {
      TermDev<W> td;
      std::memset(&td, 0, sizeof(td));
      bool d = true;
      for (int i = 0; i < W; i++) {
        td.need0[i] = terms[t].m.n0[i];
        td.flip[i] = terms[t].m.fl[i];
        td.sgn[i] = terms[t].m.sg[i];
        d &= td.flip[i] == 0;
      }
      if (!d) gd.diag = 0;
      td.vre = terms[t].re;
      td.vim = terms[t].im;
      tt.push_back(td);
      tab.slot_src.push_back({terms[t].src, terms[t].sgn});
      if (order) {
        HostTerm h;
        for (int i = 0; i < 2; i++) {
          h.n1[i] = terms[t].m.n1[i];
          h.n0[i] = terms[t].m.n0[i];
          h.fl[i] = terms[t].m.fl[i];
          h.sg[i] = terms[t].m.sg[i];
        }
        h.re = terms[t].re;
        h.im = terms[t].im;
        h.src = terms[t].src;
        h.sgn = terms[t].sgn;
        order->push_back(h);
      }
    }
    gd.end = (int)tt.size();
    g.push_back(gd);
  }
  tab.ngroups = (int)g.size();
  tab.nterms = (int)tt.size();
  // group index of every term (for kernels that hand terms, not groups, to threads)
  std::vector<uint32_t> tg(tt.size());
  for (int k = 0; k < (int)g.size(); k++)
    for (int t = g[k].begin; t < g[k].end; t++) tg[t] = (uint32_t)k;
  size_t gb = g.size() * sizeof(GroupDev<W>), tb = tt.size() * sizeof(TermDev<W>);
  size_t tgb = (tg.size() * 4 + 15) / 16 * 16;
  tab.tgrp_off = gb + tb;
  tab.bytes = gb + tb + tgb;
  std::vector<unsigned char> blob(std::max<size_t>(tab.bytes, 16), 0);
  if (gb) std::memcpy(blob.data(), g.data(), gb);
  if (tb) std::memcpy(blob.data() + gb, tt.data(), tb);
  if (!tg.empty()) std::memcpy(blob.data() + gb + tb, tg.data(), tg.size() * 4);
  cudaError_t e = cudaMalloc(&tab.d_blob, blob.size());
  if (e == cudaSuccess) e = cudaMemcpy(tab.d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice);
  tab.h_blob = std::move(blob);
  tab.d_groups = tab.d_blob;
  tab.d_terms = (unsigned char *)tab.d_blob + gb;
  st = (e == cudaSuccess) ? QG_OK : qg_cuda_fail(ctx, e, "operator table upload");
}

bool is_diag(const Entry &e) { return e.m.fl[0] == 0 && e.m.fl[1] == 0; }

}  // namespace

namespace {

// Forward terms (zero values dropped unless keep_zero) and their adjoints, with provenance.
void forward_and_adjoint(const std::vector<Masks> &order, const std::vector<std::pair<double, double>> &vals,
                         bool keep_zero, std::vector<Entry> &fwd, std::vector<Entry> &pull) {
  for (size_t t = 0; t < order.size(); t++) {
    const auto &v = vals[t];
    if (!keep_zero && v.first == 0.0 && v.second == 0.0) continue;
    Entry f;
    f.m = order[t];
    f.re = v.first;
    f.im = v.second;
    f.src = (int)t;
    fwd.push_back(f);
    int cf = 0;
    Entry a;
    a.m = adjoint(order[t], cf);
    a.sgn = cf ? -1 : 1;
    a.re = v.first * a.sgn;
    a.im = v.second * a.sgn;
    a.src = (int)t;
    pull.push_back(a);
  }
}

// Hermiticity: the adjoint of every term must be a term with the conjugate value.
int hermitian_of(const std::vector<Entry> &fwd, const std::vector<Entry> &pull) {
  double vmax = 0;
  for (auto &e : fwd) vmax = std::max(vmax, std::hypot(e.re, e.im));
  std::map<Masks, std::pair<double, double>> fm;
  for (auto &e : fwd) fm[e.m] = {e.re, e.im};
  for (auto &e : pull) {
    auto it = fm.find(e.m);
    double er = e.re, ei = -e.im;  // conj of the value of the adjoint term
    double gr = 0, gi = 0;
    if (it != fm.end()) {
      gr = it->second.first;
      gi = it->second.second;
    }
    if (std::hypot(gr - er, gi - ei) > 1e-12 * std::max(1.0, vmax)) return 0;
  }
  return 1;
}

}  // namespace

// An operator from merged forward terms (masks in creation order and their values).  With
// keep_zero, zero-valued terms stay in every table (sum operators: the structure must not
// depend on the coefficients).
static qg_status make_operator(qg_context ctx, int nf, int nterms, int maxlen, const std::vector<Masks> &order,
                               const std::vector<std::pair<double, double>> &vals, bool keep_zero,
                               qg_operator *out) {
  std::vector<Entry> fwd, pull;
  forward_and_adjoint(order, vals, keep_zero, fwd, pull);
  int herm = hermitian_of(fwd, pull);
  qg_operator op = new qg_operator_s();
  op->ctx = ctx;
  op->nf = nf;
  op->W = qg_words_for(nf);
  op->nterms_in = nterms;
  op->nterms = (int)fwd.size();
  op->hermitian = herm;
  op->max_len = maxlen;
  static uint64_t next_uid = 1;
  op->uid = next_uid++;
  op->keep_zero = keep_zero;
  op->fwd_host.resize(order.size());
  for (size_t t = 0; t < order.size(); t++) {
    HostTerm &h = op->fwd_host[t];
    for (int i = 0; i < 2; i++) {
      h.n1[i] = order[t].n1[i];
      h.n0[i] = order[t].n0[i];
      h.fl[i] = order[t].fl[i];
      h.sg[i] = order[t].sg[i];
    }
    h.re = vals[t].first;
    h.im = vals[t].second;
    h.src = (int)t;
  }
  std::vector<Entry> pull_off, diag;
  for (auto &e : pull) (is_diag(e) ? diag : pull_off).push_back(e);
  // local prefix: the leading orbitals that hold every term acting on three or more orbitals
  int minbit = nf;
  for (auto &e : fwd) {
    int cnt = 0;
    for (int i = 0; i < 2; i++) cnt += __builtin_popcountll(e.m.n1[i] | e.m.n0[i] | e.m.fl[i]);
    if (cnt < 3) continue;
    for (int p = 0; p < nf; p++) {
      uint64_t bit = 1ull << (p & 63);
      uint64_t any = e.m.n1[p >> 6] | e.m.n0[p >> 6] | e.m.fl[p >> 6];
      if (any & bit) {
        minbit = std::min(minbit, p);
        break;
      }
    }
  }
  int H = (minbit < nf) ? nf - minbit : 0;
  if (H > 20) H = 0;
  std::vector<Entry> nonlocal;
  if (H > 0) {
    uint64_t lm[2] = {0, 0};
    for (int p = nf - H; p < nf; p++) lm[p >> 6] |= 1ull << (p & 63);
    for (auto &e : pull_off) {
      bool inside = true;
      for (int i = 0; i < 2; i++) inside &= ((e.m.n1[i] | e.m.n0[i] | e.m.fl[i] | e.m.sg[i]) & ~lm[i]) == 0;
      if (inside) {
        HostTerm h;
        for (int i = 0; i < 2; i++) {
          h.n1[i] = e.m.n1[i];
          h.n0[i] = e.m.n0[i];
          h.fl[i] = e.m.fl[i];
          h.sg[i] = e.m.sg[i];
        }
        h.re = e.re;
        h.im = e.im;
        h.src = e.src;
        h.sgn = e.sgn;
        op->local_off.push_back(h);
      } else {
        nonlocal.push_back(e);
      }
    }
  } else {
    nonlocal = pull_off;
  }
  op->H = H;
  qg_status st = QG_OK;
  if (op->W == 1) {
    build_table<1>(ctx, pull, op->pull, st);
    if (st == QG_OK) build_table<1>(ctx, pull_off, op->pull_off, st);
    if (st == QG_OK) build_table<1>(ctx, nonlocal, op->pull_nl, st, &op->nl_host);
    if (st == QG_OK) build_table<1>(ctx, diag, op->diag, st);
    if (st == QG_OK) build_table<1>(ctx, fwd, op->push, st);
  } else {
    build_table<2>(ctx, pull, op->pull, st);
    if (st == QG_OK) build_table<2>(ctx, pull_off, op->pull_off, st);
    if (st == QG_OK) build_table<2>(ctx, nonlocal, op->pull_nl, st, &op->nl_host);
    if (st == QG_OK) build_table<2>(ctx, diag, op->diag, st);
    if (st == QG_OK) build_table<2>(ctx, fwd, op->push, st);
  }
  if (st != QG_OK) {
    qg_operator_destroy(op);
    return st;
  }
  *out = op;
  return QG_OK;
}


extern "C" qg_status qg_operator_create(qg_context ctx, int32_t nf, int32_t nterms, const int32_t *term_len,
                                        const uint16_t *ops, const double *v_re, const double *v_im,
                                        qg_operator *out) {
  if (!ctx || !out || nf <= 0 || nf > 127 || nterms < 0) {
    if (ctx) ctx->last_error = "qg_operator_create: need 0 < nf <= 127";
    return QG_ERR_ARG;
  }
  if (nterms > 0 && (!term_len || !v_re)) return QG_ERR_ARG;
  // digest and merge strings with identical action (the reference merges equal strings
  // through its operator hash, Core/OperatorArithmetic.cpp:322)
  std::map<Masks, std::pair<double, double>> merged;
  std::vector<Masks> order;
  int64_t off = 0;
  int maxlen = 0;
  for (int t = 0; t < nterms; t++) {
    int len = term_len[t];
    if (len < 0 || len > 64) {
      ctx->last_error = "qg_operator_create: ladder string length out of range";
      return QG_ERR_ARG;
    }
    maxlen = std::max(maxlen, len);
    Masks m;
    int c = 0;
    bool ok = digest(nf, len, ops + off, m, c);
    off += len;
    if (!ok) continue;
    double s = c ? -1.0 : 1.0;
    double re = s * v_re[t], im = s * (v_im ? v_im[t] : 0.0);
    auto it = merged.find(m);
    if (it == merged.end()) {
      merged[m] = {re, im};
      order.push_back(m);
    } else {
      it->second.first += re;
      it->second.second += im;
    }
  }
  std::vector<std::pair<double, double>> vals;
  vals.reserve(order.size());
  for (auto &m : order) vals.push_back(merged[m]);
  return make_operator(ctx, nf, nterms, maxlen, order, vals, false, out);
}

extern "C" qg_status qg_operator_destroy(qg_operator op) {
  if (!op) return QG_OK;
  cudaFree(op->pull.d_blob);
  cudaFree(op->pull_off.d_blob);
  cudaFree(op->diag.d_blob);
  cudaFree(op->pull_nl.d_blob);
  cudaFree(op->push.d_blob);
  delete op;
  return QG_OK;
}

extern "C" qg_status qg_operator_info(qg_operator op, int32_t *nterms, int32_t *ngroups, int32_t *hermitian) {
  if (!op) return QG_ERR_ARG;
  if (nterms) *nterms = op->nterms;
  if (ngroups) *ngroups = op->pull.ngroups;
  if (hermitian) *hermitian = op->hermitian;
  return QG_OK;
}

// ------------------------------------------------------------------ parameter scans

namespace {

// Rewrite the values of every term slot of a table from the forward values, and upload the
// blob on the context's stream (ordered after the work already queued that reads it).
template <int W>
qg_status patch_table(qg_context ctx, HostTable &tab, const std::vector<HostTerm> &fwd) {
  if (tab.slot_src.empty()) return QG_OK;
  size_t base = (size_t)tab.ngroups * sizeof(GroupDev<W>);
  for (size_t t = 0; t < tab.slot_src.size(); t++) {
    TermDev<W> td;
    unsigned char *at = tab.h_blob.data() + base + t * sizeof(TermDev<W>);
    std::memcpy(&td, at, sizeof(td));
    const HostTerm &f = fwd[tab.slot_src[t].first];
    td.vre = tab.slot_src[t].second * f.re;
    td.vim = tab.slot_src[t].second * f.im;
    std::memcpy(at, &td, sizeof(td));
  }
  QG_CUDA(ctx, cudaMemcpyAsync(tab.d_blob, tab.h_blob.data(), tab.h_blob.size(), cudaMemcpyHostToDevice, ctx->stream));
  return QG_OK;
}

}  // namespace

extern "C" qg_status qg_operator_create_sum(qg_context ctx, int32_t ncomp, const qg_operator *comps,
                                            const double *coef_re, const double *coef_im, qg_operator *out) {
  if (!ctx || !out || ncomp <= 0 || !comps || !coef_re) return QG_ERR_ARG;
  for (int k = 0; k < ncomp; k++)
    if (!comps[k] || comps[k]->nf != comps[0]->nf) {
      ctx->last_error = "qg_operator_create_sum: components must exist and share nf";
      return QG_ERR_ARG;
    }
  int nf = comps[0]->nf, maxlen = 0, nin = 0;
  // union of the components' forward terms, each term's contribution per component
  std::map<Masks, int> index;
  std::vector<Masks> order;
  std::vector<std::vector<std::pair<int, std::pair<double, double>>>> contrib(ncomp);
  for (int k = 0; k < ncomp; k++) {
    maxlen = std::max(maxlen, comps[k]->max_len);
    nin += comps[k]->nterms_in;
    for (const HostTerm &h : comps[k]->fwd_host) {
      if (!comps[k]->keep_zero && h.re == 0.0 && h.im == 0.0) continue;  // cancelled in the component
      Masks m;
      for (int i = 0; i < 2; i++) {
        m.n1[i] = h.n1[i];
        m.n0[i] = h.n0[i];
        m.fl[i] = h.fl[i];
        m.sg[i] = h.sg[i];
      }
      auto it = index.find(m);
      int id;
      if (it == index.end()) {
        id = (int)order.size();
        index[m] = id;
        order.push_back(m);
      } else {
        id = it->second;
      }
      contrib[k].push_back({id, {h.re, h.im}});
    }
  }
  size_t nu = order.size();
  std::vector<double> cre((size_t)ncomp * nu, 0.0), cim((size_t)ncomp * nu, 0.0);
  for (int k = 0; k < ncomp; k++)
    for (auto &c : contrib[k]) {
      cre[(size_t)k * nu + c.first] += c.second.first;
      cim[(size_t)k * nu + c.first] += c.second.second;
    }
  std::vector<std::pair<double, double>> vals(nu, {0.0, 0.0});
  for (int k = 0; k < ncomp; k++) {
    double pr = coef_re[k], pi = coef_im ? coef_im[k] : 0.0;
    for (size_t t = 0; t < nu; t++) {
      double ar = cre[(size_t)k * nu + t], ai = cim[(size_t)k * nu + t];
      vals[t].first += pr * ar - pi * ai;
      vals[t].second += pr * ai + pi * ar;
    }
  }
  QG_TRY(make_operator(ctx, nf, nin, maxlen, order, vals, true, out));
  (*out)->ncomp = ncomp;
  (*out)->comp_re = std::move(cre);
  (*out)->comp_im = std::move(cim);
  return QG_OK;
}

extern "C" qg_status qg_operator_set_coefficients(qg_operator op, const double *coef_re, const double *coef_im) {
  if (!op || !coef_re || op->ncomp <= 0) {
    if (op) op->ctx->last_error = "qg_operator_set_coefficients: not a sum operator";
    return QG_ERR_ARG;
  }
  qg_context ctx = op->ctx;
  size_t nu = op->fwd_host.size();
  for (size_t t = 0; t < nu; t++) {
    double vr = 0.0, vi = 0.0;
    for (int k = 0; k < op->ncomp; k++) {
      double pr = coef_re[k], pi = coef_im ? coef_im[k] : 0.0;
      double ar = op->comp_re[(size_t)k * nu + t], ai = op->comp_im[(size_t)k * nu + t];
      vr += pr * ar - pi * ai;
      vi += pr * ai + pi * ar;
    }
    op->fwd_host[t].re = vr;
    op->fwd_host[t].im = vi;
  }
  for (HostTerm &h : op->local_off) {
    h.re = h.sgn * op->fwd_host[h.src].re;
    h.im = h.sgn * op->fwd_host[h.src].im;
  }
  for (HostTerm &h : op->nl_host) {
    h.re = h.sgn * op->fwd_host[h.src].re;
    h.im = h.sgn * op->fwd_host[h.src].im;
  }
  HostTable *tabs[5] = {&op->pull, &op->pull_off, &op->diag, &op->pull_nl, &op->push};
  for (HostTable *t : tabs) {
    if (op->W == 1)
      QG_TRY(patch_table<1>(ctx, *t, op->fwd_host));
    else
      QG_TRY(patch_table<2>(ctx, *t, op->fwd_host));
  }
  // Hermiticity of the new values
  std::vector<Masks> order(nu);
  std::vector<std::pair<double, double>> vals(nu);
  for (size_t t = 0; t < nu; t++) {
    const HostTerm &h = op->fwd_host[t];
    for (int i = 0; i < 2; i++) {
      order[t].n1[i] = h.n1[i];
      order[t].n0[i] = h.n0[i];
      order[t].fl[i] = h.fl[i];
      order[t].sg[i] = h.sg[i];
    }
    vals[t] = {h.re, h.im};
  }
  std::vector<Entry> fwd, pull;
  forward_and_adjoint(order, vals, false, fwd, pull);
  op->hermitian = hermitian_of(fwd, pull);
  op->version++;
  return QG_OK;
}
