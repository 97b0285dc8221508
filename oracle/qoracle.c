/*
 * qoracle.c -- CPU oracle for the H*psi / Lanczos / continued-fraction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference algorithm, used
 * by tests/ as the checker and by bench.py as the timed CPU baseline.  The product (the
 * CUDA library under quanty_gb300/csrc) never links, loads or calls it.
 *
 * Parity is pinned by tests/test_oracle_golden.py against fixtures the reference binary
 * produced (the JSON files under tests/golden) and against the known answers of the reference's own tests
 * (TestScripts/CreateSpectra.Quanty golden tridiagonal tables, TestScripts/Eigensystem.Quanty
 * Mathematica eigenvalues).
 *
 * Layout follows the reference: a determinant is NWord = ceil(NF/8) bytes, orbital i in byte
 * i>>3 under mask 128>>(i&7) (Core/OperatorWaveFunction.cpp:7-43,
 * Core/WaveFunctionArithmetic.cpp:130).  A ladder code has bit 15 set for a creation
 * operator (CrAnMask, Core/StructDef.cpp:46); code[0] acts first
 * (Core/OperatorWaveFunction.cpp:98-113).  Bosons are not supported (NewWavefunction rejects
 * them, LuaInterface/ssp.cpp:951-954).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define QO_CR 0x8000u
#define QO_IDX 0x7FFFu

/* ------------------------------------------------------------------ ladder operators */

/* Parity of the occupied orbitals with index < i after the bit of orbital i has been
 * toggled, as Core/OperatorWaveFunction.cpp:30-43 computes it (bits of byte k above the
 * MSB-first position m, xor-folded with all lower bytes). */
static int qo_parity_below(const uint8_t *det, unsigned i)
{
  unsigned k = i >> 3, m = i & 7, j;
  unsigned acc = (unsigned)(det[k] >> (8 - m)) & 0xFFu;
  if (m == 0) acc = 0;
  for (j = 0; j < k; j++) acc ^= det[j];
  acc ^= acc >> 4;
  acc ^= acc >> 2;
  acc ^= acc >> 1;
  return acc & 1;
}

/* Apply one ladder string to det in place; return the sign (-1, 0, +1).
 * Restates OperatorCr / OperatorAn / OperatorLader (Core/OperatorWaveFunction.cpp:7-115). */
int qo_ladder(uint8_t *det, const uint16_t *o, int len)
{
  int phase = 1, t;
  for (t = 0; t < len; t++) {
    unsigned idx = o[t] & QO_IDX;
    unsigned k = idx >> 3;
    uint8_t bit = (uint8_t)(128u >> (idx & 7));
    if (o[t] & QO_CR) {
      if (det[k] & bit) return 0;
      det[k] |= bit;
    } else {
      if (!(det[k] & bit)) return 0;
      det[k] &= (uint8_t)~bit;
    }
    if (qo_parity_below(det, idx)) phase = -phase;
  }
  return phase;
}

/* Occupation-window filter; restates QDetNotRestricted (Core/OperatorWaveFunction.cpp:2260). */
int qo_restricted_ok(const uint8_t *det, int nword, int nres, const uint8_t *masks,
                     const int *mn, const int *mx)
{
  int r, j;
  for (r = 0; r < nres; r++) {
    int s = 0;
    for (j = 0; j < nword; j++) s += __builtin_popcount((unsigned)(masks[r * nword + j] & det[j]));
    if (s > mx[r] || s < mn[r]) return 0;
  }
  return 1;
}

/* ------------------------------------------------------------------ operator */

typedef struct {
  int nterms;
  const int *len;       /* nterms */
  const int64_t *off;   /* nterms, offset into ops */
  const uint16_t *ops;
  const double *vre, *vim;
} qo_op;

/* ------------------------------------------------------------------ wavefunction */

/* A wavefunction: determinants in insertion order plus an open-addressing index.  The
 * reference keeps a chained hash (Core/Hash.cpp:163 + KeyList/Next); the lookup structure
 * is internal and does not change any result, the insertion order is kept as the
 * reference's (append at N+1, Core/ComplexWaveFunctionArithmetic.cpp:64-190). */
typedef struct {
  int nf, nword;
  int64_t n, cap;
  uint8_t *det;
  double *re, *im;
  int64_t *slot; /* index+1, 0 = empty */
  int64_t hcap;  /* power of two */
} qo_wf;

static uint64_t qo_hash_bytes(const uint8_t *d, int nword)
{
  uint64_t h = 1469598103934665603ull;
  int i;
  for (i = 0; i < nword; i++) { h ^= d[i]; h *= 1099511628211ull; }
  h ^= h >> 29; h *= 0xbf58476d1ce4e5b9ull; h ^= h >> 32;
  return h;
}

qo_wf *qo_wf_new(int nf, int64_t cap)
{
  qo_wf *w = (qo_wf *)calloc(1, sizeof(qo_wf));
  w->nf = nf;
  w->nword = (nf + 7) / 8;
  if (cap < 16) cap = 16;
  w->cap = cap;
  w->det = (uint8_t *)malloc((size_t)cap * w->nword);
  w->re = (double *)malloc(sizeof(double) * cap);
  w->im = (double *)malloc(sizeof(double) * cap);
  w->hcap = 64;
  while (w->hcap < 2 * cap) w->hcap <<= 1;
  w->slot = (int64_t *)calloc((size_t)w->hcap, sizeof(int64_t));
  return w;
}

void qo_wf_free(qo_wf *w)
{
  if (!w) return;
  free(w->det); free(w->re); free(w->im); free(w->slot); free(w);
}

static void qo_rehash(qo_wf *w, int64_t hcap)
{
  int64_t i;
  free(w->slot);
  w->hcap = hcap;
  w->slot = (int64_t *)calloc((size_t)hcap, sizeof(int64_t));
  for (i = 0; i < w->n; i++) {
    uint64_t h = qo_hash_bytes(w->det + i * w->nword, w->nword) & (uint64_t)(hcap - 1);
    while (w->slot[h]) h = (h + 1) & (uint64_t)(hcap - 1);
    w->slot[h] = i + 1;
  }
}

int64_t qo_wf_find(const qo_wf *w, const uint8_t *d)
{
  uint64_t h = qo_hash_bytes(d, w->nword) & (uint64_t)(w->hcap - 1);
  while (w->slot[h]) {
    int64_t i = w->slot[h] - 1;
    if (memcmp(w->det + i * w->nword, d, (size_t)w->nword) == 0) return i;
    h = (h + 1) & (uint64_t)(w->hcap - 1);
  }
  return -1;
}

/* psi += a |d>, appending d if absent (ComplexWaveFunctionAddElement,
 * Core/ComplexWaveFunctionArithmetic.cpp:64). */
void qo_wf_add(qo_wf *w, const uint8_t *d, double are, double aim)
{
  int64_t i = qo_wf_find(w, d);
  uint64_t h;
  if (i >= 0) { w->re[i] += are; w->im[i] += aim; return; }
  if (w->n == w->cap) {
    w->cap *= 2;
    w->det = (uint8_t *)realloc(w->det, (size_t)w->cap * w->nword);
    w->re = (double *)realloc(w->re, sizeof(double) * w->cap);
    w->im = (double *)realloc(w->im, sizeof(double) * w->cap);
  }
  if (2 * (w->n + 1) > w->hcap) qo_rehash(w, w->hcap * 2);
  memcpy(w->det + w->n * w->nword, d, (size_t)w->nword);
  w->re[w->n] = are;
  w->im[w->n] = aim;
  h = qo_hash_bytes(d, w->nword) & (uint64_t)(w->hcap - 1);
  while (w->slot[h]) h = (h + 1) & (uint64_t)(w->hcap - 1);
  w->slot[h] = w->n + 1;
  w->n++;
}

qo_wf *qo_wf_from(int nf, int64_t n, const uint8_t *det, const double *re, const double *im)
{
  qo_wf *w = qo_wf_new(nf, n);
  int64_t i;
  for (i = 0; i < n; i++) qo_wf_add(w, det + i * w->nword, re[i], im[i]);
  return w;
}

int64_t qo_wf_size(const qo_wf *w) { return w->n; }
void qo_wf_get(const qo_wf *w, uint8_t *det, double *re, double *im)
{
  memcpy(det, w->det, (size_t)w->n * w->nword);
  memcpy(re, w->re, sizeof(double) * w->n);
  memcpy(im, w->im, sizeof(double) * w->n);
}

static qo_wf *qo_wf_copy(const qo_wf *a)
{
  qo_wf *w = qo_wf_new(a->nf, a->n);
  memcpy(w->det, a->det, (size_t)a->n * a->nword);
  memcpy(w->re, a->re, sizeof(double) * a->n);
  memcpy(w->im, a->im, sizeof(double) * a->n);
  w->n = a->n;
  qo_rehash(w, w->hcap);
  return w;
}

/* ------------------------------------------------------------------ H*psi */

/* Growing-basis H*psi: every (determinant, term) pair with a non-zero sign adds
 * phase*V*psi_i to the target, appending new targets in visiting order (OperatorPsiCC and
 * OperatorPsiRestrictedCC, Core/OperatorWaveFunction.cpp:1750-1823, :2288-2361).  With
 * nres > 0 targets failing the occupation windows are dropped. */
qo_wf *qo_operator_psi(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                       const double *vre, const double *vim, const qo_wf *psi, int nres,
                       const uint8_t *masks, const int *mn, const int *mx)
{
  qo_wf *out = qo_wf_new(psi->nf, psi->n * 4 + 16);
  uint8_t tmp[64];
  int64_t i;
  int t;
  for (i = 0; i < psi->n; i++) {
    const uint8_t *src = psi->det + i * psi->nword;
    double xr = psi->re[i], xi = psi->im[i];
    for (t = 0; t < nterms; t++) {
      int ph;
      memcpy(tmp, src, (size_t)psi->nword);
      ph = qo_ladder(tmp, ops + off[t], len[t]);
      if (!ph) continue;
      if (nres && !qo_restricted_ok(tmp, psi->nword, nres, masks, mn, mx)) continue;
      qo_wf_add(out, tmp, ph * (vre[t] * xr - vim[t] * xi), ph * (vre[t] * xi + vim[t] * xr));
    }
  }
  return out;
}

/* Fixed-basis H*psi, push form: y on the basis of x, contributions to determinants outside
 * the basis dropped, contributions with |a|^2 < 100*DBL_MIN dropped
 * (OperatorPsiConserveBasisPreAllocatedCC, Core/OperatorWaveFunction.cpp:784-838, and
 * ComplexWaveFunctionAddElementConserveBasis, Core/ComplexWaveFunctionArithmetic.cpp:355-398).
 * OpenMP over source determinants with atomic adds, as the reference.
 * Sources are rows [row0, row1) of x; y (length x->n, interleaved re/im) is overwritten
 * with zeros first. */
void qo_apply_conserve_strided(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                               const double *vre, const double *vim, const qo_wf *x, int64_t row0,
                               int64_t row1, int64_t stride, double *y);
void qo_apply_conserve(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                       const double *vre, const double *vim, const qo_wf *x, int64_t row0,
                       int64_t row1, double *y)
{
  qo_apply_conserve_strided(nterms, len, off, ops, vre, vim, x, row0, row1, 1, y);
}

/* the same over the source rows row0, row0+stride, ... < row1 (a spread sample) */
void qo_apply_conserve_strided(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                               const double *vre, const double *vim, const qo_wf *x, int64_t row0,
                               int64_t row1, int64_t stride, double *y)
{
  int64_t i, cnt = (row1 - row0 + stride - 1) / stride;
  for (i = 0; i < 2 * x->n; i++) y[i] = 0.0;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t c = 0; c < cnt; c++) {
    int64_t i = row0 + c * stride;
    uint8_t tmp[64];
    const uint8_t *src = x->det + i * x->nword;
    double xr = x->re[i], xi = x->im[i];
    int t;
    for (t = 0; t < nterms; t++) {
      int ph;
      int64_t j;
      double ar, ai;
      memcpy(tmp, src, (size_t)x->nword);
      ph = qo_ladder(tmp, ops + off[t], len[t]);
      if (!ph) continue;
      ar = ph * (vre[t] * xr - vim[t] * xi);
      ai = ph * (vre[t] * xi + vim[t] * xr);
      if (ar * ar + ai * ai < 100 * DBL_MIN) continue;
      j = qo_wf_find(x, tmp);
      if (j < 0) continue;
#pragma omp atomic
      y[2 * j] += ar;
#pragma omp atomic
      y[2 * j + 1] += ai;
    }
  }
}

/* Count the (determinant, term) pairs with a non-zero sign whose target lies in the basis,
 * for rows [row0,row1). */
int64_t qo_count_nnz(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                     const qo_wf *x, int64_t row0, int64_t row1)
{
  int64_t i, nnz = 0;
#pragma omp parallel for reduction(+ : nnz) schedule(dynamic, 64)
  for (i = row0; i < row1; i++) {
    uint8_t tmp[64];
    int t;
    for (t = 0; t < nterms; t++) {
      memcpy(tmp, x->det + i * x->nword, (size_t)x->nword);
      if (!qo_ladder(tmp, ops + off[t], len[t])) continue;
      if (qo_wf_find(x, tmp) >= 0) nnz++;
    }
  }
  return nnz;
}

/* Push-form H*psi of nvec vectors at once from the determinants of src into the basis of dst
 * (src == dst: the fixed-basis apply), x [src.n][nvec] and y [dst.n][nvec] complex
 * interleaved, y overwritten.  The same visits as qo_apply_conserve (every (determinant,
 * term) pair, ladder sign, lookup of the target, contributions with |a|^2 < 100*DBL_MIN per
 * vector dropped); the values of the determinant strings that map a source onto itself are
 * summed per source first, so the many diagonal strings cost no atomic adds.  Used for checks
 * of the multi-vector paths on bases of millions of determinants (BlockOperatorPsi,
 * Core/BlockWaveFunctionArithmetic.cpp:1575, runs the reference's loop for each vector). */
void qo_apply_multi(int nterms, const int *len, const int64_t *off, const uint16_t *ops, const double *vre,
                    const double *vim, const qo_wf *src, const qo_wf *dst, int nvec, const double *x, double *y)
{
  int64_t i;
  for (i = 0; i < 2 * dst->n * nvec; i++) y[i] = 0.0;
#pragma omp parallel for schedule(dynamic, 64)
  for (i = 0; i < src->n; i++) {
    uint8_t tmp[64];
    const uint8_t *d = src->det + i * src->nword;
    const double *xi = x + 2 * i * nvec;
    double dre = 0.0, dim = 0.0;
    int t, k, has_diag = 0;
    for (t = 0; t < nterms; t++) {
      int ph;
      int64_t j;
      memcpy(tmp, d, (size_t)src->nword);
      ph = qo_ladder(tmp, ops + off[t], len[t]);
      if (!ph) continue;
      if (src == dst && memcmp(tmp, d, (size_t)src->nword) == 0) {
        dre += ph * vre[t];
        dim += ph * vim[t];
        has_diag = 1;
        continue;
      }
      j = qo_wf_find(dst, tmp);
      if (j < 0) continue;
      for (k = 0; k < nvec; k++) {
        double xr = xi[2 * k], xm = xi[2 * k + 1];
        double ar = ph * (vre[t] * xr - vim[t] * xm), ai = ph * (vre[t] * xm + vim[t] * xr);
        if (ar * ar + ai * ai < 100 * DBL_MIN) continue;
#pragma omp atomic
        y[2 * (j * nvec + k)] += ar;
#pragma omp atomic
        y[2 * (j * nvec + k) + 1] += ai;
      }
    }
    if (has_diag) {
      for (k = 0; k < nvec; k++) {
        double xr = xi[2 * k], xm = xi[2 * k + 1];
        double ar = dre * xr - dim * xm, ai = dre * xm + dim * xr;
#pragma omp atomic
        y[2 * (i * nvec + k)] += ar;
#pragma omp atomic
        y[2 * (i * nvec + k) + 1] += ai;
      }
    }
  }
}

/* the same over the source rows row0, row0+stride, ... < row1 (a spread sample) */
int64_t qo_count_nnz_strided(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                             const qo_wf *x, int64_t row0, int64_t row1, int64_t stride)
{
  int64_t c, cnt = (row1 - row0 + stride - 1) / stride, nnz = 0;
#pragma omp parallel for reduction(+ : nnz) schedule(dynamic, 64)
  for (c = 0; c < cnt; c++) {
    uint8_t tmp[64];
    int64_t i = row0 + c * stride;
    int t;
    for (t = 0; t < nterms; t++) {
      memcpy(tmp, x->det + i * x->nword, (size_t)x->nword);
      if (!qo_ladder(tmp, ops + off[t], len[t])) continue;
      if (qo_wf_find(x, tmp) >= 0) nnz++;
    }
  }
  return nnz;
}

/* ------------------------------------------------------------------ vector algebra */

double qo_norm(const qo_wf *a)
{ /* ComplexWaveFunctionCalculateNorm, Core/ComplexWaveFunctionArithmetic.cpp:870 */
  double s = 0;
  int64_t i;
  for (i = 0; i < a->n; i++) s += a->re[i] * a->re[i] + a->im[i] * a->im[i];
  return sqrt(s);
}

void qo_scale(qo_wf *a, double f)
{ /* ComplexWaveFunctionMultiply by a real factor */
  int64_t i;
  for (i = 0; i < a->n; i++) { a->re[i] *= f; a->im[i] *= f; }
}

/* <a|b>, conjugating a (ComplexWaveFunctionDotProduct, Core/ComplexWaveFunctionArithmetic.cpp:991) */
void qo_dot(const qo_wf *a, const qo_wf *b, double *dre, double *dim)
{
  double sr = 0, si = 0;
  int64_t i;
  for (i = 0; i < a->n; i++) {
    int64_t j = qo_wf_find(b, a->det + i * a->nword);
    if (j < 0) continue;
    sr += a->re[i] * b->re[j] + a->im[i] * b->im[j];
    si += a->re[i] * b->im[j] - a->im[i] * b->re[j];
  }
  *dre = sr;
  *dim = si;
}

/* a += f*b on the union basis (ComplexWaveFunctionAddMultipliedUnionBasis, :601) */
void qo_axpy_union(qo_wf *a, const qo_wf *b, double fre, double fim)
{
  int64_t i;
  for (i = 0; i < b->n; i++)
    qo_wf_add(a, b->det + i * b->nword, fre * b->re[i] - fim * b->im[i], fre * b->im[i] + fim * b->re[i]);
}

/* drop |a_i|^2 <= eps^2, keeping order (ComplexWaveFunctionTruncateBasis, :1073-1113) */
void qo_truncate(qo_wf *a, double eps)
{
  double e2 = eps * eps;
  int64_t i, k = 0;
  for (i = 0; i < a->n; i++) {
    if (a->re[i] * a->re[i] + a->im[i] * a->im[i] > e2) {
      if (k != i) {
        memcpy(a->det + k * a->nword, a->det + i * a->nword, (size_t)a->nword);
        a->re[k] = a->re[i];
        a->im[k] = a->im[i];
      }
      k++;
    }
  }
  a->n = k;
  qo_rehash(a, a->hcap);
}

/* ------------------------------------------------------------------ Lanczos */

/* Three-term Lanczos tridiagonalisation on a growing basis with the reference's truncation
 * schedule (LanczosTriDiagonalizeCC, Core/Lanczos.cpp:2169-2263):
 *   a[0] = 0, b[0] = |psi|, v0 = psi/b0 truncated at eps;
 *   v1 = H v0, a[1] = <v0|H|v0>;
 *   for i = 1..ntri-1: v_i -= a_i v_{i-1}; b_i = |v_i|; v_i /= b_i; truncate at eps/err;
 *                      err *= b_i^2/(b_i^2 + 4 gamma^2); w = H v_i; a_{i+1} = <v_i|w>;
 *                      w -= b_i v_{i-1}.
 * a has ntri+1 entries, b has ntri.  Restrictions (nres > 0) filter every H*v. */
void qo_lanczos_tridiag(int nterms, const int *len, const int64_t *off, const uint16_t *ops,
                        const double *vre, const double *vim, const qo_wf *psi, int ntri,
                        double eps, double gamma, int nres, const uint8_t *masks, const int *mn,
                        const int *mx, double *a, double *b)
{
  qo_wf *v[3];
  double err = 1.0, junk;
  int i;
  v[0] = qo_wf_copy(psi);
  v[1] = v[2] = NULL;
  a[0] = 0;
  b[0] = qo_norm(v[0]);
  qo_scale(v[0], 1.0 / b[0]);
  qo_truncate(v[0], eps);
  v[1] = qo_operator_psi(nterms, len, off, ops, vre, vim, v[0], nres, masks, mn, mx);
  qo_dot(v[1], v[0], &a[1], &junk);
  for (i = 1; i < ntri; i++) {
    int vip = (i + 1) % 3, vi = i % 3, vim_ = (i - 1) % 3;
    qo_axpy_union(v[vi], v[vim_], -a[i], 0.0);
    b[i] = qo_norm(v[vi]);
    qo_scale(v[vi], 1.0 / b[i]);
    qo_truncate(v[vi], eps / err);
    err *= b[i] * b[i] / (b[i] * b[i] + 4 * gamma * gamma);
    qo_wf_free(v[vip]);
    v[vip] = qo_operator_psi(nterms, len, off, ops, vre, vim, v[vi], nres, masks, mn, mx);
    qo_dot(v[vip], v[vi], &a[i + 1], &junk);
    qo_axpy_union(v[vip], v[vim_], -b[i], 0.0);
  }
  qo_wf_free(v[0]);
  qo_wf_free(v[1]);
  qo_wf_free(v[2]);
}

/* ------------------------------------------------------------------ continued fraction */

/* G(w_k) for w_k = emin + k*de + e0, k = 0..ne, with Gamma/2 imaginary shift:
 * G = a0 + b0^2 / (w - a1 + i g/2 - b1^2 / (w - a2 + i g/2 - ...)), evaluated from the
 * bottom as TriDiagonalMatrixToSpectrum does (Core/Spectral.cpp:1433-1473).  a has n+1
 * entries, b has n. */
void qo_cf_spectrum(int n, const double *a, const double *b, double e0, double emin, double de,
                    int ne, double gamma, double *gre, double *gim)
{
  int k, j;
  for (k = 0; k <= ne; k++) {
    double w = (double)k * de + emin + e0;
    double den = (gamma * 0.5) * (gamma * 0.5) + (w - a[n]) * (w - a[n]);
    double vr = (w - a[n]) / den, vi = (-gamma * 0.5) / den;
    for (j = (n > 1 ? n : 1) - 1; j >= 1; j--) {
      double b2 = b[j] * b[j];
      double zr = w - a[j] - vr * b2, zi = gamma * 0.5 - vi * b2;
      den = zi * zi + zr * zr;
      vr = zr / den;
      vi = (vi * b2 - gamma * 0.5) / den;
    }
    gre[k] = a[0] + vr * b[0] * b[0];
    gim[k] = vi * b[0] * b[0];
  }
}

int qo_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ enumeration */

/* All determinants on nf orbitals with exactly nel electrons that satisfy the occupation
 * windows (nres masks in the reference byte layout), in lexicographic order of the
 * determinant string (orbital 0 first, '1' before '0' reversed: ascending binary).  Depth-first
 * over orbitals with pruning on every window.  Returns a malloc'd n*nword byte array. */
typedef struct {
  int nf, nword, nres, nel;
  const uint8_t *masks;
  const int *mn, *mx;
  int *cnt;      /* electrons so far per window */
  int *left;     /* [orbital][window]: mask orbitals at index >= orbital */
  uint8_t *cur;
  uint8_t *out;
  int64_t n, cap;
} qo_enum_state;

static int qo_in(const uint8_t *m, int i) { return (m[i >> 3] & (128 >> (i & 7))) != 0; }

static void qo_enum_rec(qo_enum_state *s, int i, int ne)
{
  int r, ok;
  if (ne > s->nel || ne + (s->nf - i) < s->nel) return;
  for (r = 0; r < s->nres; r++) {
    if (s->cnt[r] > s->mx[r]) return;
    if (s->cnt[r] + s->left[i * s->nres + r] < s->mn[r]) return;
  }
  if (i == s->nf) {
    if (s->n == s->cap) {
      s->cap = s->cap ? 2 * s->cap : 1024;
      s->out = (uint8_t *)realloc(s->out, (size_t)s->cap * s->nword);
    }
    memcpy(s->out + s->n * s->nword, s->cur, (size_t)s->nword);
    s->n++;
    return;
  }
  /* orbital i empty first, then occupied: ascending order of the reversed-bit key */
  qo_enum_rec(s, i + 1, ne);
  ok = 1;
  for (r = 0; r < s->nres; r++)
    if (qo_in(s->masks + r * s->nword, i)) s->cnt[r]++;
  s->cur[i >> 3] |= (uint8_t)(128 >> (i & 7));
  if (ok) qo_enum_rec(s, i + 1, ne + 1);
  s->cur[i >> 3] &= (uint8_t)~(128 >> (i & 7));
  for (r = 0; r < s->nres; r++)
    if (qo_in(s->masks + r * s->nword, i)) s->cnt[r]--;
}

uint8_t *qo_enumerate(int nf, int nel, int nres, const uint8_t *masks, const int *mn, const int *mx, int64_t *n_out)
{
  qo_enum_state s;
  int i, r;
  memset(&s, 0, sizeof(s));
  s.nf = nf;
  s.nword = (nf + 7) / 8;
  s.nres = nres;
  s.nel = nel;
  s.masks = masks;
  s.mn = mn;
  s.mx = mx;
  s.cnt = (int *)calloc((size_t)(nres > 0 ? nres : 1), sizeof(int));
  s.left = (int *)calloc((size_t)(nf + 1) * (nres > 0 ? nres : 1), sizeof(int));
  s.cur = (uint8_t *)calloc((size_t)s.nword, 1);
  for (i = nf - 1; i >= 0; i--)
    for (r = 0; r < nres; r++) s.left[i * nres + r] = s.left[(i + 1) * nres + r] + qo_in(masks + r * s.nword, i);
  qo_enum_rec(&s, 0, 0);
  free(s.cnt);
  free(s.left);
  free(s.cur);
  *n_out = s.n;
  return s.out;
}

void qo_free(void *p) { free(p); }

/* ------------------------------------------------------------------ Krylov-basis Lanczos */

/* Lanczos that keeps its Krylov vectors (LanczosTriDiagonalizeKrylovCC and the restricted
 * variant, Core/Lanczos.cpp:3705-3858): every new vector H K_{i-1} is orthogonalised against
 * all earlier ones by modified Gram-Schmidt in reverse order (a_i from the overlap with
 * K_{i-1}), normalised (zeroed when b_i < 100*DBL_MIN), zeroed when the summed squared
 * overlaps after normalisation exceed eps, and truncated at eps/err with
 * err *= b^2/(b^2 + DBL_MIN + DBL_EPSILON a^2).  a[ntri] = <K_{ntri-1}|H|K_{ntri-1}>.
 * K receives ntri handles (caller frees them). */
void qo_lanczos_krylov(int nterms, const int *len, const int64_t *off, const uint16_t *ops, const double *vre,
                       const double *vim, const qo_wf *psi, int ntri, double eps, int nres, const uint8_t *masks,
                       const int *mn, const int *mx, double *a, double *b, qo_wf **K)
{
  double err = 1.0;
  int i, j;
  K[0] = qo_wf_copy(psi);
  a[0] = 0;
  b[0] = qo_norm(K[0]);
  qo_scale(K[0], b[0] < 100 * DBL_MIN ? 0.0 : 1.0 / b[0]);
  qo_truncate(K[0], eps / err);
  for (i = 1; i < ntri; i++) {
    double temp = 0;
    K[i] = qo_operator_psi(nterms, len, off, ops, vre, vim, K[i - 1], nres, masks, mn, mx);
    for (j = i; j > 0;) {
      double dr, di;
      j--;
      qo_dot(K[j], K[i], &dr, &di);
      if (j == i - 1) a[i] = dr;
      qo_axpy_union(K[i], K[j], -dr, -di);
    }
    b[i] = qo_norm(K[i]);
    qo_scale(K[i], b[i] < 100 * DBL_MIN ? 0.0 : 1.0 / b[i]);
    for (j = i; j > 0;) {
      double dr, di;
      j--;
      qo_dot(K[j], K[i], &dr, &di);
      temp += dr * dr + di * di;
      if (temp > eps) {
        qo_scale(K[i], 0.0);
        break;
      }
    }
    err *= b[i] * b[i] / (b[i] * b[i] + DBL_MIN + DBL_EPSILON * a[i] * a[i]);
    qo_truncate(K[i], eps / err);
  }
  {
    qo_wf *hk = qo_operator_psi(nterms, len, off, ops, vre, vim, K[ntri - 1], nres, masks, mn, mx);
    double dr, di;
    qo_dot(K[ntri - 1], hk, &dr, &di);
    a[ntri] = dr;
    qo_wf_free(hk);
  }
}
