/*
 * qgpu.h -- C ABI of the GB300 (sm_103a) engine for second-quantized operators acting on
 * Slater-determinant wavefunctions, and the Lanczos / block-Lanczos / continued-fraction
 * iterations built on it.
 *
 * Every entry point is plain C: pointers, sizes and handles; no C++ or torch types.  Each
 * returns a qg_status (0 = ok), the reference's convention of a uint32_t status where 1 means
 * "out of memory" (Core/Lanczos.cpp:2196-2206 retries on it).  Pointers named *_dev are
 * device pointers (cudaMalloc or any allocator); *_host are host pointers.  All work is
 * issued on the context's CUDA stream; functions that return host data synchronise it.
 *
 * Layout at the boundary is the reference's:
 *   - a determinant is NWord = ceil(nf/8) bytes, orbital i in byte i>>3 under mask
 *     128>>(i&7) (Core/OperatorWaveFunction.cpp:7-43, Core/WaveFunctionArithmetic.cpp:130);
 *   - an operator term is a ladder string o[0..len-1], o[0] acting first, bit 15 set for a
 *     creation operator (CrAnMask, Core/StructDef.cpp:46; Core/OperatorWaveFunction.cpp:98);
 *   - amplitudes are complex FP64, interleaved (re, im) -- the reference's ValueRe/ValueIm
 *     pair (Core/StructDef.cpp:188-206) without the 2^14 blocking and without the unused
 *     element 0 (Core/StructDef.cpp:33-42, :184-187).
 * A multi-vector block stores vector k of determinant r at [r * nvec + k].
 */
#ifndef QGPU_H
#define QGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  QG_OK = 0,
  QG_ERR_OOM = 1,        /* allocation failed (reference: return 1 -> truncate and retry) */
  QG_ERR_TABLE_FULL = 2, /* a device hash table ran out of room; the caller may retry */
  QG_ERR_TIMEOUT = 3,    /* a bounded device wait or probe gave up */
  QG_ERR_ARG = 4,        /* bad argument (unsupported size, null pointer, mismatch) */
  QG_ERR_CUDA = 5,       /* CUDA runtime error; qg_last_error() has the text */
  QG_ERR_NOT_HERMITIAN = 6
} qg_status;

typedef struct qg_context_s *qg_context;
typedef struct qg_operator_s *qg_operator;
typedef struct qg_basis_s *qg_basis;

/* Occupation windows on orbital subsets (DeterminantRestrictionType,
 * Core/StructDef.cpp:211-221): for each r < n the number of occupied orbitals under
 * masks[r*nword .. r*nword+nword-1] must lie in [min[r], max[r]]
 * (QDetNotRestricted, Core/OperatorWaveFunction.cpp:2260). */
typedef struct {
  int32_t n;
  const uint8_t *masks; /* n * nword bytes, reference byte layout */
  const int32_t *min;
  const int32_t *max;
} qg_restrictions;

/* ------------------------------------------------------------------ context */

/* One context per host thread (the reference is called from the single Lua thread). */
qg_status qg_init(int device, qg_context *ctx);
qg_status qg_finalize(qg_context ctx);
/* stream: a cudaStream_t cast to void*; NULL selects the context's own stream. */
qg_status qg_set_stream(qg_context ctx, void *stream);
void *qg_get_stream(qg_context ctx);
const char *qg_last_error(qg_context ctx);
/* Number of kernels this library launched on the context since qg_init (for accounting). */
int64_t qg_launch_count(qg_context ctx);
qg_status qg_synchronize(qg_context ctx);

/* ------------------------------------------------------------------ operators */

/* Upload an operator: nterms ladder strings (lengths term_len[], codes concatenated in ops[])
 * with complex values.  Replaces the OperatorType the reference's dispatchers receive
 * (Core/StructDef.cpp:223-249) as built by NewOperator (LuaInterface/ssp.cpp:572).  Terms
 * that annihilate twice or create twice on the same orbital are dropped (they vanish on
 * every determinant).  nf <= 127. */
qg_status qg_operator_create(qg_context ctx, int32_t nf, int32_t nterms, const int32_t *term_len,
                             const uint16_t *ops, const double *v_re, const double *v_im,
                             qg_operator *op);
qg_status qg_operator_destroy(qg_operator op);
/* Counts after upload: kept terms, distinct annihilation groups, and whether the term list is
 * closed under Hermitian conjugation with conjugated values (QOperatorHermitian,
 * Core/OperatorArithmetic.cpp:6517; 1 = Hermitian within 1e-12 relative). */
qg_status qg_operator_info(qg_operator op, int32_t *nterms, int32_t *ngroups, int32_t *hermitian);

/* Parameter scans: H = sum_k p_k O_k over already uploaded operators (all on the same nf),
 * the reference's operator sum and scalar product (OperatorAdd, Core/OperatorArithmetic.cpp:5674,
 * after NormalOrderOperator, :1607), kept on the device so that a scan does not rebuild it.
 * The sum operator holds the union of the components' terms -- zero values included, so its
 * structure does not depend on the coefficients -- and each term's contribution per
 * component.  qg_operator_set_coefficients(op, p) recomputes the values in place (ordered on
 * the context's stream after the work already queued); bases keep their per-operator caches
 * (local blocks, connection lists) and only refresh the values on their next use.  A term
 * whose value is zero reaches no determinant in basis growth (the reference holds no zero
 * terms).  coef_im may be NULL (real coefficients).  The components may be destroyed
 * afterwards; set_coefficients returns QG_ERR_ARG for an operator that is not a sum. */
qg_status qg_operator_create_sum(qg_context ctx, int32_t ncomp, const qg_operator *components,
                                 const double *coef_re, const double *coef_im, qg_operator *op);
qg_status qg_operator_set_coefficients(qg_operator op, const double *coef_re, const double *coef_im);

/* ------------------------------------------------------------------ bases */

/* Build a basis from n determinants (reference byte layout, n * ceil(nf/8) bytes, host
 * memory).  Duplicates are merged.  The basis is kept sorted on the device (its own order);
 * perm_host (optional, n entries) receives for each input determinant its index in the
 * basis.  This is the determinant + hash part of WaveFunctionType
 * (Core/StructDef.cpp:188-206, Core/Hash.cpp:163). */
qg_status qg_basis_create(qg_context ctx, int32_t nf, int64_t n, const uint8_t *dets_host,
                          qg_basis *basis, int64_t *perm_host);
qg_status qg_basis_destroy(qg_basis basis);
int64_t qg_basis_size(qg_basis basis);
/* Copy the basis determinants out in reference byte layout (host, size * nword bytes). */
qg_status qg_basis_get_dets(qg_basis basis, uint8_t *dets_host);
/* Index of each of n determinants in the basis (-1 if absent); host in, host out. */
qg_status qg_basis_find(qg_basis basis, int64_t n, const uint8_t *dets_host, int64_t *index_host);

/* Targets of op on the determinants of basis_in: every determinant reached with a non-zero
 * sign by some term (and passing the restrictions, if any).  This is the basis OperatorPsi
 * builds (Core/OperatorWaveFunction.cpp:1750-1823; :2288-2361 with restrictions;
 * dispatchers :5573, :5598); the amplitudes follow from qg_apply(op, out, basis_in, ...).
 * Device open-addressing hash with atomicCAS insert. */
qg_status qg_operator_psi_basis(qg_context ctx, qg_operator op, qg_basis basis_in,
                                const qg_restrictions *res, qg_basis *basis_out);

/* Closure of a seed basis under repeated application of op (breadth first, device hash),
 * within the restrictions: the basis the reference's growing Lanczos / BlockGroundState
 * loops reach (Core/Lanczos.cpp:2169-2263 grows one H*psi per step;
 * Core/BlockLanczos.cpp:5843-5884 grows until converged).  max_rounds < 0 means until
 * closed; rounds_done receives the number of expansion rounds made. */
qg_status qg_basis_closure(qg_context ctx, qg_operator op, qg_basis seed, const qg_restrictions *res,
                           int32_t max_rounds, qg_basis *closed, int32_t *rounds_done);

/* Union of two bases on the same orbitals (ComplexWaveFunctionAddMultipliedUnionBasis's
 * basis, Core/ComplexWaveFunctionArithmetic.cpp:601). */
qg_status qg_basis_union(qg_context ctx, qg_basis a, qg_basis b, qg_basis *out);

/* Re-index amplitudes between bases: y[rows of dst] = x[rows of src] for determinants present
 * in both, zero elsewhere (nvec vectors, device pointers). */
qg_status qg_basis_map(qg_context ctx, qg_basis src, const double *x_dev, qg_basis dst, double *y_dev,
                       int32_t nvec);

/* ------------------------------------------------------------------ H * psi */

/* y = op x with x on basis_src and y on basis_dst (nvec vectors each), pull form: every row
 * of y gathers its sources through the adjoint ladder strings, so no float atomics are
 * used.  With basis_dst == basis_src this is OperatorPsiConserveBasisPreAllocated
 * (Core/OperatorWaveFunction.cpp:784-1127, dispatcher :5541): contributions whose source
 * lies outside the basis are absent.  With basis_dst = qg_operator_psi_basis(op, basis_src)
 * it gives the amplitudes of OperatorPsi (:1750, dispatcher :5598).  The multi-vector form is
 * BlockOperatorPsi (Core/BlockWaveFunctionArithmetic.cpp:1575). */
qg_status qg_apply(qg_context ctx, qg_operator op, qg_basis basis_dst, qg_basis basis_src,
                   const double *x_dev, double *y_dev, int32_t nvec);

/* ------------------------------------------------------------------ dense path (small bases) */

/* op as a dense matrix on a basis (OperatorToDeterminantMatrix, Core/MatrixOperator.cpp:1149):
 * m_host receives n x n complex values row-major interleaved, m[r][c] = <r|op|c>.  n <= 16384;
 * the reference takes this path below DenseBorder = 1513 determinants. */
qg_status qg_operator_dense(qg_context ctx, qg_operator op, qg_basis basis, double *m_host);

/* Spectra from lists of poles (ListOfPolesToSpectrum, Core/Spectral.cpp:1516, Gamma > 0):
 * G_s(w) = sum_k b[s][k] / (w - a[s][k] + i gamma/2) at w = emin + k*de + e0[s], k = 0..ne;
 * a_host, b_host nspec x npole row-major; g_host nspec*(ne+1) complex (interleaved). */
qg_status qg_poles_spectra(qg_context ctx, int32_t nspec, int32_t npole, const double *a_host,
                           const double *b_host, const double *e0_host, double emin, double de,
                           int32_t ne, double gamma, double *g_host);

/* Eigenpairs of a dense Hermitian matrix, computed on the device: up to k = 40 by cyclic Jacobi
 * in one block (round-robin ordering: every step rotates k/2 disjoint index pairs at once);
 * above, by Householder reduction to a real tridiagonal matrix, eigenvalues by multisection on
 * Sturm counts, eigenvectors by inverse iteration and the reflectors (k <= 12000).  a_host is
 * k x k row-major with interleaved (re, im); w_host receives all k eigenvalues ascending, v_host
 * (k x nv row-major, interleaved) the eigenvectors of the lowest nv as columns.  Replaces the
 * reference's zheevd calls on dense and projected matrices (Core/BlockLanczos.cpp:5530, :370-501;
 * HermitianCompactMatrixToListOfPoles, Core/BasicMath/BasicMath_CompactMatrixVector.cpp:3990).
 * QG_ERR_TIMEOUT if the Jacobi rotations have not converged after 60 sweeps, QG_ERR_ARG above
 * k = 12000. */
qg_status qg_hermitian_eigh(qg_context ctx, int32_t k, const double *a_host, double *w_host, double *v_host,
                            int32_t nv);

/* Autotuning of the multi-vector apply (no counterpart in the reference, whose loops handle one
 * vector at a time): the first apply of an operator with nvec >= 2 vectors on a basis (as
 * its own source and target, outside stream capture) times each number of vectors handled per
 * kernel pass and keeps the fastest for that (operator, basis, nvec): a thread per row carrying
 * 8, 4, 3, 2 or 1 vectors per pass, or (nvec >= 16) a warp per row with its lanes over 32 or 64
 * vectors per pass (chunk -32, -64).  Every choice sums each vector's connections in the same
 * order, so the result is bitwise the same.  qg_set_autotune(ctx, 0) turns the timing off
 * (passes of 8 vectors); qg_apply_chunk reports the choice in force (0 while none has been
 * made); qg_apply_set_chunk pins one. */
qg_status qg_set_autotune(qg_context ctx, int32_t on);
qg_status qg_apply_chunk(qg_context ctx, qg_operator op, qg_basis basis, int32_t nvec, int32_t *chunk);
qg_status qg_apply_set_chunk(qg_context ctx, qg_operator op, qg_basis basis, int32_t nvec, int32_t chunk);

/* Connection lists of the same-basis apply (no counterpart in the reference, which looks every
 * connection up in its hash on every H*psi, ComplexWaveFunctionAddElementConserveBasis,
 * Core/ComplexWaveFunctionArithmetic.cpp:355): on the first apply of an operator on a basis
 * (outside stream capture) the sources that need a hash lookup are resolved once into
 * per-row lists of source rows (8 bytes per connection, 8 per row), and later applies gather
 * by row.  The lists keep each row's summation order, so the result is bitwise the same as
 * the hash path.  They are not built when they would take more than a quarter of the free
 * device memory or the basis has 2^32 - 1 rows or more.  on = 0 turns them off for lists not
 * yet built; qg_apply_list_info reports whether (op, basis) has them (built = 1) and their
 * connection count. */
qg_status qg_set_connection_lists(qg_context ctx, int32_t on);
qg_status qg_apply_list_info(qg_context ctx, qg_operator op, qg_basis basis, int32_t *built, int64_t *nconn);

/* FP64 operations of one single-vector same-basis apply of op on basis (no counterpart in the
 * reference): per row 2 multiplies for a real diagonal (4 complex), per connection 2 FMAs for
 * a real value (4 complex), counted over the connection lists (built here if needed;
 * QG_ERR_ARG when they cannot be).  The exact work behind the apply's FP64 ceiling. */
qg_status qg_apply_fp64_ops(qg_context ctx, qg_operator op, qg_basis basis, int64_t *ops);

/* qg_apply with host buffers: copies x_host to the device, applies, copies y back (the
 * reference's calling convention, where psi and Opsi live in host memory).  Device staging
 * buffers are kept in the context between calls.  Page-locked (pinned) buffers are used in
 * place: the SMs pull x over the host link, and the apply writes y straight into y_host, so
 * the copy back overlaps the computation; pageable buffers are staged with copies. */
qg_status qg_apply_host(qg_context ctx, qg_operator op, qg_basis basis_dst, qg_basis basis_src,
                        const double *x_host, double *y_host, int32_t nvec);

/* Number of non-zero (row, term) connections of qg_apply(op, b, b) (sources inside b), and
 * the same count without the diagonal (flip == 0) connections. */
qg_status qg_count_nnz(qg_context ctx, qg_operator op, qg_basis basis, int64_t *nnz);
qg_status qg_count_nnz_offdiag(qg_context ctx, qg_operator op, qg_basis basis, int64_t *nnz);
/* The same count over the rows row0, row0 + stride, ... of the basis only (offdiag != 0: without
 * the diagonal connections), for checks on a spread sample of a large basis.  For a Hermitian
 * term list this equals the reference's count of the pairs its push loop visits from those
 * determinants as sources (Core/OperatorWaveFunction.cpp:784-838). */
qg_status qg_count_nnz_rows(qg_context ctx, qg_operator op, qg_basis basis, int64_t row0, int64_t stride,
                            int32_t offdiag, int64_t *nnz);

/* <psi|op|psi> for nvec vectors on one basis, complex result per vector (host out)
 * (PsiOperatorPsi / PsiHermitianOperatorPsi, Core/OperatorWaveFunction.cpp:5680, :5710). */
qg_status qg_expectation(qg_context ctx, qg_operator op, qg_basis basis, const double *x_dev,
                         int32_t nvec, double *val_host);

/* ------------------------------------------------------------------ vector algebra */

/* <x_k|y_k> per vector (conjugating x; ComplexWaveFunctionDotProductSameBasis,
 * Core/ComplexWaveFunctionArithmetic.cpp:961), host out, 2*nvec doubles. */
qg_status qg_dot(qg_context ctx, int64_t n, int32_t nvec, const double *x_dev, const double *y_dev,
                 double *dot_host);
/* ||x_k|| per vector (ComplexWaveFunctionCalculateNorm, :870), host out. */
qg_status qg_norm(qg_context ctx, int64_t n, int32_t nvec, const double *x_dev, double *norm_host);
/* y_k += alpha_k x_k (alpha complex per vector, host; ...AddComplexMultipliedSameBasis :541). */
qg_status qg_axpy(qg_context ctx, int64_t n, int32_t nvec, const double *alpha_host, const double *x_dev,
                  double *y_dev);

/* qg_dot for callers that cannot allocate device memory (no counterpart in the reference,
 * which has no GPU): per-vector <x_k|y_k> of nvec vectors of n complex entries (device
 * pointers) into out_dev (nvec complex values, device memory), on the given CUDA stream
 * (NULL = legacy default stream).  It takes no context: it runs on the calling thread's
 * current device (cudaGetDevice), to which the pointers and the stream must belong.  It calls
 * no cudaMalloc/cudaFree: the block partial sums
 * live in a fixed device array inside the library (1 MiB per device), so nvec is limited to
 * 64 (larger values return QG_ERR_ARG).  The first call on a device looks up that array's
 * address and should come before any stream capture.  All calls on a device share the
 * array: calls that may overlap on the GPU race and must be ordered by the caller. */
qg_status qg_dot_noalloc(int64_t n, int32_t nvec, const double *x_dev, const double *y_dev, double *out_dev,
                         void *stream);

/* ------------------------------------------------------------------ Krylov drivers */

/* Three-term Lanczos tridiagonalisation of op from nvec starting vectors at once (all on
 * one basis), NTri steps, the reference's truncation schedule (drop |v|<=eps/err with
 * err *= b^2/(b^2+4 gamma^2)) applied as zeroing on the fixed basis; no reorthogonalisation
 * (LanczosTriDiagonalize{RC,CC,MC,RR} and the Restricted variants, Core/Lanczos.cpp:1905-2830,
 * dispatchers :5228, :5274).  v0_dev is not modified.  a_host receives nvec*(ntri+1)
 * entries (vector k at [k*(ntri+1)], a[0] = 0), b_host nvec*ntri (b[0] = |v0_k|).
 * krylov_dev (optional, ntri * n * nvec complex) receives the normalised Krylov vectors
 * (LanczosTriDiagonalizeKrylov, :5405). */
qg_status qg_lanczos_tridiag(qg_context ctx, qg_operator op, qg_basis basis, const double *v0_dev,
                             int32_t nvec, int32_t ntri, double eps, double gamma, double *a_host,
                             double *b_host, double *krylov_dev);

/* Bases of at most 2048 determinants whose rows hold at most 32768 terms run
 * qg_lanczos_tridiag as one persistent kernel, one block per vector with the whole recursion
 * on chip; each vector's coefficients are bitwise those of the general path run with that
 * vector alone.  on = 0 keeps every call on the general path (default 1). */
qg_status qg_set_small_basis_lanczos(qg_context ctx, int32_t on);

/* With a real operator (every value real), start vectors whose imaginary or real part is zero
 * are real Lanczos chains (the reference's real-vector variants, LanczosTriDiagonalizeRR,
 * Core/Lanczos.cpp:1905-2830), and qg_lanczos_tridiag runs them two per complex vector (real
 * and imaginary parts), one apply serving both; each chain's coefficients equal those of its
 * run alone (bitwise for a single pair, to rounding otherwise).  on = 0 runs every vector as
 * complex (default 1). */
qg_status qg_set_split_chains(qg_context ctx, int32_t on);

/* Continued fraction G_s(w_k) = a0 + b0^2/(w - a1 + i g/2 - b1^2/(...)) for nspec spectra
 * and w_k = emin + k*de + e0[s], k = 0..ne, in one kernel (TriDiagonalMatrixToSpectrum,
 * Core/Spectral.cpp:1433).  Spectrum s uses a[s*(ntri+1) ..], b[s*ntri ..]; host in; g_host
 * receives nspec*(ne+1) complex values (interleaved). */
qg_status qg_cf_spectra(qg_context ctx, int32_t nspec, int32_t ntri, const double *a_host,
                        const double *b_host, const double *e0_host, double emin, double de,
                        int32_t ne, double gamma, double *g_host);

/* Lowest nvec eigenpairs of a Hermitian op on a fixed basis by restarted block (band)
 * Lanczos with full reorthogonalisation (BlockLanczosGroundStateConserveBasis,
 * Core/BlockLanczos.cpp:5707, its Krylov solver :5350).  x_dev holds nvec start vectors
 * on input (n * nvec) and the eigenvectors on output; energies_host nvec doubles.
 * tol is the reference's "Zero" (variance convergence); max_krylov caps the Krylov space,
 * which starts at nvec + 100 vectors and grows by nvec + 10 per restart (NKrylovStart,
 * NKrylovStep).  For nvec > 3 up to min(nvec/2, 8) guard vectors join the block; only the
 * nvec wanted states must converge. */
qg_status qg_block_groundstate(qg_context ctx, qg_operator op, qg_basis basis, int32_t nvec,
                               double *x_dev, double *energies_host, double tol, int32_t max_krylov,
                               int32_t max_restarts, int32_t *iterations);

/* Lanczos that keeps its Krylov vectors, with the reference's full modified Gram-Schmidt
 * reorthogonalisation and orthogonality test (LanczosTriDiagonalizeKrylovCC,
 * Core/Lanczos.cpp:3705-3858).  One start vector; krylov_dev receives ntri * n complex values
 * (vector-major); a_host ntri+1, b_host ntri. */
qg_status qg_lanczos_krylov(qg_context ctx, qg_operator op, qg_basis basis, const double *v0_dev, int32_t ntri,
                            double eps, double *a_host, double *b_host, double *krylov_dev);

/* Block Lanczos tridiagonalisation of op from m start vectors (v0_dev, n x m row-major on one
 * basis), NTri blocks (LanczosBlockTriDiagonalize{RR,RC,CC}, Core/BlockLanczos.cpp:1647-2660, as
 * CreateSpectra with Tensor = true calls it, LuaInterface/ssp.cpp:2753-2800): Loewdin
 * orthonormalisation with the reference's deflation (a direction whose singular value is not
 * above max(singular_value, 3 sqrt(DBL_EPSILON) s_max) is dropped), two projections against
 * each of the last two blocks, entries below eps zeroed.  a_host receives (ntri + 1) blocks
 * and b_host ntri blocks of m x m complex values (interleaved, row-major, zero beyond a
 * deflated block's size; a_0 = 0, b_0(i, j) = <q_j|v0_i>, A_k = Q_k^H H Q_k,
 * B_k = Q_k^H H Q_{k+1}); sizes_host (ntri + 1) the block sizes (sizes[0] = m).  krylov_dev
 * (optional, ntri * m * n complex) receives the blocks Q_1 .. Q_ntri as Krylov vectors,
 * vector (k - 1) * m + c at [((k - 1) * m + c) * n], zero beyond a block's size
 * (LanczosBlockTriDiagonalizeKrylov, Core/BlockLanczos.cpp:3649ff). */
qg_status qg_block_lanczos(qg_context ctx, qg_operator op, qg_basis basis, const double *v0_dev, int32_t m,
                           int32_t ntri, double eps, double singular_value, double *a_host, double *b_host,
                           int32_t *sizes_host, double *krylov_dev);

/* Dense complex block products on device arrays (row-major, complex interleaved), by the
 * library's own FP64 kernels (no BLAS): C (ka x kb) = A^H B over n rows, and
 * X (n x kb) = beta X + alpha A M with M ka x kb.  They replace the reference's BLAS products
 * of eigenvector matrices in the dense RIXS branch (ResonantSpectraDense,
 * Core/ResonantSpectra.cpp:290-660). */
qg_status qg_block_adjoint_product(qg_context ctx, const double *A_dev, int32_t lda, int32_t ka,
                                   const double *B_dev, int32_t ldb, int32_t kb, int64_t n,
                                   double *C_dev);
qg_status qg_block_product(qg_context ctx, const double *A_dev, int32_t lda, int32_t ka,
                           const double *M_dev, int32_t kb, int64_t n, double alpha, double beta,
                           double *X_dev, int32_t ldx);

/* out_dev (n x np row-major) = sum_i K_i C[i][:] for nk vectors K_i stored vector-major (K_dev,
 * K_i at [i * n]) and C_host (nk x np row-major complex): the combination of stored Krylov
 * vectors with the coefficients of a projected resolvent (the G1 T1 psi of RIXS,
 * Core/ResonantSpectra.cpp:123-195, :1441-1478). */
qg_status qg_krylov_combine(qg_context ctx, const double *K_dev, int64_t n, int32_t nk, const double *C_host,
                            int32_t np, double *out_dev);

/* The m x m matrix of spectra of a block tridiagonal matrix by the block continued fraction
 * (BlockTriDiagonalMatrixToSpectraWithBroadening, Core/BasicMathBlock/BasicMath_BlockTypeConversion.cpp:1636):
 * G_ij(w) = <v0_i| (w - H + i gamma/2)^-1 |v0_j> at w = emin + k*de + e0, k = 0..ne, one thread
 * per frequency; a_host, b_host as qg_block_lanczos returns them; m <= 8; g_host receives
 * m*m spectra of ne+1 complex points, spectrum i*m + j. */
qg_status qg_block_cf_spectra(qg_context ctx, int32_t m, int32_t ntri, const double *a_host, const double *b_host,
                              double e0, double emin, double de, int32_t ne, double gamma, double *g_host);

/* Settings of a resonant spectrum (ConvergenceSettingsType fields NTri1, NTri2, epsilon,
 * Emin1..Gamma2, restrictions1/2, Core/StructDef.cpp:252; energies E0_1/E0_2).  Emin/Emax set
 * to +-DBL_MAX and Gamma to 0 are resolved as the reference does and written back; NE1 and NE2
 * must be given (> 0). */
typedef struct {
  int32_t ntri1, ntri2;
  double epsilon;
  double emin1, emax1;
  int32_t ne1;
  double gamma1;
  double emin2, emax2;
  int32_t ne2;
  double gamma2;
  double energy1, energy2; /* DBL_MAX: <psi|H|psi> / <psi|psi> */
  const qg_restrictions *res1, *res2;
} qg_rixs_settings;

/* <psi|T1^dag G1^dag T2^dag G2 T2 G1 T1|psi> (ResonantSpectra, Core/ResonantSpectra.cpp:6):
 * Krylov-projected G1 = 1/(w1 + E1 - H1 + i Gamma1/2) on T1|psi>, then for every incident
 * energy and every T2 a Lanczos of H2 and the continued fraction.  g_host receives
 * nt2 * (ne1+1) spectra of ne2+1 complex points, spectrum i*(ne1+1) + p. */
qg_status qg_resonant_spectra(qg_context ctx, qg_operator H1, qg_operator H2, qg_operator T1,
                              const qg_operator *T2, int32_t nt2, qg_basis psi_basis, const double *psi_dev,
                              qg_rixs_settings *settings, double *g_host);

#ifdef __cplusplus
}
#endif

#endif /* QGPU_H */
