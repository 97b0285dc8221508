// Test and measurement infrastructure only: times the reference's own fixed-basis H*psi
// (OperatorPsiConserveBasisPreAllocated, Core/OperatorWaveFunction.cpp:5541, and the loops it
// dispatches to, :784-1127) on a basis and operator read from a file, and writes its result.
// The reference's translation unit is compiled into this program unmodified (its main() is
// renamed); the functions called are its own: InitOperator / InitOperatorFixedLength /
// OperatorAddLader (Core/OperatorArithmetic.cpp:74, :219, :1188), WaveFunctionInit and
// WaveFunctionInitCopyBasis (Core/WaveFunctionArithmetic.cpp:124, :264),
// ComplexWaveFunctionAddElement (Core/ComplexWaveFunctionArithmetic.cpp:64).  Nothing in the
// product links or runs this program.
//
// Input file (little endian):
//   int32 nf, int32 nterms, int64 ndet
//   int32 len[nterms], uint16 codes[sum len], double vre[nterms], double vim[nterms]
//   uint8 dets[ndet][nword]   the basis (lookup targets), in its order
//   double x[ndet][2]         the amplitudes
// The reference's loop runs over a wavefunction holding the source determinants and adds into
// a wavefunction holding the whole basis (the function reads sources from psi and looks targets
// up in Opsi's table, :806-834), so the sources can be a spread sample of the basis: every
// stride-th row, giving the push-form result of x restricted to those rows on the full basis.
//
// usage: ref_hpsi <input> <run>[,<run>...] [<output y>]
//   run = <threads>:<spec>:<calls>, spec = s<stride> (sources are rows 0, stride, 2 stride, ...)
//   or t<seconds> (a probe call on a thin sample picks the stride for about that many seconds)
// The output y is the result of the first run's last call on the whole basis.
// stdout: one line per run:
//   "threads=<T> stride=<m> sources=<S> pairs=<S * nterms> basis_s=<s> call_s=<s0> <s1> ..."
#define main quanty_reference_main
#include "LuaInterface/main.cpp"
#undef main

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

template <class T>
static bool rd(FILE *f, T *p, size_t n) {
  return fread(p, sizeof(T), n, f) == n;
}

static bool build_sources(WaveFunctionType *psi, int nf, int nword, const std::vector<uint8_t> &dets,
                          const std::vector<double> &x, int64_t ndet, int64_t stride) {
  psi->NFermion = (uint32_t)nf;
  psi->NBoson = 0;
  uint32_t bits = 10;
  while (bits < 28 && ((int64_t)1 << bits) < 2 * (ndet / stride + 1)) bits++;
  psi->NBitsKey = bits;
  psi->QComplex = 1;
  if (WaveFunctionInit(psi)) return false;
  for (int64_t r = 0; r < ndet; r += stride)
    if (ComplexWaveFunctionAddElement(psi, &dets[(size_t)r * nword], x[2 * r], x[2 * r + 1])) return false;
  return true;
}

static double timed_call(const OperatorType &H, const WaveFunctionType &psi, WaveFunctionType &Opsi) {
  auto a = std::chrono::steady_clock::now();
  if (OperatorPsiConserveBasisPreAllocated(&H, &psi, &Opsi)) return -1.0;
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <input> <threads>:<s<stride>|t<seconds>>:<calls>[,...] [<output y>]\n", argv[0]);
    return 2;
  }
  bool y_done = false;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t nf = 0, nterms = 0;
  int64_t ndet = 0;
  if (!rd(f, &nf, 1) || !rd(f, &nterms, 1) || !rd(f, &ndet, 1)) return 3;
  const int nword = (nf + 7) / 8;
  std::vector<int32_t> len(nterms);
  if (!rd(f, len.data(), (size_t)nterms)) return 3;
  size_t ncodes = 0;
  int maxlen = 0;
  for (int32_t l : len) {
    ncodes += (size_t)l;
    if (l > maxlen) maxlen = l;
    if (l < 1) return 3;  // scalar terms are not part of these operators
  }
  std::vector<uint16_t> codes(ncodes + 1);
  std::vector<double> vre(nterms), vim(nterms);
  std::vector<uint8_t> dets((size_t)ndet * nword);
  std::vector<double> x(2 * (size_t)ndet);
  if (!rd(f, codes.data(), ncodes) || !rd(f, vre.data(), (size_t)nterms) || !rd(f, vim.data(), (size_t)nterms) ||
      !rd(f, dets.data(), dets.size()) || !rd(f, x.data(), x.size()))
    return 3;
  fclose(f);

  // the operator, string by string, through the reference's own constructors
  OperatorType H;
  if (InitOperator(&H)) return 4;
  H.NFermion = (uint32_t)nf;
  H.NBoson = 0;
  H.NWord = (uint32_t)nword;
  for (int l = 1; l <= maxlen; l++)
    if (InitOperatorFixedLength(&H, (uint32_t)l, 10)) return 4;
  size_t off = 0;
  for (int32_t t = 0; t < nterms; t++) {
    if (OperatorAddLader(&H, codes.data() + off, (uint32_t)len[t], vre[t], vim[t])) return 4;
    off += (size_t)len[t];
  }
  SetQComplexOperator(&H);

  // the basis with the reference's hash sized as its block eigensolver sizes it (about 2N keys)
  auto t0 = std::chrono::steady_clock::now();
  uint32_t bits = 10;
  while (bits < 31 && ((int64_t)1 << bits) < 2 * ndet) bits++;
  WaveFunctionType full;
  full.NFermion = (uint32_t)nf;
  full.NBoson = 0;
  full.NBitsKey = bits;
  full.QComplex = 1;
  if (WaveFunctionInit(&full)) return 5;
  for (int64_t r = 0; r < ndet; r++)
    if (ComplexWaveFunctionAddElement(&full, &dets[(size_t)r * nword], 0.0, 0.0)) return 5;
  if ((int64_t)full.N != ndet) {
    fprintf(stderr, "basis has duplicate determinants (%u of %lld kept)\n", full.N, (long long)ndet);
    return 5;
  }
  WaveFunctionType Opsi;
  if (WaveFunctionInitCopyBasis(&Opsi, full)) return 5;
  double basis_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  for (char *p = argv[2]; *p;) {
    int threads = atoi(p);
    while (*p && *p != ':') p++;
    if (!*p) return 2;
    p++;
    const bool by_time = *p == 't';
    const double spec = atof(p + 1);
    while (*p && *p != ':') p++;
    if (!*p) return 2;
    p++;
    const int calls = atoi(p);
    while (*p && *p != ',') p++;
    if (*p) p++;
    if (threads < 1 || calls < 1 || spec <= 0) return 2;
    omp_set_num_threads(threads);
    int64_t stride = (int64_t)spec;
    if (by_time) {  // a thin probe (about 4000 sources per thread) sets the stride
      int64_t probe = std::max<int64_t>(1, ndet / (4000 * (int64_t)threads));
      WaveFunctionType pp;
      if (!build_sources(&pp, nf, nword, dets, x, ndet, probe)) return 5;
      double dt = timed_call(H, pp, Opsi);
      if (dt < 0) return 6;
      stride = std::max<int64_t>(1, (int64_t)ceil((double)ndet * (dt / (double)pp.N) / spec));
      WaveFunctionFree(&pp);
    }
    WaveFunctionType psi;
    if (!build_sources(&psi, nf, nword, dets, x, ndet, stride)) return 5;
    printf("threads=%d stride=%lld sources=%u pairs=%lld basis_s=%.3f call_s=", threads, (long long)stride, psi.N,
           (long long)psi.N * (long long)nterms, basis_s);
    for (int c = 0; c < calls; c++) {
      double dt = timed_call(H, psi, Opsi);
      if (dt < 0) return 6;
      printf("%s%.4f", c ? " " : "", dt);
      fflush(stdout);
    }
    printf("\n");
    if (argc > 3 && !y_done) {
      FILE *o = fopen(argv[3], "wb");
      if (!o) return 7;
      for (int64_t r = 1; r <= ndet; r++) {
        double v[2] = {Opsi.ValueRe[BlokElement((uint32_t)r)], Opsi.ValueIm[BlokElement((uint32_t)r)]};
        fwrite(v, sizeof(double), 2, o);
      }
      fclose(o);
      y_done = true;
    }
    WaveFunctionFree(&psi);
  }
  return 0;
}
