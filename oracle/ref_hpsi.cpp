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
//   int32 nf, int32 nterms, int64 ndet, int64 nsrc
//   int32 len[nterms], uint16 codes[sum len], double vre[nterms], double vim[nterms]
//   uint8 dets[ndet][nword]                     the basis (lookup targets), in its order
//   int64 src_rows[nsrc], double x[nsrc][2]     the source rows and their amplitudes
// The reference's loop runs over a wavefunction holding only the source determinants and
// adds into a wavefunction holding the whole basis (the function reads sources from psi and
// looks targets up in Opsi's table, :806-834), so a spread sample of source rows gives the
// push-form result of x restricted to those rows on the full basis.
//
// usage: ref_hpsi <input> <threads> <repeats> [<output y>]
// stdout: one line "basis_s=<s> call_s=<s0> <s1> ... pairs=<ndet_src * nterms>"
#define main quanty_reference_main
#include "LuaInterface/main.cpp"
#undef main

#include <omp.h>

#include <chrono>
#include <cstdio>
#include <vector>

template <class T>
static bool rd(FILE *f, T *p, size_t n) {
  return fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s <input> <threads> <repeats> [<output y>]\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t nf = 0, nterms = 0;
  int64_t ndet = 0, nsrc = 0;
  if (!rd(f, &nf, 1) || !rd(f, &nterms, 1) || !rd(f, &ndet, 1) || !rd(f, &nsrc, 1)) return 3;
  const int nword = (nf + 7) / 8;
  std::vector<int32_t> len(nterms);
  if (!rd(f, len.data(), (size_t)nterms)) return 3;
  size_t ncodes = 0;
  int maxlen = 0;
  for (int32_t l : len) {
    ncodes += (size_t)l;
    if (l > maxlen) maxlen = l;
  }
  std::vector<uint16_t> codes(ncodes + 1);
  std::vector<double> vre(nterms), vim(nterms);
  std::vector<uint8_t> dets((size_t)ndet * nword);
  std::vector<int64_t> src(nsrc);
  std::vector<double> x(2 * (size_t)nsrc);
  if (!rd(f, codes.data(), ncodes) || !rd(f, vre.data(), (size_t)nterms) || !rd(f, vim.data(), (size_t)nterms) ||
      !rd(f, dets.data(), dets.size()) || !rd(f, src.data(), (size_t)nsrc) || !rd(f, x.data(), x.size()))
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
  WaveFunctionType psi;
  psi.NFermion = (uint32_t)nf;
  psi.NBoson = 0;
  psi.NBitsKey = 20;
  psi.QComplex = 1;
  if (WaveFunctionInit(&psi)) return 5;
  for (int64_t s = 0; s < nsrc; s++)
    if (ComplexWaveFunctionAddElement(&psi, &dets[(size_t)src[s] * nword], x[2 * s], x[2 * s + 1])) return 5;
  double basis_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  omp_set_num_threads(atoi(argv[2]));
  int reps = atoi(argv[3]);
  printf("basis_s=%.3f call_s=", basis_s);
  for (int it = 0; it < reps; it++) {
    auto a = std::chrono::steady_clock::now();
    if (OperatorPsiConserveBasisPreAllocated(&H, &psi, &Opsi)) return 6;
    printf("%s%.4f", it ? " " : "", std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count());
    fflush(stdout);
  }
  printf(" pairs=%lld\n", (long long)psi.N * (long long)nterms);
  if (argc > 4) {
    FILE *o = fopen(argv[4], "wb");
    if (!o) return 7;
    for (int64_t r = 1; r <= ndet; r++) {
      double v[2] = {Opsi.ValueRe[BlokElement((uint32_t)r)], Opsi.ValueIm[BlokElement((uint32_t)r)]};
      fwrite(v, sizeof(double), 2, o);
    }
    fclose(o);
  }
  return 0;
}
