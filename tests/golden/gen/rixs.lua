-- RIXS (CreateResonantSpectra) of the reference on the 16-orbital 2p -> 3d case (the
-- Hamiltonians of c0_xas.lua): the dense branch it takes by default on bases below
-- DenseBorder, with lists of absorption operators, emission operators and initial states;
-- the tensor form of the dense branch; the Krylov branch (DenseBorder 0) with lists; and the
-- Krylov tensor form, all as Spectra.Print text.
dofile("common.lua")
NF = 16
Dn2p, Up2p = {0, 2, 4}, {1, 3, 5}
Dn3d, Up3d = {6, 8, 10, 12, 14}, {7, 9, 11, 13, 15}
Hdd = 10.0 * NewOperator("U", NF, Up3d, Dn3d, {0, 1, 0}) + 6.2 * NewOperator("U", NF, Up3d, Dn3d, {0, 0, 1})
Hcf = 1.1 * NewOperator("CF", NF, Up3d, Dn3d, PotentialExpandedOnClm("Oh", 2, {0.6, -0.4}))
Hso = 0.08 * NewOperator("ldots", NF, Up3d, Dn3d)
H = Hdd + Hcf + Hso
Hpd = 6.2 * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 1}, {0, 0})
    + 4.6 * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 0}, {1, 0})
    + 2.6 * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 0}, {0, 1})
HX = H + 11.5 * NewOperator("ldots", NF, Up2p, Dn2p) + Hpd
r = math.sqrt(0.5)
Tx = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, -1, r}, {1, 1, -r}})
Ty = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, -1, r * I}, {1, 1, r * I}})
Tz = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, 0, 1}})
Txd = ConjugateTranspose(Tx)
Tyd = ConjugateTranspose(Ty)
Tzd = ConjugateTranspose(Tz)
R = {NF, 0, {"111111 0000000000", 6, 6}, {"000000 1111111111", 8, 8}}
psiList = Eigensystem(H, R, 2)
psi1, psi2 = psiList[1], psiList[2]
for _, n in ipairs({"H", "HX", "Tx", "Ty", "Txd", "Tyd", "Tzd", "psi1", "psi2"}) do io.put("dump", n) end

function opts(extra)
  local o = {{"Emin1", -5}, {"Emax1", 15}, {"NE1", 4}, {"Gamma1", 0.8},
             {"Emin2", -2}, {"Emax2", 8}, {"NE2", 64}, {"Gamma2", 0.3}}
  for _, v in ipairs(extra) do o[#o + 1] = v end
  return o
end
-- dense branch, lists of T1, T2 and psi
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd, Tzd}, {psi1, psi2}, opts({}))
S.Print({{"file", "dump/dense_lists.dat"}})
-- dense branch, automatic energy ranges
S = CreateResonantSpectra(HX, H, Tx, {Txd, Tyd}, psi1, {{"NE1", 4}, {"Gamma1", 0.8}, {"NE2", 64}, {"Gamma2", 0.3}})
S.Print({{"file", "dump/dense_auto.dat"}})
-- dense tensor form
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Tensor", true}}))
S.Print({{"file", "dump/dense_tensor.dat"}})
S = CreateResonantSpectra(HX, H, {Tx}, {Tyd}, {psi1, psi2}, opts({{"Tensor", true}}))
S.Print({{"file", "dump/dense_tensor_psi.dat"}})
-- Krylov branch with lists
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, {psi1, psi2}, opts({{"DenseBorder", 0}, {"Epsilon", 0}}))
S.Print({{"file", "dump/krylov_lists.dat"}})
-- Krylov tensor form
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}, {"NTri1", 40}, {"NTri2", 40}}))
S.Print({{"file", "dump/krylov_tensor.dat"}})
-- Krylov tensor form with automatic energy ranges
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd}, psi1, {{"NE1", 3}, {"NE2", 48}, {"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}, {"NTri1", 40}, {"NTri2", 40}})
S.Print({{"file", "dump/krylov_tensor_auto.dat"}})
-- Krylov tensor form with two initial states
S = CreateResonantSpectra(HX, H, {Tx}, {Tyd}, {psi1, psi2}, opts({{"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}, {"NTri1", 40}, {"NTri2", 40}}))
S.Print({{"file", "dump/krylov_tensor_psi.dat"}})
-- dense branch with given energy shifts
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd}, {psi1, psi2}, opts({{"E0_1", -37.0}, {"E0_2", -17.0}}))
S.Print({{"file", "dump/dense_shifts.dat"}})
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd}, {psi1, psi2}, opts({{"E0", -30.0}}))
S.Print({{"file", "dump/dense_e0.dat"}})
-- final-state restrictions (four down-spin 3d electrons) in both branches
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Restrictions2", {NF, 0, {"000000 1010101010", 4, 4}}}}))
S.Print({{"file", "dump/dense_res2.dat"}})
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Restrictions2", {NF, 0, {"000000 1010101010", 4, 4}}}, {"DenseBorder", 0}, {"Epsilon", 0}}))
S.Print({{"file", "dump/krylov_res2.dat"}})
-- intermediate-state restrictions (five down-spin 3d electrons) in every branch
R1 = {NF, 0, {"000000 1010101010", 5, 5}}
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Restrictions1", R1}}))
S.Print({{"file", "dump/dense_res1.dat"}})
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Restrictions1", R1}, {"DenseBorder", 0}, {"Epsilon", 0}}))
S.Print({{"file", "dump/krylov_res1.dat"}})
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"Restrictions1", R1}, {"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}}))
S.Print({{"file", "dump/krylov_tensor_res1.dat"}})
-- Krylov tensor form with incomplete Krylov spaces (8 intermediate and 20 final Krylov vectors
-- on 60 and 45 determinants): the result depends on both block recursions
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd, Tyd}, psi1, opts({{"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}, {"NTri1", 4}, {"NTri2", 5}}))
S.Print({{"file", "dump/krylov_tensor_short.dat"}})
S = CreateResonantSpectra(HX, H, {Tx, Ty}, {Txd}, psi1, {{"NE1", 3}, {"NE2", 48}, {"DenseBorder", 0}, {"Epsilon", 0}, {"Tensor", true}, {"NTri1", 6}, {"NTri2", 8}})
S.Print({{"file", "dump/krylov_tensor_short_auto.dat"}})
print("rixs done")
