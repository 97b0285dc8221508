-- Small plain case: 2p -> 3d XAS of a d8 ion in Oh on 16 spin-orbitals (6 2p + 10 3d).
-- 3d Coulomb F2=10.0, F4=6.2 (F0=0); 2p-3d F2=6.2, G1=4.6, G3=2.6; zeta3d=0.08,
-- zeta2p=11.5; 10Dq=1.1.  Eigensystem for the lowest 3 states, then CreateSpectra of x/y/z
-- dipoles, NE=1024 on [-10,20], Gamma=0.5, by Lanczos (DenseBorder 0) at Epsilon 0 and at
-- the default epsilon, plus a small RIXS run.
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

for _, n in ipairs({"H", "HX", "Tx", "Ty", "Tz"}) do io.put("dump", n) end

R = {NF, 0, {"111111 0000000000", 6, 6}, {"000000 1111111111", 8, 8}}
psiList = Eigensystem(H, R, 3)
E = {}
for i = 1, 3 do
  _G["psi" .. i] = psiList[i]
  io.put("dump", "psi" .. i)
  E[i] = Complex.Re(psiList[i] * H * psiList[i])
end
dump_reals("dump/energies_dense.txt", E)
-- the Krylov eigensolver on the same problem
psiK = Eigensystem(H, R, 3, {{"DenseBorder", 0}, {"Zero", 1e-14}, {"Epsilon", 0}})
EK = {}
for i = 1, 3 do EK[i] = Complex.Re(psiK[i] * H * psiK[i]) end
dump_reals("dump/energies_krylov.txt", EK)

opts = {{"Emin", -10}, {"Emax", 20}, {"NE", 1024}, {"Gamma", 0.5}, {"Method", "Lanczos"}}
for _, eps in ipairs({"0", "default"}) do
  local o = {}
  for k, v in ipairs(opts) do o[k] = v end
  if eps == "0" then o[#o + 1] = {"Epsilon", 0} end
  local S, G = CreateSpectra(HX, {Tx, Ty, Tz}, psiList, o)
  S.Print({{"file", "dump/spec_eps" .. eps .. ".dat"}})
  for i = 1, #G do dump_tri("dump/tri_eps" .. eps .. "_" .. i .. ".txt", G[i]) end
end
-- dense reference spectra for the same call
Sd = CreateSpectra(HX, {Tx, Ty, Tz}, psiList, {{"Emin", -10}, {"Emax", 20}, {"NE", 1024}, {"Gamma", 0.5}, {"Method", "Dense"}})
Sd.Print({{"file", "dump/spec_dense.dat"}})
-- RIXS: 2p -> 3d absorption (x), intermediate Hamiltonian HX, final Hamiltonian H, emission y
Tyd = ConjugateTranspose(Ty)
io.put("dump", "Tyd")
Sr = CreateResonantSpectra(HX, H, Tx, Tyd, psiList[1],
  {{"Emin1", -5}, {"Emax1", 15}, {"NE1", 4}, {"Gamma1", 0.8}, {"Emin2", -2}, {"Emax2", 8}, {"NE2", 256}, {"Gamma2", 0.3}, {"DenseBorder", 0}, {"Epsilon", 0}})
Sr.Print({{"file", "dump/rixs.dat"}})
-- the same at the default epsilon (the Krylov-basis Lanczos of the intermediate states zeroes
-- a new vector whose squared overlaps with the earlier ones exceed epsilon, so epsilon 0
-- keeps one Krylov vector)
Sd = CreateResonantSpectra(HX, H, Tx, Tyd, psiList[1],
  {{"Emin1", -5}, {"Emax1", 15}, {"NE1", 4}, {"Gamma1", 0.8}, {"Emin2", -2}, {"Emax2", 8}, {"NE2", 256}, {"Gamma2", 0.3}, {"DenseBorder", 0}})
Sd.Print({{"file", "dump/rixs_default.dat"}})
print("c0_xas done")
