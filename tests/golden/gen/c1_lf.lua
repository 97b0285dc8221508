-- Ligand-field (charge-transfer) impurity on 26 spin-orbitals: 6 2p, 10 3d, 10 ligand.
-- Udd=7.5, Upd=8.5, Delta=3.0, Veg=2.0, Vt2g=1.2; Slater integrals and spin-orbit values of
-- the 16-orbital d8 case.  3-state Eigensystem plus 3-polarisation CreateSpectra with
-- NTri=200 and 2048 frequencies (Lanczos, Epsilon 0).
dofile("common.lua")
NF = 26
Dn2p, Up2p = {0, 2, 4}, {1, 3, 5}
Dn3d, Up3d = {6, 8, 10, 12, 14}, {7, 9, 11, 13, 15}
DnL, UpL = {16, 18, 20, 22, 24}, {17, 19, 21, 23, 25}
nd, Udd, Upd, Delta = 8, 7.5, 8.5, 3.0
F2dd, F4dd, F2pd, G1pd, G3pd = 10.0, 6.2, 6.2, 4.6, 2.6
zeta3d, zeta2p, tenDq, Veg, Vt2g = 0.08, 11.5, 1.1, 2.0, 1.2
F0dd = Udd + (F2dd + F4dd) * 2 / 63
F0pd = Upd + G1pd / 15 + G3pd * 3 / 70
-- charge-transfer site energies (d^nd L^10 reference, Delta = E(d^{n+1} L^9) - E(d^n L^10))
ed = (10 * Delta - nd * (19 + nd) * Udd / 2) / (10 + nd)
eL = nd * ((1 + nd) * Udd / 2 - Delta) / (10 + nd)
epf = (10 * Delta + (1 + nd) * (nd * Udd / 2 - (10 + nd) * Upd)) / (16 + nd)
edf = (10 * Delta - nd * (31 + nd) * Udd / 2 - 90 * Upd) / (16 + nd)
eLf = ((1 + nd) * (nd * Udd / 2 + 6 * Upd) - (6 + nd) * Delta) / (16 + nd)

Uop = {}
for k, v in ipairs({{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}) do Uop[k] = NewOperator("U", NF, Up3d, Dn3d, v) end
CF = NewOperator("CF", NF, Up3d, Dn3d, PotentialExpandedOnClm("Oh", 2, {0.6, -0.4}))
SO3 = NewOperator("ldots", NF, Up3d, Dn3d)
N3d = NewOperator("Number", NF, Up3d, Up3d, {1, 1, 1, 1, 1}) + NewOperator("Number", NF, Dn3d, Dn3d, {1, 1, 1, 1, 1})
NL = NewOperator("Number", NF, UpL, UpL, {1, 1, 1, 1, 1}) + NewOperator("Number", NF, DnL, DnL, {1, 1, 1, 1, 1})
N2p = NewOperator("Number", NF, Up2p, Up2p, {1, 1, 1}) + NewOperator("Number", NF, Dn2p, Dn2p, {1, 1, 1})
Akm = PotentialExpandedOnClm("Oh", 2, {1, 0})
Veg_op = NewOperator("CF", NF, Up3d, Dn3d, UpL, DnL, Akm) + NewOperator("CF", NF, UpL, DnL, Up3d, Dn3d, Akm)
Akm = PotentialExpandedOnClm("Oh", 2, {0, 1})
Vt2g_op = NewOperator("CF", NF, Up3d, Dn3d, UpL, DnL, Akm) + NewOperator("CF", NF, UpL, DnL, Up3d, Dn3d, Akm)
Hbase = F0dd * Uop[1] + F2dd * Uop[2] + F4dd * Uop[3] + tenDq * CF + zeta3d * SO3 + Veg * Veg_op + Vt2g * Vt2g_op
H = Hbase + ed * N3d + eL * NL
Upd_op = F0pd * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {1, 0}, {0, 0})
       + F2pd * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 1}, {0, 0})
       + G1pd * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 0}, {1, 0})
       + G3pd * NewOperator("U", NF, Up2p, Dn2p, Up3d, Dn3d, {0, 0}, {0, 1})
HX = Hbase + edf * N3d + eLf * NL + epf * N2p + zeta2p * NewOperator("ldots", NF, Up2p, Dn2p) + Upd_op
r = math.sqrt(0.5)
Tx = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, -1, r}, {1, 1, -r}})
Ty = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, -1, r * I}, {1, 1, r * I}})
Tz = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, 0, 1}})
for _, n in ipairs({"H", "HX", "Tx", "Ty", "Tz"}) do io.put("dump", n) end

R = {NF, 0, {"111111 0000000000 0000000000", 6, 6}, {"000000 1111111111 1111111111", 18, 18}}
psiList = Eigensystem(H, R, 3, {{"DenseBorder", 0}, {"Zero", 1e-14}, {"Epsilon", 0}})
E = {}
for i = 1, 3 do
  _G["psi" .. i] = psiList[i]
  io.put("dump", "psi" .. i)
  E[i] = Complex.Re(psiList[i] * H * psiList[i])
end
dump_reals("dump/energies_krylov.txt", E)
psiD = Eigensystem(H, R, 3)
ED = {}
for i = 1, 3 do ED[i] = Complex.Re(psiD[i] * H * psiD[i]) end
dump_reals("dump/energies_dense.txt", ED)
S, G = CreateSpectra(HX, {Tx, Ty, Tz}, psiList, {{"Emin", -10}, {"Emax", 20}, {"NE", 2048}, {"Gamma", 0.5}, {"NTri", 200}, {"Method", "Lanczos"}, {"Epsilon", 0}})
S.Print({{"file", "dump/spec_eps0.dat"}})
for i = 1, #G do dump_tri("dump/tri_eps0_" .. i .. ".txt", G[i]) end
print("c1_lf done")
