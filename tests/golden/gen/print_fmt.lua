-- Spectra.Print output of the reference, for the byte layout of the spectra files: the
-- 16-orbital 2p -> 3d XAS (the same Hamiltonian as c0_xas.lua) with few frequencies, through
-- the Lanczos branch with given and with default energy ranges, and through the dense branch.
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
Tz = NewOperator("CF", NF, Up3d, Dn3d, Up2p, Dn2p, {{1, 0, 1}})
for _, n in ipairs({"HX", "Tz"}) do io.put("dump", n) end
R = {NF, 0, {"111111 0000000000", 6, 6}, {"000000 1111111111", 8, 8}}
psiList = Eigensystem(H, R, 2)
psi1, psi2 = psiList[1], psiList[2]
io.put("dump", "psi1")
io.put("dump", "psi2")
S = CreateSpectra(HX, Tz, {psi1, psi2}, {{"Emin", -10}, {"Emax", 20}, {"NE", 16}, {"Gamma", 0.5}, {"Method", "Lanczos"}, {"Epsilon", 0}})
S.Print({{"file", "dump/print_lanczos.dat"}})
S = CreateSpectra(HX, Tz, psi1, {{"NE", 12}, {"Method", "Lanczos"}, {"Epsilon", 0}})
S.Print({{"file", "dump/print_defaults.dat"}})
S = CreateSpectra(HX, Tz, psi1, {{"NE", 12}, {"Method", "Dense"}})
S.Print({{"file", "dump/print_dense.dat"}})
print("print_fmt done")
