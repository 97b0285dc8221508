-- Tensor spectra (CreateSpectra with Tensor = true) of the reference on the 16-orbital
-- 2p -> 3d XAS (the Hamiltonian of c0_xas.lua): the 3 x 3 matrix of dipole spectra of the
-- ground state, dense branch and block-Lanczos branch, as Spectra.Print text.
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
for _, n in ipairs({"HX", "Tx", "Ty", "Tz"}) do io.put("dump", n) end
R = {NF, 0, {"111111 0000000000", 6, 6}, {"000000 1111111111", 8, 8}}
psi1 = Eigensystem(H, R, 1)
io.put("dump", "psi1")
S = CreateSpectra(HX, {Tx, Ty, Tz}, psi1, {{"Tensor", true}, {"Method", "Dense"}, {"NE", 40}, {"Emin", -5}, {"Emax", 15}, {"Gamma", 0.6}})
S.Print({{"file", "dump/tensor_dense.dat"}})
S = CreateSpectra(HX, {Tx, Ty, Tz}, psi1, {{"Tensor", true}, {"Method", "Dense"}, {"NE", 24}})
S.Print({{"file", "dump/tensor_dense_defaults.dat"}})
S = CreateSpectra(HX, {Tx, Ty, Tz}, psi1, {{"Tensor", true}, {"Method", "Lanczos"}, {"NE", 40}, {"Emin", -5}, {"Emax", 15}, {"Gamma", 0.6}, {"Epsilon", 0}})
S.Print({{"file", "dump/tensor_lanczos.dat"}})
-- block Lanczos with an incomplete Krylov space (15 and 24 Krylov vectors on the final-state
-- basis): the result depends on the block recursion itself, not only on H
S = CreateSpectra(HX, {Tx, Ty, Tz}, psi1, {{"Tensor", true}, {"Method", "Lanczos"}, {"NTri", 5}, {"NE", 40}, {"Emin", -5}, {"Emax", 15}, {"Gamma", 0.6}, {"Epsilon", 0}})
S.Print({{"file", "dump/tensor_lanczos_short.dat"}})
S = CreateSpectra(HX, {Tx, Ty, Tz}, psi1, {{"Tensor", true}, {"Method", "Lanczos"}, {"NTri", 8}, {"NE", 32}})
S.Print({{"file", "dump/tensor_lanczos_short_auto.dat"}})
print("tensor done")
