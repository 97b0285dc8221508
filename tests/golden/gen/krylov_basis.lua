-- KrylovBasis option of CreateSpectra (runs after the operator and state definitions of
-- rixs.lua, lines 1-28): the Lanczos branch returns the Krylov vectors of every (T, psi) pair
-- (LanczosTriDiagonalizeKrylov; a single list for one pair), the dense branch the eigenstates
-- of H on the dense basis.
o = {{"NE", 32}, {"Emin", -10}, {"Emax", 20}, {"Gamma", 0.5}}
function with(extra)
  local t = {}
  for _, v in ipairs(o) do t[#t + 1] = v end
  for _, v in ipairs(extra) do t[#t + 1] = v end
  return t
end
S, G, K = CreateSpectra(HX, Tz, psi1, with({{"Method", "Lanczos"}, {"KrylovBasis", true}, {"NTri", 80}}))
S.Print({{"file", "dump/lanczos_one.dat"}})
for i = 1, #K do _G["kone" .. i] = K[i]; io.put("dump", "kone" .. i) end
dump_reals("dump/count_one.txt", {#K})
S, G, K = CreateSpectra(HX, {Tx, Tz}, {psi1, psi2}, with({{"Method", "Lanczos"}, {"KrylovBasis", true}, {"NTri", 80}, {"Epsilon", 0}}))
S.Print({{"file", "dump/lanczos_lists.dat"}})
n = {}
for p = 1, #K do
  n[p] = #K[p]
  for i = 1, #K[p] do _G["klist" .. p .. "x" .. i] = K[p][i]; io.put("dump", "klist" .. p .. "x" .. i) end
end
dump_reals("dump/count_lists.txt", n)
S, G, K = CreateSpectra(HX, Tz, psi1, with({{"Method", "Dense"}, {"KrylovBasis", true}}))
S.Print({{"file", "dump/dense_states.dat"}})
E = {}
for i = 1, #K do E[i] = Complex.Re(K[i] * HX * K[i]) end
dump_reals("dump/dense_energies.txt", E)
Tz = Tz
io.put("dump", "Tz")
print("krylov_basis done")
