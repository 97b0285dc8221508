-- Basis growth of Eigensystem (runs after the operator definitions of c1_lf.lua, lines 1-44):
-- start restrictions that allow only d8 L10 (138 of the 190 determinants of the 18-electron
-- sector are reached by hybridisation), without and with the Restrictions option that
-- confines the growth.  Without it the reference grows into d9 L9 and d10 L8.
Rn = {NF, 0, {"111111 0000000000 0000000000", 6, 6}, {"000000 1111111111 0000000000", 8, 8}, {"000000 0000000000 1111111111", 10, 10}}
psiN = Eigensystem(H, Rn, 3)
E = {}
for i = 1, 3 do E[i] = Complex.Re(psiN[i] * H * psiN[i]) end
dump_reals("dump/energies_grown.txt", E)
psiR = Eigensystem(H, Rn, 3, {{"Restrictions", Rn}})
for i = 1, 3 do E[i] = Complex.Re(psiR[i] * H * psiR[i]) end
dump_reals("dump/energies_confined.txt", E)
-- the second call form: start from wavefunctions (copies of the confined states), which it
-- replaces in place, grown without limit
psiW = {psiR[1] * 1, psiR[2] * 1, psiR[3] * 1}
Eigensystem(H, psiW)
for i = 1, 3 do E[i] = Complex.Re(psiW[i] * H * psiW[i]) end
dump_reals("dump/energies_from_states.txt", E)
print("eigen_growth done")
