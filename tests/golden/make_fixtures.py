"""Generate the golden fixtures under tests/golden/ from the reference Quanty binary.

Test infrastructure only; run in a container that has the reference sources:

    oracle/build_ref.sh                 # builds oracle/_ref/Quanty from the reference
    python tests/golden/make_fixtures.py

Each generator in tests/golden/gen/*.lua runs under the reference binary with one OpenMP
thread and a pinned srand() seed; it writes operators and wavefunctions with Quanty's own
``io.put`` and numbers with full precision.  Two generators wrap code taken at run time
from the reference's own test scripts (the impurity-chain model and its golden tridiagonal
tables from TestScripts/CreateSpectra.Quanty, the f-shell atom and its Mathematica
eigenvalues from TestScripts/Eigensystem.Quanty), so those known answers are checked
against the reference here and kept as fixtures.  The JSON files written here are what the
tests read; nothing at test time touches the reference or its binary.
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from quanty_gb300.quanty_text import parse_operator, parse_wavefunction  # noqa: E402

REF = os.environ.get("QUANTY_REFERENCE", "/root/reference")
# the binary the generators run under (another build of Quanty may be named, e.g. the one whose
# H*psi path runs through libqgpu, to compare its outputs with the fixtures)
QUANTY = os.environ.get("QUANTY_BINARY", os.path.join(ROOT, "oracle", "_ref", "Quanty"))
# when a dict, generated fixtures are stored here by name instead of written to tests/golden
SINK = None


def run(script_text, name):
    work = tempfile.mkdtemp(prefix="qfx_")
    shutil.copy(os.path.join(HERE, "gen", "common.lua"), work)
    with open(os.path.join(work, name), "w") as f:
        f.write(script_text)
    os.makedirs(os.path.join(work, "dump"))
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run([QUANTY, name], cwd=work, env=env, capture_output=True, text=True, timeout=1800)
    if p.returncode != 0 or "Error" in p.stdout:
        sys.stderr.write(p.stdout[-3000:] + p.stderr[-3000:])
        raise RuntimeError("generator %s failed" % name)
    return work


def fname(var):
    """io.put file name of a Lua global: upper-case letters are written as ^ + lower case."""
    return re.sub(r"[A-Z]", lambda m: "^" + m.group(0).lower(), var) + ".Quanty"


def op(work, var):
    o = parse_operator(open(os.path.join(work, "dump", fname(var))).read())
    return {"nf": o["nf"], "terms": [[list(t[0]), t[1], t[2]] for t in o["terms"]]}


def wf(work, var):
    return parse_wavefunction(open(os.path.join(work, "dump", fname(var))).read())


def reals(work, f):
    return [float(x) for x in open(os.path.join(work, "dump", f)).read().split()]


def complexes(work, f):
    v = [float(x) for x in open(os.path.join(work, "dump", f)).read().split()]
    return [[v[2 * i], v[2 * i + 1]] for i in range(len(v) // 2)]


def tri(work, f):
    v = open(os.path.join(work, "dump", f)).read().split()
    na, nb = int(v[0]), int(v[1])
    x = [float(t) for t in v[2:]]
    return {"a": x[:na], "b": x[na:na + nb]}


def spectra(work, f):
    """Parse a Spectra.Print file: header lines then 'E Re0 Im0 Re1 Im1 ...' rows."""
    lines = open(os.path.join(work, "dump", f)).read().splitlines()
    n = int(lines[0].split(":")[1])
    hdr = {}
    for ln in lines[1:4]:
        k = ln.split()[0]
        hdr[k] = [float(t) for t in ln.split()[1:]]
    rows = []
    for ln in lines:
        t = ln.split()
        if not t:
            continue
        try:
            rows.append([float(x) for x in t])
        except ValueError:
            continue
    rows = [r for r in rows if len(r) == 1 + 2 * n]
    return {
        "nspec": n,
        "emin": hdr["Emin______Emax"][0], "emax": hdr["Emin______Emax"][1],
        "de": hdr["dE________Gamma"][0], "gamma": hdr["dE________Gamma"][1],
        "energy": [r[0] for r in rows],
        "re": [[r[1 + 2 * s] for r in rows] for s in range(n)],
        "im": [[r[2 + 2 * s] for r in rows] for s in range(n)],
    }


def save(name, obj):
    if SINK is not None:
        SINK[name] = obj
        return
    path = os.path.join(HERE, name)
    with open(path, "w") as f:
        json.dump(obj, f, separators=(",", ":"))
    print("wrote %s (%d bytes)" % (path, os.path.getsize(path)))


def gen_hpsi():
    src = open(os.path.join(HERE, "gen", "hpsi_cases.lua")).read()
    work = run(src, "hpsi_cases.lua")
    names = sorted({f.split("_")[0] for f in os.listdir(os.path.join(work, "dump"))})
    cases = []
    for n in names:
        lohi = reals(work, n + "_restriction.txt")
        nf = wf(work, n + "_psi")["nf"]
        mask = "".join("1" if i < nf // 2 else "0" for i in range(nf))
        cases.append({
            "name": n, "H": op(work, n + "_H"), "psi": wf(work, n + "_psi"),
            "Hpsi": wf(work, n + "_Hpsi"), "Hpsir": wf(work, n + "_Hpsir"),
            "restrictions": [[mask, int(lohi[0]), int(lohi[1])]],
        })
    save("hpsi_cases.json", {"source": "tests/golden/gen/hpsi_cases.lua", "cases": cases})


def gen_c0():
    work = run(open(os.path.join(HERE, "gen", "c0_xas.lua")).read(), "c0_xas.lua")
    out = {"source": "tests/golden/gen/c0_xas.lua"}
    for n in ["H", "HX", "Tx", "Ty", "Tz", "Tyd"]:
        out[n] = op(work, n)
    out["psi"] = [wf(work, "psi%d" % i) for i in (1, 2, 3)]
    out["energies_dense"] = reals(work, "energies_dense.txt")
    out["energies_krylov"] = reals(work, "energies_krylov.txt")
    out["restrictions"] = [["1111110000000000", 6, 6], ["0000001111111111", 8, 8]]
    out["spectra_opts"] = {"Emin": -10, "Emax": 20, "NE": 1024, "Gamma": 0.5}
    for eps in ("0", "default"):
        out["spec_eps" + eps] = spectra(work, "spec_eps%s.dat" % eps)
        out["tri_eps" + eps] = [tri(work, "tri_eps%s_%d.txt" % (eps, i)) for i in range(1, 10)]
    out["spec_dense"] = spectra(work, "spec_dense.dat")
    out["rixs_opts"] = {"Emin1": -5, "Emax1": 15, "NE1": 4, "Gamma1": 0.8, "Emin2": -2, "Emax2": 8,
                        "NE2": 256, "Gamma2": 0.3, "Epsilon": 0}
    out["rixs"] = spectra(work, "rixs.dat")
    out["rixs_default"] = spectra(work, "rixs_default.dat")
    save("c0_xas.json", out)


def gen_c1():
    work = run(open(os.path.join(HERE, "gen", "c1_lf.lua")).read(), "c1_lf.lua")
    out = {"source": "tests/golden/gen/c1_lf.lua"}
    for n in ["H", "HX", "Tx", "Ty", "Tz"]:
        out[n] = op(work, n)
    out["psi"] = [wf(work, "psi%d" % i) for i in (1, 2, 3)]
    out["energies_krylov"] = reals(work, "energies_krylov.txt")
    out["energies_dense"] = reals(work, "energies_dense.txt")
    out["restrictions"] = [["11111100000000000000000000", 6, 6], ["00000011111111111111111111", 18, 18]]
    out["spectra_opts"] = {"Emin": -10, "Emax": 20, "NE": 2048, "Gamma": 0.5, "NTri": 200, "Epsilon": 0}
    out["spec_eps0"] = spectra(work, "spec_eps0.dat")
    out["tri_eps0"] = [tri(work, "tri_eps0_%d.txt" % i) for i in range(1, 10)]
    save("c1_lf.json", out)


CHAIN_DRIVER = r"""
dofile("common.lua")
%s
combos = {}
for ih, Hname in ipairs({"H0", "H1", "H2"}) do
  for _, Tn in ipairs({"Dn", "Up"}) do
    for ip = 1, 2 do
      combos[#combos + 1] = {Hname, "T" .. Tn, "psi" .. ip, "G" .. (ih - 1) .. Tn .. ip}
    end
  end
end
for _, n in ipairs({"H0", "H1", "H2", "TDn", "TUp", "psi1", "psi2"}) do io.put("dump", n) end
dump_reals("dump/omega.txt", omegaList)
for k, c in ipairs(combos) do
  local gold = _G[c[4]]
  local vals = {}
  for i, w in ipairs(omegaList) do vals[i] = gold(w, 0.1) end
  dump_complex("dump/gold_" .. k .. ".txt", vals)
  dump_tri("dump/goldtri_" .. k .. ".txt", gold)
  local spec, G = CreateSpectra(_G[c[1]], _G[c[2]], _G[c[3]], {{"DenseBorder", 1}, {"Tensor", false}})
  G = G[1]
  local got = {}
  for i, w in ipairs(omegaList) do got[i] = G(w, 0.1) end
  dump_complex("dump/ref_" .. k .. ".txt", got)
  dump_tri("dump/reftri_" .. k .. ".txt", G)
  local f = io.open("dump/combo_" .. k .. ".txt", "w"); f:write(table.concat(c, " ")); f:close()
end
print("chain done")
"""


def gen_chain():
    lines = open(os.path.join(REF, "TestScripts", "CreateSpectra.Quanty")).read().splitlines()
    s = next(i for i, l in enumerate(lines) if l.startswith("-- Define some model Hamiltonian"))
    e = next(i for i, l in enumerate(lines) if l.startswith("threshold"))
    model = "\n".join(lines[s:e + 1])
    work = run(CHAIN_DRIVER % model, "chain.lua")
    out = {"source": "TestScripts/CreateSpectra.Quanty:%d-%d (model, golden tables, omega list, threshold)" % (s + 1, e + 1),
           "gamma": 0.1, "threshold": 1e-12, "omega": reals(work, "omega.txt")}
    for n in ["H0", "H1", "H2", "TDn", "TUp"]:
        out[n] = op(work, n)
    out["psi1"] = wf(work, "psi1")
    out["psi2"] = wf(work, "psi2")
    combos = []
    k = 1
    while os.path.exists(os.path.join(work, "dump", "combo_%d.txt" % k)):
        c = open(os.path.join(work, "dump", "combo_%d.txt" % k)).read().split()
        combos.append({"H": c[0], "T": c[1], "psi": c[2], "golden": c[3],
                       "golden_G": complexes(work, "gold_%d.txt" % k),
                       "golden_tri": tri(work, "goldtri_%d.txt" % k),
                       "ref_G": complexes(work, "ref_%d.txt" % k),
                       "ref_tri": tri(work, "reftri_%d.txt" % k)})
        k += 1
    out["combos"] = combos
    save("chain_spectra.json", out)


FSHELL_DRIVER = r"""
dofile("common.lua")
%s
io.put("dump", "Hamiltonian1")
dump_reals("dump/expected.txt", expectedEn)
f10 = Eigensystem(Hamiltonian1, StartRestrictions, 10)
E = {}
for i = 1, 10 do E[i] = Complex.Re(f10[i] * Hamiltonian1 * f10[i]) end
dump_reals("dump/energies_default.txt", E)
f10t = Eigensystem(Hamiltonian1, StartRestrictions, 10, {{"Zero", 1e-14}, {"Epsilon", 0}})
E = {}
for i = 1, 10 do E[i] = Complex.Re(f10t[i] * Hamiltonian1 * f10t[i]) end
dump_reals("dump/energies_tight.txt", E)
print("fshell done")
"""


def gen_fshell():
    lines = open(os.path.join(REF, "TestScripts", "Eigensystem.Quanty")).read().splitlines()
    a = next(i for i, l in enumerate(lines) if l.startswith("::atom::"))
    keep = []
    for i in range(a, len(lines)):
        l = lines[i]
        if re.match(r"^(Basis_dn|Basis_up|Hamiltonian1|StartRestrictions|expectedEn)\s*=", l):
            keep.append((i + 1, l))
        if l.startswith("expectedEn"):
            break
    model = "\n".join(l for _, l in keep)
    work = run(FSHELL_DRIVER % model, "fshell.lua")
    out = {"source": "TestScripts/Eigensystem.Quanty:" + ",".join(str(i) for i, _ in keep),
           "H": op(work, "Hamiltonian1"), "restrictions": [["11111111111111", 6, 6]],
           "expected_mathematica": reals(work, "expected.txt"),
           "energies_default": reals(work, "energies_default.txt"),
           "energies_tight": reals(work, "energies_tight.txt")}
    save("fshell_eigen.json", out)


def gen_print():
    """Spectra.Print files of the reference, kept as text (the byte layout of spectra files)."""
    work = run(open(os.path.join(HERE, "gen", "print_fmt.lua")).read(), "print_fmt.lua")
    out = {"source": "tests/golden/gen/print_fmt.lua", "HX": op(work, "HX"), "Tz": op(work, "Tz"),
           "psi": [wf(work, "psi1"), wf(work, "psi2")]}
    for k in ("lanczos", "defaults", "dense"):
        out["print_" + k] = open(os.path.join(work, "dump", "print_%s.dat" % k)).read()
    for k in ("psi1", "psi2", "Tz"):
        out["put_" + k] = open(os.path.join(work, "dump", fname(k))).read()
    save("print_fmt.json", out)


def gen_tensor():
    """Tensor spectra (3 x 3 dipole matrix) of the reference, dense and block-Lanczos branches."""
    work = run(open(os.path.join(HERE, "gen", "tensor.lua")).read(), "tensor.lua")
    out = {"source": "tests/golden/gen/tensor.lua", "psi": wf(work, "psi1")}
    for n in ("HX", "Tx", "Ty", "Tz"):
        out[n] = op(work, n)
    for k in ("dense", "dense_defaults", "lanczos", "lanczos_short", "lanczos_short_auto"):
        out["tensor_" + k] = open(os.path.join(work, "dump", "tensor_%s.dat" % k)).read()
    save("tensor.json", out)


def gen_rixs():
    """CreateResonantSpectra of the reference: dense branch (lists of T1, T2 and psi, automatic
    energy ranges, tensor form) and Krylov branch (lists, tensor form)."""
    work = run(open(os.path.join(HERE, "gen", "rixs.lua")).read(), "rixs.lua")
    out = {"source": "tests/golden/gen/rixs.lua", "psi": [wf(work, "psi1"), wf(work, "psi2")],
           "opts": {"Emin1": -5, "Emax1": 15, "NE1": 4, "Gamma1": 0.8, "Emin2": -2, "Emax2": 8, "NE2": 64,
                    "Gamma2": 0.3}}
    for n in ("H", "HX", "Tx", "Ty", "Txd", "Tyd", "Tzd"):
        out[n] = op(work, n)
    for k in ("dense_lists", "dense_auto", "dense_tensor", "dense_tensor_psi", "krylov_lists", "krylov_tensor",
              "krylov_tensor_auto", "krylov_tensor_psi", "dense_shifts", "dense_e0", "dense_res2", "krylov_res2", "dense_res1", "krylov_res1",
              "krylov_tensor_res1", "krylov_tensor_short", "krylov_tensor_short_auto"):
        out[k] = spectra(work, k + ".dat")
    save("rixs.json", out)


def gen_eigen_growth():
    """Eigensystem's basis growth beyond the start restrictions, and its confinement by the
    Restrictions option, on the 26-orbital ligand-field ion (operators of c1_lf.lua)."""
    head = open(os.path.join(HERE, "gen", "c1_lf.lua")).read().splitlines()[:44]
    tail = open(os.path.join(HERE, "gen", "eigen_growth.lua")).read()
    work = run("\n".join(head) + "\n" + tail, "eigen_growth.lua")
    out = {"source": "tests/golden/gen/c1_lf.lua:1-44 + tests/golden/gen/eigen_growth.lua",
           "start_restrictions": [["11111100000000000000000000", 6, 6], ["00000011111111110000000000", 8, 8],
                                  ["00000000000000001111111111", 10, 10]]}
    for k in ("grown", "confined", "from_states"):
        out["energies_" + k] = reals(work, "energies_%s.txt" % k)
    save("eigen_growth.json", out)


RIXS_ONEBODY_DRIVER = """dofile("common.lua")
%s
H1 = H0 + 10
T2 = ConjugateTranspose(OppT)
psi1, psi2, psi3, psi4, psi5, psi6 = psilist[1], psilist[2], psilist[3], psilist[4], psilist[5], psilist[6]
Tpsi0 = OppT * psi0  -- the zero constant of "OppT = 0 + ..." reaches psi0's determinants
for _, n in ipairs({"H0", "H1", "OppT", "T2", "psi0", "psi1", "psi2", "psi3", "psi4", "psi5", "psi6", "Tpsi0"}) do io.put("dump", n) end
function o(border)
  return {{"DenseBorder", border}, {"NE1", 5}, {"NE2", 200}, {"Emin1", 0}, {"Emax1", 10}, {"Gamma1", 0.1},
          {"Emin2", -5}, {"Emax2", 15}, {"Gamma2", 0.1}, {"NTri1", 200}, {"NTri2", 200}, {"epsilon", 1E-10}}
end
CreateResonantSpectra(H1, H0, OppT, T2, psilist, o(10000)).Print({{"file", "dump/list_dense.dat"}})
CreateResonantSpectra(H1, H0, OppT, T2, psilist, o(1)).Print({{"file", "dump/list_krylov.dat"}})
CreateResonantSpectra(H1, H0, OppT, T2, psi0, o(10000)).Print({{"file", "dump/psi0_dense.dat"}})
CreateResonantSpectra(H1, H0, OppT, T2, psi0, o(1)).Print({{"file", "dump/psi0_krylov.dat"}})
-- automatic energy ranges: the zero constant of OppT puts psi0's sector into the dense bases
CreateResonantSpectra(H1, H0, OppT, T2, psi0, {{"NE1", 5}, {"Gamma1", 0.1}, {"NE2", 200}, {"Gamma2", 0.1}}).Print({{"file", "dump/psi0_dense_auto.dat"}})
CreateSpectra(H1, OppT, psi0, {{"NE", 100}}).Print({{"file", "dump/xas_dense_auto.dat"}})
print("rixs_onebody done")
"""


def gen_rixs_onebody():
    """The one-particle RIXS model of the reference's own test (TestScripts/
    CreateResonantSpectra.Quanty, its model lines taken at run time): a list of six one-particle
    states and a superposition, both branches, on a coarser final-state grid."""
    lines = open(os.path.join(REF, "TestScripts", "CreateResonantSpectra.Quanty")).read().splitlines()
    a = next(i for i, l in enumerate(lines) if l.startswith("NF = 6"))
    b = next(i for i in range(a, len(lines)) if lines[i].startswith("print("))
    work = run(RIXS_ONEBODY_DRIVER % "\n".join(lines[a:b]), "rixs_onebody.lua")
    out = {"source": "TestScripts/CreateResonantSpectra.Quanty:%d-%d" % (a + 1, b),
           "opts": {"NE1": 5, "NE2": 200, "Emin1": 0, "Emax1": 10, "Gamma1": 0.1, "Emin2": -5, "Emax2": 15,
                    "Gamma2": 0.1, "NTri1": 200, "NTri2": 200, "Epsilon": 1e-10}}
    for n in ("H0", "H1", "OppT", "T2"):
        out[n] = op(work, n)
    out["psi0"] = wf(work, "psi0")
    out["Tpsi0"] = wf(work, "Tpsi0")
    out["psilist"] = [wf(work, "psi%d" % i) for i in range(1, 7)]
    for k in ("list_dense", "list_krylov", "psi0_dense", "psi0_krylov", "psi0_dense_auto", "xas_dense_auto"):
        out[k] = spectra(work, k + ".dat")
    save("rixs_onebody.json", out)


def gen_krylov_basis():
    """CreateSpectra with KrylovBasis: the Krylov vectors of the Lanczos branch (one pair, and
    lists at Epsilon 0) and the eigenstate energies of the dense branch."""
    head = open(os.path.join(HERE, "gen", "rixs.lua")).read().splitlines()[:28]
    tail = open(os.path.join(HERE, "gen", "krylov_basis.lua")).read()
    work = run("\n".join(head) + "\n" + tail, "krylov_basis.lua")
    out = {"source": "tests/golden/gen/rixs.lua:1-28 + tests/golden/gen/krylov_basis.lua", "Tz": op(work, "Tz")}
    n1 = int(reals(work, "count_one.txt")[0])
    out["krylov_one"] = [wf(work, "kone%d" % i) for i in range(1, n1 + 1)]
    counts = [int(x) for x in reals(work, "count_lists.txt")]
    out["krylov_lists"] = [[wf(work, "klist%dx%d" % (p, i)) for i in range(1, c + 1)] for p, c in enumerate(counts, 1)]
    out["dense_energies"] = reals(work, "dense_energies.txt")
    for k in ("lanczos_one", "lanczos_lists", "dense_states"):
        out[k] = spectra(work, k + ".dat")
    save("krylov_basis.json", out)


if __name__ == "__main__":
    if not os.path.exists(QUANTY):
        sys.exit("build the reference first: oracle/build_ref.sh")
    which = sys.argv[1:] or ["hpsi", "c0", "c1", "chain", "fshell", "print", "tensor", "rixs", "eigen_growth", "krylov_basis", "rixs_onebody"]
    for w in which:
        globals()["gen_" + w]()
