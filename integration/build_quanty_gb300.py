"""Build Quanty with its H*psi path routed through libqgpu (the drop-in, end to end).

    python integration/build_quanty_gb300.py <reference-dir> [<out-dir>]

What a Quanty maintainer does, applied to a copy of the reference sources (the reference tree
itself is never written): add integration/qgpu_shim.cpp as Core/QGpu.cpp, include it at the top
of Core/Core.cpp under QUANTY_GB300, put a guarded early return at the top of each routed
dispatcher, then compile the one translation unit with -DQUANTY_GB300 against include/qgpu.h and
link quanty_gb300/libqgpu.so.  The BLAS/LAPACK and seed-pinning headers are oracle/build_ref.sh's.
The binary lands in <out-dir>/Quanty_gb300 (default integration/_build/).
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# (file, dispatcher signature start, call placed at the top of its body)
HOOKS = [
    ("Core/OperatorWaveFunction.cpp",
     "uint32_t OperatorPsiConserveBasisPreAllocated(const OperatorType *O, const WaveFunctionType *psi,",
     "QGpuOperatorPsiConserveBasisPreAllocated(O, psi, Opsi)"),
    ("Core/OperatorWaveFunction.cpp",
     "uint32_t OperatorPsiRestricted(const OperatorType &O, const WaveFunctionType &psi, WaveFunctionType * const Opsi,",
     "QGpuOperatorPsiRestricted(O, psi, Opsi, &restrictions)"),
    ("Core/OperatorWaveFunction.cpp",
     "uint32_t OperatorPsi(const OperatorType &O, const WaveFunctionType &psi, WaveFunctionType * const Opsi)",
     "QGpuOperatorPsi(O, psi, Opsi)"),
    ("Core/Lanczos.cpp",
     "uint32_t LanczosTriDiagonalizeRestricted(const OperatorType H, WaveFunctionType psi, DeterminantRestrictionType Restrictions,",
     "QGpuLanczosTriDiagonalizeRestricted(H, psi, &Restrictions, epsilon, M, Gamma)"),
    ("Core/Lanczos.cpp",
     "uint32_t LanczosTriDiagonalize(const OperatorType H, WaveFunctionType psi, double epsilon, TriDiagonalMatrixType * const M, double Gamma)",
     "QGpuLanczosTriDiagonalize(H, psi, epsilon, M, Gamma)"),
]


def patch(src, dst):
    if os.path.exists(dst):
        shutil.rmtree(dst)
    shutil.copytree(src, dst)
    shutil.copy(os.path.join(HERE, "qgpu_shim.cpp"), os.path.join(dst, "Core", "QGpu.cpp"))
    core = os.path.join(dst, "Core", "Core.cpp")
    text = open(core).read()
    open(core, "w").write('#ifdef QUANTY_GB300\n#include "QGpu.cpp"\n#endif\n' + text)
    for rel, sig, call in HOOKS:
        path = os.path.join(dst, rel)
        text = open(path).read()
        # the definition (a signature line followed by its opening brace), not a prototype
        m = re.search(re.escape(sig) + r"[^;{]*\{", text)
        if not m:
            raise RuntimeError("dispatcher not found in %s: %s" % (rel, sig))
        hook = ("\n#ifdef QUANTY_GB300\n  { uint32_t qgpu_r = %s; if (qgpu_r != 2) return qgpu_r; }\n#endif" % call)
        text = text[:m.end()] + hook + text[m.end():]
        open(path, "w").write(text)


def build(ref, out):
    work = os.path.join(out, "src")
    patch(ref, work)
    from quanty_gb300 import build as qb
    lib = qb.build()
    r = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), ref, "headers"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    refout = os.path.join(ROOT, "oracle", "_ref")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(lib)
    cmd = ["g++", os.path.join(work, "LuaInterface", "main.cpp"), "-include", os.path.join(refout, "blas_names.h"),
           "-include", os.path.join(refout, "pin_seed.h"), "-D", "LUA_USE_LINUX", "-DBLASunderscore",
           "-DQUANTY_GB300", "-O2", "-fopenmp", "-w", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), "-L", refout, "-lscipyob", "-L", libdir, "-lqgpu",
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + ":".join([libdir, os.path.join(cuda, "lib64"),
                                     os.path.dirname(os.path.realpath(os.path.join(refout, "libscipyob.so")))]),
           "-o", os.path.join(out, "Quanty_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + r.stderr[-4000:])
    return os.path.join(out, "Quanty_gb300")


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    ref = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(HERE, "_build")
    os.makedirs(out, exist_ok=True)
    print(build(ref, out))
