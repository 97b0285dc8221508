"""The Quanty shim (integration/qgpu_shim.cpp) compiles against the reference's own types: it is
syntax-checked together with the reference's single translation unit (LuaInterface/main.cpp,
which includes every source file), and every qg_* function it calls is declared in
include/qgpu.h.  The reference tree is located through QUANTY_REFERENCE, else the copy staged in
baseline/_ref by oracle/stage_ref.sh; the compile check is skipped where neither exists (the
reference never travels with this repository) or g++ is absent.  The patch script is checked
to find every dispatcher it hooks."""
import os
import re
import shutil
import subprocess
import sys

import pytest

from conftest import ROOT

SHIM = os.path.join(ROOT, "integration", "qgpu_shim.cpp")


def _reference():
    for d in (os.environ.get("QUANTY_REFERENCE"), os.path.join(ROOT, "baseline", "_ref")):
        if d and os.path.isfile(os.path.join(d, "LuaInterface", "main.cpp")):
            return d
    return None


def test_shim_calls_only_exported_entry_points():
    from quanty_gb300 import qgpu
    called = set(re.findall(r"\b(qg_[a-z_0-9]+)\s*\(", open(SHIM).read()))
    assert called, "no qg_ call found in the shim"
    declared = set(qgpu.header_symbols())
    assert called <= declared, called - declared


@pytest.mark.skipif(_reference() is None or not shutil.which("g++"), reason="reference sources or g++ not available")
def test_shim_compiles_against_the_reference(tmp_path):
    ref = _reference()
    (tmp_path / "shim_check.cpp").write_text(
        "#define main quanty_reference_main\n"
        '#include "%s"\n'
        "#undef main\n"
        "#define QUANTY_GB300\n"
        '#include "%s"\n' % (os.path.join(ref, "LuaInterface", "main.cpp"), SHIM))
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.isfile(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("CUDA headers not found")
    r = subprocess.run(["g++", "-fsyntax-only", "-std=gnu++17", "-fopenmp", "-w", "-D", "LUA_USE_LINUX",
                        "-DBLASunderscore", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                        str(tmp_path / "shim_check.cpp")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(_reference() is None, reason="reference sources not available")
def test_patch_finds_every_dispatcher(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "integration"))
    import build_quanty_gb300 as b
    b.patch(_reference(), str(tmp_path / "src"))
    text = open(tmp_path / "src" / "Core" / "Core.cpp").read()
    assert text.startswith('#ifdef QUANTY_GB300\n#include "QGpu.cpp"')
    hooked = open(tmp_path / "src" / "Core" / "OperatorWaveFunction.cpp").read() + \
        open(tmp_path / "src" / "Core" / "Lanczos.cpp").read()
    for _, _, call in b.HOOKS:
        assert call in hooked, call
