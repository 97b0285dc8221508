"""The C++ shim the integration guide gives a Quanty maintainer (its first C++ block) compiles
against the reference's own types: the block is extracted and syntax-checked together with the
reference's single translation unit (LuaInterface/main.cpp, which includes every source file),
and each qg_* function it calls is declared in include/qgpu.h and exported by libqgpu.so.
Skipped where the reference sources or g++ are absent (the reference never travels with this
repository)."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("QUANTY_REFERENCE", "/root/reference")


def _shim():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```cpp\n(.*?)```", text, re.S)[0]


def test_shim_calls_only_exported_entry_points():
    from quanty_gb300 import qgpu
    called = set(re.findall(r"\b(qg_[a-z_0-9]+)\s*\(", _shim()))
    assert called, "no qg_ call found in the shim"
    declared = set(qgpu.header_symbols())
    assert called <= declared, called - declared


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "LuaInterface", "main.cpp")) or not shutil.which("g++"),
                    reason="reference sources or g++ not available")
def test_shim_compiles_against_the_reference(tmp_path):
    (tmp_path / "shim_body.inc").write_text(_shim())
    (tmp_path / "shim_check.cpp").write_text(
        "#define main quanty_reference_main\n"
        '#include "%s"\n'
        "#undef main\n"
        "#define QUANTY_GB300\n"
        "#include <vector>\n"
        '#include "shim_body.inc"\n' % os.path.join(REF, "LuaInterface", "main.cpp"))
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.isfile(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("CUDA headers not found")
    r = subprocess.run(["g++", "-fsyntax-only", "-std=gnu++17", "-fopenmp", "-w", "-D", "LUA_USE_LINUX",
                        "-DBLASunderscore", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                        str(tmp_path / "shim_check.cpp")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
