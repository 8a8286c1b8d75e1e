"""CPU: the headers build the way a reference caller would use them, and the
programs run their host-only paths against the built libraries (no GPU call
is made): a strict C99 caller of include/gcoo.h linked with libgcoo.so alone
(what a cgo or N-API binding compiles), the ShGCOOSpDM plugin class with
libgcoo.so alone, and the SpGemmBuilder factory, which names the baseline
plugins too and so links libgcoo_baselines.so as well."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT

BUILD = os.path.join(ROOT, "gcoospdm_gb300", "_build")
INC = os.path.join(ROOT, "include")
CUDA_INC = "/usr/local/cuda/include"

C_CALLER = r"""
#include "gcoo.h"
#include <stdio.h>
int main(void)
{
    gcoo_params p;
    gcoo_handle *h = 0;
    if (gcoo_params_default(&p) != GCOO_SUCCESS || p.rows_per_group != 4)
        return 1;
    if (gcoo_abi_version() != 1)
        return 2;
    if (gcoo_create(&h, 0, 4, 4, &p) != GCOO_ERROR_INVALID_VALUE || h != 0)
        return 3;                      /* NULL dense operand: refused on the host */
    if (gcoo_build(0, 0) != GCOO_ERROR_INVALID_VALUE)
        return 4;
    printf("%s|%s\n", gcoo_status_string(GCOO_ERROR_FORMAT), gcoo_last_error());
    return 0;
}
"""

PLUGIN_CALLER = r"""
#include "ShGCOOSpDM.h"
#include <cstdio>
int main()
{
    ShGCOOSpDM g(nullptr, 4, 4);       // NULL operand: reported, nothing launched
    float c = 0.f;
    std::printf("%g\n", g.runKernelTest(nullptr, 4, 4, &c));
    return 0;
}
"""

FACTORY_CALLER = r"""
#include "SpGemmBuilder.h"
#include <cstdio>
int main()
{
    ShGemm *g = SpGemmBuilder::getShGemmAlgo(nullptr, 4, 4, "ell");
    std::printf("%s\n", g ? "object" : "null");
    return g ? 1 : 0;
}
"""


def build_and_run(tmp_path, compiler, std, src, name, libs, extra=()):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not installed")
    path = tmp_path / name
    path.write_text(src)
    exe = str(tmp_path / (name + ".bin"))
    cmd = [compiler, f"-std={std}", "-Wall", "-Wextra", "-Werror", *extra, f"-I{INC}", f"-I{CUDA_INC}", str(path),
           f"-L{BUILD}", *libs, f"-Wl,-rpath,{BUILD}", "-Wl,-rpath,/usr/local/cuda/lib64", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    return out


def test_c99_caller_links_libgcoo_alone(native, tmp_path):
    out = build_and_run(tmp_path, "gcc", "c99", C_CALLER, "caller.c", ["-lgcoo"], extra=("-pedantic",))
    assert out.returncode == 0, out.stderr
    status, message = out.stdout.strip().split("|")
    assert status == "GCOO_ERROR_FORMAT"
    assert message.startswith("GCOO_ERROR_INVALID_VALUE")   # the last failure: gcoo_build(NULL)


def test_plugin_class_links_libgcoo_alone(native, tmp_path):
    out = build_and_run(tmp_path, "g++", "c++17", PLUGIN_CALLER, "plugin.cpp", ["-lgcoo"])
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "-1"                         # -(GCOO_ERROR_INVALID_VALUE)
    assert "dense matrix pointer is NULL" in out.stderr


def test_factory_links_both_libraries(native, tmp_path):
    if not os.path.exists(os.path.join(BUILD, "libgcoo_baselines.so")):
        pytest.skip("baselines library not built")
    out = build_and_run(tmp_path, "g++", "c++17", FACTORY_CALLER, "factory.cpp", ["-lgcoo_baselines", "-lgcoo"])
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "null"                       # unknown name: NULL, as in the reference
