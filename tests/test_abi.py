"""CPU: the C-ABI library loads, exports every symbol include/gcoo.h declares,
and rejects invalid arguments on the host (no GPU needed for any of this)."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def header_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gcoo_[a-z0-9_]+)\s*\(", text)
    typedef_fns = set(re.findall(r"\(\*\s*(gcoo_[a-z0-9_]+)\)", text))
    return sorted(set(n for n in names if n not in typedef_fns))


def test_header_and_binding_agree(native):
    declared = header_functions(os.path.join(ROOT, "include", "gcoo.h"))
    assert set(declared) == set(native.EXPORTS), set(declared) ^ set(native.EXPORTS)


def test_library_exports_every_declared_symbol(native):
    L = native.lib()
    for name in header_functions(os.path.join(ROOT, "include", "gcoo.h")):
        assert hasattr(L, name), name


def test_version_and_strings(native):
    L = native.lib()
    assert L.gcoo_abi_version() == 1
    assert L.gcoo_status_string(0) == b"GCOO_SUCCESS"
    assert L.gcoo_status_string(7) == b"GCOO_ERROR_TIMEOUT"


def test_params_default_is_reference_constant(native):
    p = native.Params()
    assert native.lib().gcoo_params_default(C.byref(p)) == 0
    assert p.rows_per_group == 4  # src/constants.h:4 COLUMN_PER_GROUP
    assert p.fp32_sum == 0  # the sequential chain (the reference's order) by default


@pytest.mark.parametrize("fp32_sum,err", [(0, 0), (1, 0), (2, 1), (-1, 1)])
def test_create_checks_fp32_sum(native, fp32_sum, err):
    L = native.lib()
    h = C.c_void_p()
    p = native.Params()
    L.gcoo_params_default(C.byref(p))
    p.fp32_sum = fp32_sum
    st = L.gcoo_create(C.byref(h), C.c_void_p(0x1000), 8, 8, C.byref(p))  # the operand is not read here
    assert st == err
    if h.value:
        assert L.gcoo_destroy(h) == 0


@pytest.mark.parametrize("m,k,rpg,err", [(0, 5, 4, 1), (5, 0, 4, 1), (-1, 5, 4, 1), (1 << 31, 5, 4, 1),
                                         (5, 5, 3, 1), (5, 5, 64, 1), (5, 5, 0, 1)])
def test_create_rejects_bad_arguments(native, m, k, rpg, err):
    L = native.lib()
    h = C.c_void_p()
    p = native.Params()
    L.gcoo_params_default(C.byref(p))
    p.rows_per_group = rpg
    st = L.gcoo_create(C.byref(h), C.c_void_p(0x1000), m, k, C.byref(p))
    assert st == err
    assert not h.value
    assert L.gcoo_last_error()


def test_null_pointers_rejected(native):
    L = native.lib()
    h = C.c_void_p()
    assert L.gcoo_create(C.byref(h), None, 4, 4, None) == 1
    assert L.gcoo_build(None, None) == 1
    assert L.gcoo_spdm(None, None, 4, None, None) == 1
    assert L.gcoo_export(None, None) == 1
    assert L.gcoo_destroy(None) == 0


def test_not_built_and_bad_n(native):
    L = native.lib()
    h = C.c_void_p()
    assert L.gcoo_create(C.byref(h), C.c_void_p(0x1000), 8, 8, None) == 0
    try:
        # multiply before build: rejected on the host, nothing launched
        assert L.gcoo_spdm(h, C.c_void_p(0x2000), 4, C.c_void_p(0x3000), None) == 4
        assert L.gcoo_spdm_ex(h, C.c_void_p(0x2000), 4, C.c_void_p(0x3000), 1, None) == 4
        v = native.View()
        assert L.gcoo_export(h, C.byref(v)) == 4
        assert L.gcoo_multiply_by(h, C.c_void_p(0x2000), 0, C.c_void_p(0x3000), None) == 1
    finally:
        L.gcoo_destroy(h)


def test_allocator_hook_validation(native):
    L = native.lib()
    assert L.gcoo_set_allocator(native._native.ALLOC_FN(lambda n, c: None), native._native.FREE_FN(0), None) == 1
    assert L.gcoo_set_allocator(native._native.ALLOC_FN(0), native._native.FREE_FN(0), None) == 0


def test_product_path_has_no_oracle_dependency():
    """Nothing under the package or the C sources may reach the oracle."""
    pkg = os.path.join(ROOT, "gcoospdm_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".cuh", ".hpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "liboracle" not in text and "ref_emu" not in text, f


def test_python_fails_loudly_without_library(tmp_path, monkeypatch):
    import gcoospdm_gb300._native as nat
    monkeypatch.setattr(nat, "_lib", None)
    monkeypatch.setattr(nat, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(nat.NativeLibraryError):
        nat.lib()
