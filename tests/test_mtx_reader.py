"""CPU: the Matrix Market reader behind the driver's -file= input
(gcoo_read_matrix_market, host code). Checked against the reference's own
rules restated here (src/MatrixReader.cpp:11-84): 1-based coordinates, a
banner without "general" mirrors every entry, a later line overwrites an
earlier one in the dense buffer; plus this library's two stated
differences (pattern entries 1.0, skew-symmetric mirrors negated) and its
errors. The driver's refusals run here too (they precede any CUDA call)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

MAIN = os.path.join(ROOT, "gcoospdm_gb300", "_build", "gcoo_main")


def write(tmp_path, text, name="m.mtx"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def dense_from_triplets(rows, cols, vals, m, k):
    D = np.zeros((m, k), np.float32)
    for r, c, v in zip(rows, cols, vals):   # file order: a later triplet overwrites
        D[r, c] = v
    return D


def reference_dense(text):
    """The reference reader's dense buffer for a real-valued file: the first
    line decides general vs mirrored, '%' lines are skipped, then the size
    line and 1-based 'row col value' lines, each written (and, unless
    general, also written at (col, row)) in order."""
    lines = text.splitlines()
    general = "general" in lines[0]
    i = 1
    while lines[i].startswith("%"):
        i += 1
    m, k, _ = (int(x) for x in lines[i].split())
    D = np.zeros((m, k), np.float32)
    for ln in lines[i + 1:]:
        if not ln.strip():
            continue
        r, c, v = ln.split()
        r, c, v = int(r) - 1, int(c) - 1, np.float32(float(v))
        D[r, c] = v
        if not general:
            D[c, r] = v
    return D


def test_general_real_with_comments_duplicates_and_zeros(native, tmp_path):
    text = ("%%MatrixMarket matrix coordinate real general\n% a comment\n%\n4 5 6\n"
            "1 1 1.5\n4 5 -2.25e-3\n2 3 7\n2 3 -7\n3 2 0\n1 5 1e-40\n")
    rows, cols, vals, m, k = native.read_matrix_market(write(tmp_path, text))
    assert (m, k) == (4, 5)
    assert rows.tolist() == [0, 3, 1, 1, 2, 0] and cols.tolist() == [0, 4, 2, 2, 1, 4]
    assert vals.dtype == np.float32 and vals[5] == np.float32(1e-40)   # subnormal kept as written
    assert np.array_equal(dense_from_triplets(rows, cols, vals, m, k), reference_dense(text))


def test_symmetric_mirrors_after_each_entry(native, tmp_path):
    text = "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 2\n3 1 -1\n2 2 4\n3 2 0.5\n"
    rows, cols, vals, m, k = native.read_matrix_market(write(tmp_path, text))
    assert list(zip(rows.tolist(), cols.tolist(), vals.tolist())) == [
        (0, 0, 2.0), (2, 0, -1.0), (0, 2, -1.0), (1, 1, 4.0), (2, 1, 0.5), (1, 2, 0.5)]
    D = dense_from_triplets(rows, cols, vals, m, k)
    assert np.array_equal(D, D.T) and np.array_equal(D, reference_dense(text))


def test_random_files_match_the_reference_rules(native, tmp_path):
    rng = np.random.default_rng(5)
    for sym in ("general", "symmetric"):
        for trial in range(4):
            n = int(rng.integers(5, 40))
            e = int(rng.integers(1, 3 * n))
            r = rng.integers(1, n + 1, size=e)
            c = rng.integers(1, n + 1, size=e)
            if sym == "symmetric":
                r, c = np.maximum(r, c), np.minimum(r, c)   # lower triangle, as the format stores it
            v = rng.standard_normal(e).astype(np.float32)
            v[rng.random(e) < 0.1] = 0.0
            body = "".join(f"{a} {b} {x:.9g}\n" for a, b, x in zip(r, c, v))
            text = f"%%MatrixMarket matrix coordinate real {sym}\n{n} {n} {e}\n" + body
            rows, cols, vals, m, k = native.read_matrix_market(write(tmp_path, text, f"{sym}{trial}.mtx"))
            assert np.array_equal(dense_from_triplets(rows, cols, vals, m, k), reference_dense(text)), (sym, trial)


def test_pattern_integer_and_skew(native, tmp_path):
    rows, cols, vals, _, _ = native.read_matrix_market(
        write(tmp_path, "%%MatrixMarket matrix coordinate pattern general\n2 3 2\n1 3\n2 1\n"))
    assert vals.tolist() == [1.0, 1.0] and rows.tolist() == [0, 1] and cols.tolist() == [2, 0]
    _, _, vals, _, _ = native.read_matrix_market(
        write(tmp_path, "%%MatrixMarket matrix coordinate integer general\n2 2 1\n2 2 -17\n", "i.mtx"))
    assert vals.tolist() == [-17.0]
    rows, cols, vals, _, _ = native.read_matrix_market(
        write(tmp_path, "%%MatrixMarket matrix coordinate real skew-symmetric\n3 3 1\n3 1 2.5\n", "s.mtx"))
    assert list(zip(rows.tolist(), cols.tolist(), vals.tolist())) == [(2, 0, 2.5), (0, 2, -2.5)]
    # an empty matrix
    rows, _, _, m, k = native.read_matrix_market(
        write(tmp_path, "%%MatrixMarket matrix coordinate real general\n7 9 0\n", "e.mtx"))
    assert rows.size == 0 and (m, k) == (7, 9)


def test_hermitian_real_reads_like_symmetric(native, tmp_path):
    """For real, integer and pattern fields a Hermitian matrix is a symmetric
    one (the reference mirrors every banner without "general")."""
    body = "3 3 3\n1 1 2\n3 1 -1.5\n3 2 4\n"
    herm = native.read_matrix_market(write(tmp_path, "%%MatrixMarket matrix coordinate real hermitian\n" + body, "h.mtx"))
    sym = native.read_matrix_market(write(tmp_path, "%%MatrixMarket matrix coordinate real symmetric\n" + body, "s.mtx"))
    for a, b in zip(herm[:3], sym[:3]):
        assert np.array_equal(a, b)
    text = "%%MatrixMarket matrix coordinate real hermitian\n" + body
    assert np.array_equal(dense_from_triplets(*herm), reference_dense(text))
    rows, cols, vals, _, _ = native.read_matrix_market(
        write(tmp_path, "%%MatrixMarket matrix coordinate pattern hermitian\n2 2 1\n2 1\n", "hp.mtx"))
    assert list(zip(rows.tolist(), cols.tolist(), vals.tolist())) == [(1, 0, 1.0), (0, 1, 1.0)]


_ALLOC_CHILD = r"""
import ctypes as C, os, resource, sys
sys.path.insert(0, sys.argv[1])
from gcoospdm_gb300 import _native as nat
L = nat.lib()
# the library is loaded; now cap the address space a little above what is mapped
with open("/proc/self/status") as f:
    vm = next(int(l.split()[1]) for l in f if l.startswith("VmSize:")) * 1024
resource.setrlimit(resource.RLIMIT_AS, (vm + (40 << 20), resource.RLIM_INFINITY))
m, k, n = C.c_int64(), C.c_int64(), C.c_int64()
r, c = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
v = C.POINTER(C.c_float)()
st = L.gcoo_read_matrix_market(os.fsencode(sys.argv[2]), C.byref(m), C.byref(k), C.byref(n), C.byref(r),
                               C.byref(c), C.byref(v))
print(st, bool(r), L.gcoo_last_error().decode())
"""


def test_host_allocation_failure_returns_a_status(native, tmp_path):
    """The reader's vectors cannot grow under an address-space limit: the
    entry point returns GCOO_ERROR_ALLOC (no C++ exception ends the process).
    A symmetric file whose size line promises 4 M entries makes the reader
    reserve 3 x 32 MB up front; the child process allows 40 MB more than it
    has mapped."""
    p = write(tmp_path, "%%MatrixMarket matrix coordinate real symmetric\n9 9 4194304\n1 1 1\n", "big.mtx")
    out = subprocess.run(["python", "-c", _ALLOC_CHILD, ROOT, p], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    status, got_rows, msg = out.stdout.split(" ", 2)
    assert int(status) == 2 and got_rows == "False" and "allocation" in msg


@pytest.mark.parametrize("text,status", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", 5),
    ("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", 5),
    ("not a banner\n2 2 1\n1 1 1\n", 1),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n", 1),    # row out of range
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1\n", 1),    # 0 in a 1-based file
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n", 1),    # truncated
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n2 2 2\n", 1),  # more than stated
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n", 1),      # no value
    ("%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 1 1\n", 1),  # symmetric, not square
    ("%%MatrixMarket matrix coordinate real general\n", 1),                  # no size line
])
def test_errors(native, tmp_path, text, status):
    with pytest.raises(native.GcooError) as e:
        native.read_matrix_market(write(tmp_path, text))
    assert e.value.status == status


def test_missing_file(native, tmp_path):
    with pytest.raises(native.GcooError) as e:
        native.read_matrix_market(str(tmp_path / "absent.mtx"))
    assert e.value.status == 1 and "cannot open" in str(e.value)


def test_driver_refuses_bad_files_before_any_device_work(native, tmp_path):
    if not os.path.exists(MAIN):
        pytest.skip("driver not built")
    out = subprocess.run([MAIN, f"-file={tmp_path / 'absent.mtx'}"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 2 and "cannot open" in out.stderr
    p = write(tmp_path, "%%MatrixMarket matrix coordinate real general\n2 3 1\n1 1 1\n", "r.mtx")
    out = subprocess.run([MAIN, f"-file={p}"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 2 and "square" in out.stderr
