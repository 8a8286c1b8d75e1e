"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle (gcoo_oracle.c)
and, where it was built, of the reference kernels run under the host emulator
(ref_emu). Only the tests, the smoke check and the CPU-baseline legs of the
benchmark import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libref_emu.so")

_i64 = C.c_int64
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

_lib = None
_ref = None


def build() -> None:
    """Compile the oracle, and the reference kernels (host emulation and
    sm_103a cubin) when GCOO_REFERENCE_TREE names a reference checkout."""
    cmd = ["make", "-s", "-C", _HERE, "-f", "Makefile"]
    tree = os.environ.get("GCOO_REFERENCE_TREE", "")
    if tree:
        cmd.append(f"REF={tree}")
    subprocess.run(cmd, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        L.orc_group_count.argtypes = [_f32p, _i64, _i64, C.c_int, _i32p, C.c_int]
        L.orc_group_count.restype = _i64
        L.orc_exclusive_scan.argtypes = [_i32p, _i64, _i32p]
        L.orc_scatter.argtypes = [_f32p, _i64, _i64, C.c_int, _i32p, _f32p, _i32p, _i32p, C.c_int]
        L.orc_spdm.argtypes = [_i64, _i64, C.c_int, _i32p, _i32p, _f32p, _i32p, _i32p, _f32p, _i64, _f32p, C.c_int]
        L.orc_spdm_f64.argtypes = [_i64, _i64, C.c_int, _i32p, _i32p, _f32p, _i32p, _i32p, _f32p, _i64, _f64p, C.c_int]
        L.orc_dense_gemm_f64.argtypes = [_f32p, _f32p, _i64, _i64, _i64, _f64p, C.c_int]
        L.orc_rel_fro.argtypes = [_f32p, _f64p, _i64]
        L.orc_rel_fro.restype = C.c_double
        L.orc_multiply_by.argtypes = [_f32p, _i64, _i64, C.c_int, _f32p, _i64, _f32p, C.c_int]
        L.orc_multiply_by.restype = _i64
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(_REF)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(_REF)
        R.ref_emu_convert.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _i32p, _i32p, _f32p, _i32p, _i32p, C.c_longlong]
        R.ref_emu_convert.restype = C.c_longlong
        R.ref_emu_spdm.argtypes = [_f32p, _i32p, _i32p, _i32p, _i32p, C.c_int, C.c_int, _f32p, C.c_int, _f32p]
        R.ref_emu_column_per_group.restype = C.c_int
        R.ref_emu_bs.restype = C.c_int
        _ref = R
    return _ref


class Gcoo:
    """Host GCOO arrays in the reference's layout."""

    def __init__(self, m, k, cpg, groupIndex, nnzPerGroup, vals, rows, cols):
        self.m, self.k, self.cpg = m, k, cpg
        self.groupIndex, self.nnzPerGroup = groupIndex, nnzPerGroup
        self.vals, self.rows, self.cols = vals, rows, cols

    @property
    def nnz(self) -> int:
        return int(self.vals.size)

    @property
    def n_group(self) -> int:
        return (self.m + self.cpg - 1) // self.cpg


def convert(A: np.ndarray, cpg: int = 4, nthreads: int = 0) -> Gcoo:
    """Dense -> GCOO (count, exclusive scan, stable scatter)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    m, k = A.shape
    ng = (m + cpg - 1) // cpg
    npg = np.zeros(ng + 1, dtype=np.int32)
    nnz = lib().orc_group_count(A, m, k, cpg, npg, nthreads)
    if nnz < 0:
        raise ValueError("nnz does not fit the int32 GCOO format")
    gi = np.zeros(ng + 1, dtype=np.int32)
    lib().orc_exclusive_scan(npg, ng + 1, gi)
    vals = np.empty(max(nnz, 1), dtype=np.float32)
    rows = np.empty(max(nnz, 1), dtype=np.int32)
    cols = np.empty(max(nnz, 1), dtype=np.int32)
    lib().orc_scatter(A, m, k, cpg, gi, vals, rows, cols, nthreads)
    return Gcoo(m, k, cpg, gi, npg, vals[:nnz], rows[:nnz], cols[:nnz])


def _arr(x, dt):
    x = np.ascontiguousarray(x, dtype=dt)
    return x if x.size else np.zeros(1, dtype=dt)


def spdm(g: Gcoo, B: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """FP32 GCOO x dense with the reference kernel's accumulation order."""
    B = np.ascontiguousarray(B, dtype=np.float32)
    n = B.shape[1]
    Cm = np.empty((g.m, n), dtype=np.float32)
    if g.m == 0 or n == 0:
        return Cm
    lib().orc_spdm(g.m, g.k, g.cpg, g.groupIndex, g.nnzPerGroup, _arr(g.vals, np.float32),
                   _arr(g.rows, np.int32), _arr(g.cols, np.int32), _arr(B, np.float32), n, Cm, nthreads)
    return Cm


def spdm_f64(g: Gcoo, B: np.ndarray, nthreads: int = 0) -> np.ndarray:
    B = np.ascontiguousarray(B, dtype=np.float32)
    n = B.shape[1]
    Cm = np.empty((g.m, n), dtype=np.float64)
    if g.m == 0 or n == 0:
        return Cm
    lib().orc_spdm_f64(g.m, g.k, g.cpg, g.groupIndex, g.nnzPerGroup, _arr(g.vals, np.float32),
                       _arr(g.rows, np.int32), _arr(g.cols, np.int32), _arr(B, np.float32), n, Cm, nthreads)
    return Cm


def dense_gemm_f64(A: np.ndarray, B: np.ndarray, nthreads: int = 0) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    m, k = A.shape
    n = B.shape[1]
    Cm = np.empty((m, n), dtype=np.float64)
    lib().orc_dense_gemm_f64(A, B, m, k, n, Cm, nthreads)
    return Cm


def rel_fro(Cm: np.ndarray, C64: np.ndarray) -> float:
    Cm = np.ascontiguousarray(Cm, dtype=np.float32).ravel()
    C64 = np.ascontiguousarray(C64, dtype=np.float64).ravel()
    return float(lib().orc_rel_fro(_arr(Cm, np.float32), _arr(C64, np.float64), Cm.size))


def multiply_by(A: np.ndarray, B: np.ndarray, cpg: int = 4, nthreads: int = 0) -> np.ndarray:
    """Host convert + multiply (the CPU restatement of mutiplyBy)."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    m, k = A.shape
    n = B.shape[1]
    Cm = np.empty((m, n), dtype=np.float32)
    r = lib().orc_multiply_by(A, m, k, cpg, B, n, Cm, nthreads)
    if r < 0:
        raise RuntimeError("oracle multiply_by failed")
    return Cm


def max_threads() -> int:
    return int(lib().orc_max_threads())


# --- the reference kernels under the host emulator (only where built) -------

def ref_convert(A: np.ndarray, cpg: int = 4) -> Gcoo:
    A = np.ascontiguousarray(A, dtype=np.float32)
    m, k = A.shape
    ng = (m + cpg - 1) // cpg
    cap = max(m * k, 1)
    gi = np.zeros(ng + 1, dtype=np.int32)
    npg = np.zeros(ng + 1, dtype=np.int32)
    vals = np.zeros(cap, dtype=np.float32)
    rows = np.zeros(cap, dtype=np.int32)
    cols = np.zeros(cap, dtype=np.int32)
    nnz = ref().ref_emu_convert(_arr(A, np.float32), m, k, cpg, gi, npg, vals, rows, cols, cap)
    if nnz < 0:
        raise RuntimeError(f"ref_emu_convert failed ({nnz})")
    return Gcoo(m, k, cpg, gi, npg, vals[:nnz].copy(), rows[:nnz].copy(), cols[:nnz].copy())


def ref_spdm(g: Gcoo, B: np.ndarray) -> np.ndarray:
    if g.cpg != ref().ref_emu_column_per_group():
        raise ValueError("the reference multiply is compiled for COLUMN_PER_GROUP=%d" % ref().ref_emu_column_per_group())
    B = np.ascontiguousarray(B, dtype=np.float32)
    n = B.shape[1]
    Cm = np.zeros((g.m, n), dtype=np.float32)
    ref().ref_emu_spdm(_arr(g.vals, np.float32), _arr(g.cols, np.int32), _arr(g.rows, np.int32),
                       g.groupIndex, g.nnzPerGroup, g.m, g.k, _arr(B, np.float32), n, Cm)
    return Cm


# --- the reference kernels compiled for sm_103a (only where the cubin exists) -

_REFGPU_CUBIN = os.path.join(_HERE, "_ref", "ref_gcoo_sm103a.cubin")
_REFGPU_RUNNER = os.path.join(_HERE, "_build", "libref_gpu_runner.so")
_refgpu = None


def refgpu_available() -> bool:
    """The reference's own kernels, compiled from its source into a cubin where
    the reference tree exists; the runner is built wherever CUDA is."""
    return os.path.exists(_REFGPU_CUBIN)


def refgpu():
    """Load the runner and the cubin into the current CUDA context."""
    global _refgpu
    if _refgpu is None:
        if not os.path.exists(_REFGPU_RUNNER):
            build()
        R = C.CDLL(_REFGPU_RUNNER)
        R.refgpu_error.restype = C.c_char_p
        R.refgpu_load.argtypes = [C.c_char_p]
        R.refgpu_count_scan.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_uint64, C.c_uint64,
                                        C.POINTER(C.c_longlong)]
        R.refgpu_scatter.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int] + [C.c_uint64] * 5
        R.refgpu_spdm.argtypes = [C.c_uint64] * 5 + [C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_uint64]
        if R.refgpu_load(_REFGPU_CUBIN.encode()) != 0:
            raise RuntimeError("reference cubin: " + R.refgpu_error().decode())
        _refgpu = R
    return _refgpu


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference kernels: " + refgpu().refgpu_error().decode())


def refgpu_convert(dA, cpg: int = 4) -> dict:
    """The reference conversion on the GPU over a device tensor A (m x k FP32).
    Returns device tensors groupIndex, nnzPerGroup (nGroup+1 each), vals, rows,
    cols (nnz each) and nnz."""
    import torch
    m, k = int(dA.shape[0]), int(dA.shape[1])
    ng = (m + cpg - 1) // cpg
    R = refgpu()
    gi = torch.zeros(2 * (ng + 1), dtype=torch.int32, device=dA.device)  # one allocation, like the reference
    nnz = C.c_longlong(0)
    _check(R.refgpu_count_scan(cpg, dA.data_ptr(), m, k, gi.data_ptr(), gi[ng + 1:].data_ptr(), C.byref(nnz)))
    n = int(nnz.value)
    vals = torch.empty(max(n, 1), dtype=torch.float32, device=dA.device)
    rc = torch.empty(2 * max(n, 1), dtype=torch.int32, device=dA.device)
    _check(R.refgpu_scatter(cpg, dA.data_ptr(), m, k, gi.data_ptr(), gi[ng + 1:].data_ptr(), vals.data_ptr(),
                            rc.data_ptr(), rc[max(n, 1):].data_ptr()))
    return {"groupIndex": gi[:ng + 1], "nnzPerGroup": gi[ng + 1:], "vals": vals[:n], "rows": rc[:n],
            "cols": rc[max(n, 1):max(n, 1) + n], "nnz": n, "m": m, "k": k, "cpg": cpg,
            "_keep": (gi, vals, rc)}


def refgpu_column_per_group() -> int:
    return int(refgpu().refgpu_column_per_group())


def refgpu_spdm(g: dict, dB, dC) -> None:
    """The reference multiply kernel on the GPU (compiled CPG and BS)."""
    if g["cpg"] != refgpu_column_per_group():
        raise ValueError("the reference multiply is compiled for COLUMN_PER_GROUP=%d" % refgpu_column_per_group())
    gi, vals, rc = g["_keep"]
    n = int(dB.shape[1])
    nn = max(g["nnz"], 1)
    _check(refgpu().refgpu_spdm(vals.data_ptr(), rc[nn:].data_ptr(), rc.data_ptr(), g["groupIndex"].data_ptr(),
                                g["nnzPerGroup"].data_ptr(), g["m"], g["k"], dB.data_ptr(), n, dC.data_ptr()))
