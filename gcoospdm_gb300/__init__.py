"""GB300-native GCOO sparse x dense multiply, a drop-in for the -algo=gcoospdm
path of hclhkbu/gcoospdm.

Python face of the C ABI in include/gcoo.h (libgcoo.so). Device buffers are
torch CUDA tensors (float32, row-major, contiguous); streams default to
torch's current stream. The reference's plugin surface is mirrored by
``ShGemm`` / ``ShGCOOSpDM`` / ``SpGemmBuilder`` (src/ShGemm.h,
src/ShGCOOSpDM.h, src/SpGemmBuilder.h of the reference) with the same names,
argument meaning and return values.

Orientation (the reference kernel's row-major reading): A is m x k (the sparse
operand, given dense), B is k x n, C = A @ B is m x n.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

from ._native import (  # noqa: F401
    BASELINES_PATH, ENGINE, EXPORTS, LIB_PATH, MAIN_PATH, PREC, GcooError, NativeLibraryError, Params,
    Problem, View, build, check, lib,
)

__all__ = ["GcooHandle", "GcooBatch", "ShGemm", "ShGCOOSpDM", "SpGemmBuilder", "GcooError",
           "NativeLibraryError", "build", "lib", "autotune_save", "autotune_load", "autotune_clear"]


def _torch():
    import torch
    return torch


def _stream_ptr(stream) -> Optional[int]:
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def _check_f32(t, name, shape=None):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")


class _DevArray:
    """__cuda_array_interface__ wrapper: a torch view of library-owned memory.
    It holds its owner (the handle), and the tensor made from it holds the
    wrapper, so the handle's arrays outlive every view of them; a later build
    may still move them (views are of the arrays as built)."""

    def __init__(self, ptr, n, typestr, owner=None):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": typestr, "data": (int(ptr or 0), False),
                                         "version": 3, "strides": None}


def _view_tensor(ptr, n, typestr, owner=None):
    torch = _torch()
    if n == 0 or not ptr:
        return torch.empty(0, dtype=torch.float32 if typestr == "<f4" else torch.int32, device="cuda")
    return torch.as_tensor(_DevArray(ptr, n, typestr, owner), device="cuda")


FP32_ORDER = {"auto": 0, "rows": 1, "groups": 2}
FP32_SUM = {"chain": 0, "split": 1}


def make_params(rows_per_group=4, vec=0, warps=0, col_warps=0, engine="auto", depth=0, fp32_order="auto",
                fp32_sum="chain") -> Params:
    p = Params()
    check(lib().gcoo_params_default(C.byref(p)))
    p.rows_per_group = rows_per_group
    p.vec, p.warps, p.col_warps, p.depth = vec, warps, col_warps, depth
    p.fp32_order = FP32_ORDER[fp32_order] if isinstance(fp32_order, str) else int(fp32_order)
    p.fp32_sum = FP32_SUM[fp32_sum] if isinstance(fp32_sum, str) else int(fp32_sum)
    p.engine = ENGINE[engine] if isinstance(engine, str) else int(engine)
    return p


class GcooHandle:
    """One sparse operand: conversion state plus the multiply entry points."""

    def __init__(self, A, rows_per_group: int = 4, vec: int = 0, warps: int = 0, col_warps: int = 0,
                 engine: str = "auto", depth: int = 0, fp32_order: str = "auto", fp32_sum: str = "chain"):
        _check_f32(A, "A")
        if A.dim() != 2:
            raise ValueError("A must be 2-D")
        self._A = A  # keeps the dense operand alive while the handle may read it
        self.m, self.k = int(A.shape[0]), int(A.shape[1])
        self._h = C.c_void_p()
        p = make_params(rows_per_group, vec, warps, col_warps, engine, depth, fp32_order, fp32_sum)
        check(lib().gcoo_create(C.byref(self._h), C.c_void_p(A.data_ptr()), self.m, self.k, C.byref(p)))
        self.rows_per_group = rows_per_group

    @classmethod
    def from_coo(cls, rows, cols, vals, m: int, k: int, rows_per_group: int = 4, **params) -> "GcooHandle":
        """Handle built from device COO triplets (int32 rows/cols, float32 vals),
        without a dense m x k buffer; duplicates: the later triplet wins."""
        torch = _torch()
        for t, dt in ((rows, torch.int32), (cols, torch.int32), (vals, torch.float32)):
            if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != dt or not t.is_contiguous():
                raise ValueError("rows/cols must be int32 and vals float32 contiguous CUDA tensors")
        self = cls.__new__(cls)
        self._A = (rows, cols, vals)  # the handle reads the triplets at build time
        self.m, self.k = int(m), int(k)
        self._h = C.c_void_p()
        p = make_params(rows_per_group, **params)
        check(lib().gcoo_create_coo(C.byref(self._h), self.m, self.k, C.c_void_p(rows.data_ptr()),
                                    C.c_void_p(cols.data_ptr()), C.c_void_p(vals.data_ptr()), int(vals.numel()),
                                    C.byref(p)))
        self.rows_per_group = rows_per_group
        return self

    @classmethod
    def from_matrix_market(cls, path: str, rows_per_group: int = 4, **params) -> "GcooHandle":
        """Handle for the matrix of a Matrix Market file (the reference
        driver's -file= input), through COO triplets on the current CUDA
        device; see read_matrix_market for the file semantics."""
        torch = _torch()
        rows, cols, vals, m, k = read_matrix_market(path)
        dev = torch.device("cuda")
        return cls.from_coo(torch.from_numpy(rows).to(dev), torch.from_numpy(cols).to(dev),
                            torch.from_numpy(vals).to(dev), m, k, rows_per_group, **params)

    @property
    def ptr(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gcoo_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, stream=None) -> "GcooHandle":
        check(lib().gcoo_build(self._h, _stream_ptr(stream)))
        return self

    def export(self) -> dict:
        v = View()
        check(lib().gcoo_export(self._h, C.byref(v)))
        ng = int(v.n_group)
        return {"m": v.m, "k": v.k, "nnz": int(v.nnz), "n_group": ng, "rows_per_group": v.rows_per_group,
                "groupIndex": _view_tensor(v.group_index, ng + 1, "<i4", self),
                "nnzPerGroup": _view_tensor(v.nnz_per_group, ng + 1, "<i4", self),
                "vals": _view_tensor(v.vals, v.nnz, "<f4", self),
                "rows": _view_tensor(v.rows, v.nnz, "<i4", self),
                "cols": _view_tensor(v.cols, v.nnz, "<i4", self)}

    @property
    def nnz(self) -> int:
        v = View()
        check(lib().gcoo_export(self._h, C.byref(v)))
        return int(v.nnz)

    def _out(self, B, Cout):
        torch = _torch()
        _check_f32(B, "B")
        if B.dim() != 2 or B.shape[0] != self.k:
            raise ValueError(f"B must be {self.k} x n")
        n = int(B.shape[1])
        if Cout is None:
            Cout = torch.empty((self.m, n), dtype=torch.float32, device=B.device)
        _check_f32(Cout, "C", (self.m, n))
        return n, Cout

    def spdm(self, B, Cout=None, prec: str = "fp32", stream=None):
        n, Cout = self._out(B, Cout)
        s = _stream_ptr(stream)
        if prec == "fp32":
            check(lib().gcoo_spdm(self._h, C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()), s))
        else:
            check(lib().gcoo_spdm_ex(self._h, C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()),
                                     PREC[prec], s))
        return Cout

    def spdm_left(self, D, Cout=None, stream=None):
        """C = D @ A (the other orientation): D is p x m, C is p x k."""
        torch = _torch()
        _check_f32(D, "D")
        if D.dim() != 2 or D.shape[1] != self.m:
            raise ValueError(f"D must be p x {self.m}")
        p = int(D.shape[0])
        if Cout is None:
            Cout = torch.empty((p, self.k), dtype=torch.float32, device=D.device)
        _check_f32(Cout, "C", (p, self.k))
        check(lib().gcoo_spdm_left(self._h, C.c_void_p(D.data_ptr()), p, C.c_void_p(Cout.data_ptr()),
                                   _stream_ptr(stream)))
        return Cout

    def prepare(self, n: int, prec: str, stream=None):
        check(lib().gcoo_prepare(self._h, int(n), PREC[prec], _stream_ptr(stream)))

    def multiply_by(self, B, Cout=None, stream=None):
        n, Cout = self._out(B, Cout)
        check(lib().gcoo_multiply_by(self._h, C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()),
                                     _stream_ptr(stream)))
        return Cout

    def error_norm(self, B, Cout, stream=None) -> float:
        n = int(B.shape[1])
        out = C.c_double()
        check(lib().gcoo_error_norm(self._h, C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()),
                                    C.byref(out), _stream_ptr(stream)))
        return float(out.value)

    def query_engine(self, prec: str) -> bool:
        t = C.c_int32()
        check(lib().gcoo_query_engine(self._h, PREC[prec], C.byref(t)))
        return bool(t.value)

    def check_arrays(self, stream=None) -> int:
        """Structural validation of the built arrays on the GPU (gcoo_check_arrays):
        0 when every invariant holds, else the number of offending groups."""
        bad = C.c_int64()
        st = lib().gcoo_check_arrays(self._h, _stream_ptr(stream), C.byref(bad))
        if st not in (0, 6):
            check(st)
        return int(bad.value)

    def device_status(self, stream=None) -> int:
        s = C.c_uint32()
        st = lib().gcoo_device_status(self._h, _stream_ptr(stream), C.byref(s))
        if st not in (0, 7):
            check(st)
        return int(s.value)

    def autotune(self, B, Cout=None, stream=None) -> dict:
        n, Cout = self._out(B, Cout)
        p = Params()
        check(lib().gcoo_autotune(self._h, C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()),
                                  _stream_ptr(stream), C.byref(p)))
        return {"vec": p.vec, "warps": p.warps, "col_warps": p.col_warps}


def read_matrix_market(path: str):
    """A Matrix Market coordinate file as (rows, cols, vals, m, k): int32,
    int32 and float32 NumPy arrays of 0-based triplets in file order, each
    mirror (symmetric, skew-symmetric) right after its entry; pattern
    entries are 1.0. Host code only (gcoo_read_matrix_market)."""
    import numpy as np
    m, k, n = C.c_int64(), C.c_int64(), C.c_int64()
    r, c = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    v = C.POINTER(C.c_float)()
    L = lib()
    check(L.gcoo_read_matrix_market(os.fsencode(path), C.byref(m), C.byref(k), C.byref(n), C.byref(r),
                                    C.byref(c), C.byref(v)))
    try:
        cnt = int(n.value)
        rows = np.ctypeslib.as_array(r, shape=(max(cnt, 1),))[:cnt].copy()
        cols = np.ctypeslib.as_array(c, shape=(max(cnt, 1),))[:cnt].copy()
        vals = np.ctypeslib.as_array(v, shape=(max(cnt, 1),))[:cnt].copy()
    finally:
        for ptr in (r, c, v):
            L.gcoo_free_host(C.cast(ptr, C.c_void_p))
    return rows, cols, vals, int(m.value), int(k.value)


def convert_count(A, rows_per_group=4, stream=None):
    """Count + scan on caller arrays; returns (groupIndex, nnzPerGroup, nnz)."""
    torch = _torch()
    _check_f32(A, "A")
    m, k = A.shape
    ng = (m + rows_per_group - 1) // rows_per_group
    gi = torch.empty(ng + 1, dtype=torch.int32, device=A.device)
    npg = torch.empty(ng + 1, dtype=torch.int32, device=A.device)
    nnz = C.c_int64()
    check(lib().gcoo_convert_count(C.c_void_p(A.data_ptr()), m, k, rows_per_group, C.c_void_p(gi.data_ptr()),
                                   C.c_void_p(npg.data_ptr()), C.byref(nnz), _stream_ptr(stream)))
    return gi, npg, int(nnz.value)


def convert_scatter(A, group_index, nnz, rows_per_group=4, stream=None):
    torch = _torch()
    m, k = A.shape
    vals = torch.empty(max(nnz, 1), dtype=torch.float32, device=A.device)
    rows = torch.empty(max(nnz, 1), dtype=torch.int32, device=A.device)
    cols = torch.empty(max(nnz, 1), dtype=torch.int32, device=A.device)
    check(lib().gcoo_convert_scatter(C.c_void_p(A.data_ptr()), m, k, rows_per_group,
                                     C.c_void_p(group_index.data_ptr()), C.c_void_p(vals.data_ptr()),
                                     C.c_void_p(rows.data_ptr()), C.c_void_p(cols.data_ptr()), _stream_ptr(stream)))
    return vals[:nnz], rows[:nnz], cols[:nnz]


def spdm_view(m, k, rows_per_group, group_index, nnz_per_group, vals, rows, cols, B, Cout=None, stream=None):
    """Multiply from caller-owned arrays in the reference's GCOO layout."""
    torch = _torch()
    n = int(B.shape[1])
    if Cout is None:
        Cout = torch.empty((m, n), dtype=torch.float32, device=B.device)
    v = View()
    v.m, v.k, v.nnz = m, k, int(vals.numel())
    v.n_group = (m + rows_per_group - 1) // rows_per_group
    v.rows_per_group = rows_per_group
    v.group_index, v.nnz_per_group = group_index.data_ptr(), nnz_per_group.data_ptr()
    v.vals, v.rows, v.cols = vals.data_ptr(), rows.data_ptr(), cols.data_ptr()
    check(lib().gcoo_spdm_view(C.byref(v), C.c_void_p(B.data_ptr()), n, C.c_void_p(Cout.data_ptr()),
                               _stream_ptr(stream)))
    return Cout


class GcooBatch:
    """Many independent multiplies in one persistent launch (gcoo_batch_*)."""

    def __init__(self, problems, prec: str = "fp32", stream=None):
        arr = (Problem * len(problems))()
        self._keep = []
        for i, (h, B, Cout) in enumerate(problems):
            arr[i].a = h.ptr.value
            arr[i].dB = B.data_ptr()
            arr[i].n = int(B.shape[1])
            arr[i].dC = Cout.data_ptr()
            self._keep.append((h, B, Cout))
        self._b = C.c_void_p()
        check(lib().gcoo_batch_create(C.byref(self._b), arr, len(problems), PREC[prec], _stream_ptr(stream)))

    def run(self, stream=None):
        check(lib().gcoo_batch_run(self._b, _stream_ptr(stream)))

    @property
    def launches(self) -> int:
        n = C.c_int32()
        check(lib().gcoo_batch_launches(self._b, C.byref(n)))
        return int(n.value)

    def close(self):
        if getattr(self, "_b", None) and self._b.value:
            lib().gcoo_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GcooSession:
    """mutiplyBy from HOST buffers (gcoo_session_*): A moves in row panels, each
    panel converted and multiplied as soon as it and B are on the device, C
    panels copied back while later panels are in flight. Same bits as
    GcooHandle.multiply_by. Host tensors should be pinned for full link speed."""

    def __init__(self, rows_per_group: int = 4, panel_rows: int = 0, **params):
        p = make_params(rows_per_group=rows_per_group, **params)
        self._s = C.c_void_p()
        check(lib().gcoo_session_create(C.byref(self._s), C.byref(p), int(panel_rows)))

    def multiply(self, A, B, Cout=None, stream=None):
        """C = A x B with A, B, C CPU tensors (float32, row-major contiguous)."""
        torch = _torch()
        for t, name in ((A, "A"), (B, "B")):
            if t.device.type != "cpu" or t.dtype != torch.float32 or not t.is_contiguous() or t.dim() != 2:
                raise ValueError(f"{name} must be a contiguous 2-D float32 host tensor")
        m, k = int(A.shape[0]), int(A.shape[1])
        if int(B.shape[0]) != k:
            raise ValueError("B must have k rows")
        n = int(B.shape[1])
        if Cout is None:
            Cout = torch.empty((m, n), dtype=torch.float32, pin_memory=A.is_pinned())
        if Cout.device.type != "cpu" or tuple(Cout.shape) != (m, n) or not Cout.is_contiguous() \
                or Cout.dtype != torch.float32:
            raise ValueError("C must be a contiguous m x n float32 host tensor")
        check(lib().gcoo_session_multiply(self._s, C.c_void_p(A.data_ptr()), m, k, C.c_void_p(B.data_ptr()), n,
                                          C.c_void_p(Cout.data_ptr()), _stream_ptr(stream)))
        return Cout

    def stats(self) -> dict:
        launches, panels = C.c_int32(), C.c_int32()
        check(lib().gcoo_session_stats(self._s, C.byref(launches), C.byref(panels)))
        return {"launches": int(launches.value), "panels": int(panels.value)}

    def close(self):
        if getattr(self, "_s", None) and self._s.value:
            lib().gcoo_session_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_save(path: str):
    check(lib().gcoo_autotune_save(path.encode()))


def autotune_load(path: str):
    check(lib().gcoo_autotune_load(path.encode()))


def autotune_clear():
    check(lib().gcoo_autotune_clear())


# ---- the reference's plugin surface ------------------------------------------------

class ShGemm:
    """src/ShGemm.h:7-24: constructed from the sparse operand (dense buffer)."""

    def __init__(self, nRows: int = 0, nCols: int = 0):
        self.m_nRows, self.m_nCols = nRows, nCols
        self.m_pDenseMatrix = None

    def mutiplyBy(self, A, nRows, nCols, C_):  # noqa: N802 - the reference's name
        raise NotImplementedError

    def mutiply(self, B, nRows, nCols, C_):  # noqa: N802
        raise NotImplementedError

    def build(self):
        raise NotImplementedError

    def runKernelTest(self, A, nRows, nCols, C_):  # noqa: N802
        raise NotImplementedError


class ShGCOOSpDM(ShGemm):
    """src/ShGCOOSpDM.h: denseMatrix is m x k (nRows x nCols), the dense operand
    A given to mutiplyBy / runKernelTest is k x n (its nRows x nCols), C is
    m x n. Returns 0.0 like the reference; failures raise GcooError (the
    reference exited the process)."""

    def __init__(self, denseMatrix, nRows: int, nCols: int, **params):
        super().__init__(nRows, nCols)
        if tuple(denseMatrix.shape) != (nRows, nCols):
            raise ValueError("denseMatrix shape does not match nRows x nCols")
        self.m_pDenseMatrix = denseMatrix
        self._h = GcooHandle(denseMatrix, **params)
        self.m_nGroup = (nRows + self._h.rows_per_group - 1) // self._h.rows_per_group
        self._arrays = None

    def _sync(self):
        _torch().cuda.current_stream().synchronize()

    def mutiplyBy(self, A, nRows, nCols, C_):  # noqa: N802
        if tuple(A.shape) != (nRows, nCols):
            raise ValueError("A shape does not match nRows x nCols")
        self._h.multiply_by(A, C_)
        self._sync()
        return 0.0

    def mutiply(self, B, nRows, nCols, C_):  # noqa: N802
        """C = B x self (B nRows x nCols with nCols == self's rows); empty in the
        reference's GCOO plugin (src/ShGCOOSpDM.h:21)."""
        if tuple(B.shape) != (nRows, nCols) or nCols != self.m_nRows:
            raise ValueError("B must be nRows x (rows of the sparse operand)")
        if self._arrays is None:
            self.build()
            self._arrays = True
        self._h.spdm_left(B, C_)
        self._sync()
        return 0.0

    def build(self):
        self._h.build()
        self._sync()
        a = self._h.export()
        self.m_pGroupIndex, self.m_pNnzPerGroup = a["groupIndex"], a["nnzPerGroup"]
        self.m_pVals, self.m_pRows, self.m_pCols = a["vals"], a["rows"], a["cols"]
        self.m_nGroup = a["n_group"]

    def runKernelTest(self, A, nRows, nCols, C_, prec: str = "fp32"):  # noqa: N802
        if tuple(A.shape) != (nRows, nCols):
            raise ValueError("A shape does not match nRows x nCols")
        self._h.spdm(A, C_, prec=prec)
        self._sync()
        return 0.0

    @property
    def handle(self) -> GcooHandle:
        return self._h


class _BaselineGemm(ShGemm):
    """cuBLAS / cuSPARSE / CSR plugins of libgcoo_baselines.so (same C = self x A)."""

    _L = None

    @classmethod
    def _lib(cls):
        if cls._L is None:
            lib()  # libgcoo.so first (dependency)
            L = C.CDLL(BASELINES_PATH)
            L.gcoo_baseline_create.restype = C.c_void_p
            L.gcoo_baseline_create.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_int]
            for f in ("gcoo_baseline_multiply_by", "gcoo_baseline_run_kernel"):
                getattr(L, f).restype = C.c_double
                getattr(L, f).argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
            L.gcoo_baseline_build.argtypes = [C.c_void_p]
            L.gcoo_baseline_destroy.argtypes = [C.c_void_p]
            L.gcoo_refalgo_create.restype = C.c_void_p
            L.gcoo_refalgo_create.argtypes = [C.c_void_p, C.c_int64, C.c_int64]
            for f in ("gcoo_refalgo_multiply_by", "gcoo_refalgo_run_kernel"):
                getattr(L, f).restype = C.c_int
                getattr(L, f).argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
            L.gcoo_refalgo_build.restype = C.c_int
            L.gcoo_refalgo_build.argtypes = [C.c_void_p]
            L.gcoo_refalgo_destroy.argtypes = [C.c_void_p]
            L.gcoo_measure_l2_read_gbs.restype = C.c_double
            L.gcoo_measure_l2_read_gbs.argtypes = [C.c_int]
            cls._L = L
        return cls._L

    def __init__(self, algo, denseMatrix, nRows, nCols):
        super().__init__(nRows, nCols)
        self.m_pDenseMatrix = denseMatrix
        self._g = self._lib().gcoo_baseline_create(algo.encode(), denseMatrix.data_ptr(), nRows, nCols)

    def mutiplyBy(self, A, nRows, nCols, C_):  # noqa: N802
        return self._lib().gcoo_baseline_multiply_by(self._g, A.data_ptr(), nRows, nCols, C_.data_ptr())

    def mutiply(self, B, nRows, nCols, C_):  # noqa: N802
        return -5.0

    def build(self):
        self._lib().gcoo_baseline_build(self._g)

    def runKernelTest(self, A, nRows, nCols, C_):  # noqa: N802
        return self._lib().gcoo_baseline_run_kernel(self._g, A.data_ptr(), nRows, nCols, C_.data_ptr())

    def __del__(self):
        try:
            if self._g:
                self._lib().gcoo_baseline_destroy(self._g)
        except Exception:
            pass


def measure_l2_read_gbs(reps: int = 3) -> float:
    """The L2 -> SM read peak of the current GPU in GB/s: 512-byte warp-wide
    loads at random offsets of an L2-resident 32 MB region (the shape of the
    multiply's B-row loads), best of `reps` launches. 0.0 on a CUDA error."""
    return float(_BaselineGemm._lib().gcoo_measure_l2_read_gbs(int(reps)))


class RefAlgoBaseline:
    """Baseline only: the reference's GCOO algorithm restated for the GPU
    (libgcoo_baselines.so): per-call allocation, single-thread serial scan,
    one CTA per 4-row group, scalar B loads. Timed beside this library."""

    def __init__(self, A):
        _check_f32(A, "A")
        self._A = A
        self.m, self.k = int(A.shape[0]), int(A.shape[1])
        self._L = _BaselineGemm._lib()
        self._h = self._L.gcoo_refalgo_create(A.data_ptr(), self.m, self.k)

    def multiply_by(self, B, Cout):
        if self._L.gcoo_refalgo_multiply_by(self._h, B.data_ptr(), int(B.shape[1]), Cout.data_ptr()) != 0:
            raise GcooError(3, "reference-algorithm baseline failed")
        return Cout

    def build(self):
        if self._L.gcoo_refalgo_build(self._h) != 0:
            raise GcooError(3, "reference-algorithm baseline build failed")

    def run_kernel(self, B, Cout):
        if self._L.gcoo_refalgo_run_kernel(self._h, B.data_ptr(), int(B.shape[1]), Cout.data_ptr()) != 0:
            raise GcooError(3, "reference-algorithm baseline multiply failed")
        return Cout

    def close(self):
        if getattr(self, "_h", None):
            self._L.gcoo_refalgo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SpGemmBuilder:
    """src/SpGemmBuilder.h:10-24: "gcoospdm" | "cublas" | "cusparse" | "csr", else None."""

    @staticmethod
    def getShGemmAlgo(denseMatrix, nRows, nCols, desc):  # noqa: N802
        if desc == "gcoospdm":
            return ShGCOOSpDM(denseMatrix, nRows, nCols)
        if desc in ("cublas", "cusparse", "csr"):
            return _BaselineGemm(desc, denseMatrix, nRows, nCols)
        return None
