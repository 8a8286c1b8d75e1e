"""GPU: gcoo_convert_count_static, the count + scan entry point that
allocates nothing (for callers that cannot allocate device memory when they
convert: memory owned by another runtime's pool, loops that must not pay
cudaMalloc's implicit synchronisation, bindings without an allocator).

Called through the C ABI twice in a row on different matrices, each result
compared with the allocating entry point gcoo_convert_count (integer
outputs: exact equality). Kept in a file of its own that pytest collects
last."""
from __future__ import annotations

import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 20


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _static_count(native, torch, A, rows_per_group):
    m, k = A.shape
    ng = (m + rows_per_group - 1) // rows_per_group
    # sentinels: every entry must be overwritten
    gi = torch.full((ng + 1,), -7, dtype=torch.int32, device="cuda")
    npg = torch.full((ng + 1,), -7, dtype=torch.int32, device="cuda")
    nnz = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream or None
    st = native.lib().gcoo_convert_count_static(C.c_void_p(A.data_ptr()), m, k, rows_per_group,
                                                C.c_void_p(gi.data_ptr()), C.c_void_p(npg.data_ptr()),
                                                C.byref(nnz), stream)
    native.check(st)
    return gi, npg, int(nnz.value)


def test_static_count_matches_allocating_entry_point_twice(native, torch):
    from gcoospdm_gb300 import datagen as dg
    cases = [(1000, 777, 0.05, 4, 301), (70001, 129, 0.02, 8, 302)]  # second call: more rows, other group height
    for m, k, p, rpg, seed in cases:
        A = dg.bernoulli_dense_torch(seed, m, k, p, device="cuda")
        gi_ref, npg_ref, nnz_ref = native.convert_count(A, rpg)
        gi, npg, nnz = _static_count(native, torch, A, rpg)
        torch.cuda.synchronize()
        assert nnz == nnz_ref
        assert torch.equal(gi, gi_ref)
        assert torch.equal(npg, npg_ref)
        assert int(gi[-1]) == nnz and int(npg[-1]) == 0


def test_static_count_at_the_row_limit_with_allocation_refused(native, torch):
    """m = 2^20 exactly (the largest accepted: 256 scan blocks, the total in
    the array's last slot), run while the library's allocator hook refuses
    every request: the static entry point still succeeds and never asks."""
    from gcoospdm_gb300 import _native as nat
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(303, MAX_ROWS, 4, 0.3, device="cuda")
    gi_ref, npg_ref, nnz_ref = native.convert_count(A, 4)
    calls = {"n": 0}

    def alloc(nbytes, ctx):
        calls["n"] += 1
        return None

    def release(ptr, ctx):
        calls["n"] += 1

    L = native.lib()
    a_cb, f_cb = nat.ALLOC_FN(alloc), nat.FREE_FN(release)
    assert L.gcoo_set_allocator(a_cb, f_cb, None) == 0
    try:
        for _ in range(2):
            gi, npg, nnz = _static_count(native, torch, A, 4)
            torch.cuda.synchronize()
            assert nnz == nnz_ref
            assert torch.equal(gi, gi_ref)
            assert torch.equal(npg, npg_ref)
    finally:
        assert L.gcoo_set_allocator(nat.ALLOC_FN(0), nat.FREE_FN(0), None) == 0
    assert calls["n"] == 0


def test_static_count_rejects_rows_beyond_limit(native, torch):
    A = torch.zeros(4, 4, device="cuda")
    gi = torch.zeros(8, dtype=torch.int32, device="cuda")
    nnz = C.c_int64(-1)
    st = native.lib().gcoo_convert_count_static(C.c_void_p(A.data_ptr()), MAX_ROWS + 1, 4, 4,
                                                C.c_void_p(gi.data_ptr()), C.c_void_p(gi.data_ptr()),
                                                C.byref(nnz), None)
    assert st == 1  # GCOO_ERROR_INVALID_VALUE, nothing launched
    assert b"static scratch limit" in native.lib().gcoo_last_error()
    assert nnz.value == -1
