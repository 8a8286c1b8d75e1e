"""GPU: failure detection without faulting a GPU -- a bounded device wait that
is made to run out (nothing arrives on its barrier), allocation failures
injected through the allocator hook, and the driver's error and check paths."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_bounded_wait_gives_up_and_context_survives(native, torch):
    L = native.lib()
    st = L.gcoo_check_bounded_wait(2_000_000, None)  # 2 ms
    assert st == 7  # GCOO_ERROR_TIMEOUT, reported by the kernel itself
    assert b"gave up" in L.gcoo_last_error()
    # the context is still usable
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(3, 64, 64, 0.2, device="cuda")
    B = dg.dense_pm1_torch(3, 5, 64, 32, device="cuda")
    h = native.GcooHandle(A).build()
    C_ = h.spdm(B)
    ref = A.double() @ B.double()
    assert float((C_.double() - ref).abs().max()) < 1e-5
    assert h.device_status() == 0
    assert L.gcoo_check_bounded_wait(0, None) == 1


def test_allocation_failure_injected_through_hook(native, torch):
    from gcoospdm_gb300 import _native as nat
    from gcoospdm_gb300 import datagen as dg
    L = native.lib()
    state = {"calls": 0, "fail_after": 2, "live": {}}

    def alloc(nbytes, ctx):
        state["calls"] += 1
        if state["calls"] > state["fail_after"]:
            return None
        t = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device="cuda")
        state["live"][t.data_ptr()] = t
        return t.data_ptr()

    def release(ptr, ctx):
        state["live"].pop(ptr, None)

    a_cb, f_cb = nat.ALLOC_FN(alloc), nat.FREE_FN(release)
    A = dg.bernoulli_dense_torch(4, 300, 200, 0.05, device="cuda")
    assert L.gcoo_set_allocator(a_cb, f_cb, None) == 0
    try:
        h = native.GcooHandle(A)
        with pytest.raises(native.GcooError) as e:
            h.build()
        assert e.value.status == 2  # GCOO_ERROR_ALLOC, no exception escaped, nothing launched half-way
        state["fail_after"] = 10_000
        h.build()  # the same handle recovers once memory is available
        B = dg.dense_pm1_torch(4, 5, 200, 64, device="cuda")
        ref = native.GcooHandle(A)  # created under the hook too
        ref.build()
        assert torch.equal(h.spdm(B), ref.spdm(B))
        assert state["live"]  # the library's buffers really came from the hook
        h.close()
        ref.close()
        assert not state["live"]  # and went back through it
    finally:
        assert L.gcoo_set_allocator(nat.ALLOC_FN(0), nat.FREE_FN(0), None) == 0


def _main(native, *args):
    return subprocess.run([native.MAIN_PATH, *args], capture_output=True, text=True, timeout=300)


@pytest.mark.parametrize("algo", ["gcoospdm", "cusparse", "cublas", "csr"])
def test_driver_check_passes(native, algo):
    r = _main(native, "-sparsity=0.9", "-nRowsA=300", "-nColsA=260", "-nRowsB=200", "-nColsB=300",
              f"-algo={algo}", "-check=1", "-reps=3")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Test passed" in r.stdout and "Time:" in r.stdout


@pytest.mark.parametrize("prec", ["bf16", "split", "fp8"])
def test_driver_precision_forms(native, prec):
    r = _main(native, "-sparsity=0.95", "-nRowsA=512", "-nColsA=256", "-nRowsB=384", "-nColsB=512",
              "-algo=gcoospdm", "-kernelonly=1", f"-prec={prec}", "-check=1", "-reps=3")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Test passed" in r.stdout


def test_driver_rejects_unknown_algo_and_shape(native):
    r = _main(native, "-algo=ell", "-nRowsA=64", "-nColsA=64", "-nRowsB=64", "-nColsB=64")
    assert r.returncode == 2 and "unknown -algo" in r.stderr
    r = _main(native, "-algo=gcoospdm", "-nRowsA=64", "-nColsA=64", "-nRowsB=64", "-nColsB=63")
    assert r.returncode == 2


def test_reference_algorithm_baseline_bit_identical(native, torch):
    """The GPU restatement of the reference algorithm (a timing baseline) gives
    the same FP32 bits as the library, end to end and kernel only."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(90, 1001, 700, 0.05, device="cuda")
    B = dg.dense_pm1_torch(90, 5, 700, 300, device="cuda")
    ours = native.GcooHandle(A).build().spdm(B)
    ref = native.RefAlgoBaseline(A)
    C1 = torch.empty_like(ours)
    ref.multiply_by(B, C1)
    assert torch.equal(C1, ours)
    ref.build()
    C2 = torch.zeros_like(ours)
    ref.run_kernel(B, C2)
    assert torch.equal(C2, ours)
    ref.close()


def test_check_arrays_accepts_built_handles_and_reports_corruption(native, torch):
    """gcoo_check_arrays: silent on a built handle (both conversion paths and
    COO ingestion), and reports each kind of damage written into the arrays
    (no multiply ever runs on damaged arrays; the check reads in bounds)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(61, 1001, 700, 0.05, device="cuda")
    h = native.GcooHandle(A).build()
    assert h.check_arrays() == 0
    h.build()  # the one-pass rebuild
    assert h.check_arrays() == 0
    r, c = torch.nonzero(A, as_tuple=True)
    hc = native.GcooHandle.from_coo(r.int().contiguous(), c.int().contiguous(), A[r, c].contiguous(), 1001, 700).build()
    assert hc.check_arrays() == 0
    a = h.export()

    def damaged(name, idx, value):
        t = a[name]
        old = t[idx].clone()
        t[idx] = value
        torch.cuda.synchronize()
        bad = h.check_arrays()
        t[idx] = old
        torch.cuda.synchronize()
        return bad

    assert damaged("cols", 3, 705) >= 1             # column out of range
    assert damaged("vals", 10, -0.0) >= 1           # an explicit zero entry
    assert damaged("rows", 7, 1000) >= 1            # row outside its group
    assert damaged("groupIndex", 5, 2 ** 30) >= 1   # offset far out of range, never dereferenced
    assert damaged("cols", 0, int(a["cols"][1]) + 1) >= 1  # (column, row) order broken
    assert h.check_arrays() == 0                    # everything restored
