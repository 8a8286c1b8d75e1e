"""GPU: the host-buffer session (gcoo_session_*): A, B and C in host memory,
copy-in / convert / multiply / copy-out overlapped by row panels. Every case
must give the same bits as the device-resident plugin path (build + FP32
multiply), which the other tests pin to the reference."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def device_result(native, torch, A, B, rows_per_group=4):
    h = native.GcooHandle(A.cuda(), rows_per_group=rows_per_group).build()
    return h.spdm(B.cuda()).cpu()


def same_bits(torch, x, y):
    return x.shape == y.shape and bool(torch.equal(x.view(torch.int32), y.view(torch.int32)))


def test_session_matches_fixture_readme(native, torch, manifest):
    entry = manifest["cases"]["readme_800"]
    A, B = golden_inputs(entry, "readme_800")
    s = native.GcooSession(panel_rows=96)
    C = s.multiply(torch.from_numpy(A).pin_memory(), torch.from_numpy(B).pin_memory())
    assert hashlib.sha256(C.numpy().tobytes()).hexdigest() == entry["digests"]["C"]
    st = s.stats()
    assert st["panels"] == 9  # 800 rows in 96-row panels
    assert st["launches"] >= 4 * st["panels"]
    s.close()


@pytest.mark.parametrize("m,k,n,p,panel_rows,cpg", [
    (1001, 517, 333, 0.05, 0, 4),    # odd n: 1-wide columns; ragged last panel
    (3, 5, 7, 0.6, 0, 4),            # fewer rows than a group
    (4097, 256, 128, 0.02, 1000, 4),  # explicit panel height, ragged tail
    (640, 130, 96, 0.1, 64, 8),      # k % 4 != 0: scalar scatter; 8-row groups
    (512, 512, 64, 0.0, 0, 4),       # no nonzeros at all
    (300, 2048, 1024, 0.3, 32, 2),   # many small panels
])
def test_session_bit_identical(native, torch, m, k, n, p, panel_rows, cpg):
    from gcoospdm_gb300 import datagen as dg
    A = torch.from_numpy(dg.bernoulli_dense(m + k, m, k, p)).pin_memory()
    B = torch.from_numpy(dg.dense_pm1(n, 5, k, n)).pin_memory()
    s = native.GcooSession(rows_per_group=cpg, panel_rows=panel_rows)
    C = s.multiply(A, B)
    assert same_bits(torch, C, device_result(native, torch, A, B, cpg))
    s.close()


def test_session_edge_values_and_pageable_memory(native, torch, manifest):
    entry = manifest["cases"]["edge_values"]
    A, B = golden_inputs(entry, "edge_values")
    At, Bt = torch.from_numpy(np.ascontiguousarray(A)), torch.from_numpy(np.ascontiguousarray(B))  # pageable
    s = native.GcooSession()
    C = s.multiply(At, Bt)
    assert same_bits(torch, C, device_result(native, torch, At, Bt))  # same ISA: NaN payloads included
    s.close()


def test_session_reuse_grows_and_orders_on_stream(native, torch):
    """One session, calls of different sizes (buffers grow, never stale), the
    work ordered after a user stream."""
    from gcoospdm_gb300 import datagen as dg
    s = native.GcooSession()
    stream = torch.cuda.Stream()
    for i, (m, k, n) in enumerate([(256, 256, 128), (2048, 1024, 512), (512, 300, 200), (2048, 1024, 512)]):
        A = torch.from_numpy(dg.bernoulli_dense(40 + i, m, k, 0.03)).pin_memory()
        B = torch.from_numpy(dg.dense_pm1(40 + i, 5, k, n)).pin_memory()
        C = s.multiply(A, B, stream=stream)
        assert same_bits(torch, C, device_result(native, torch, A, B))
    s.close()


def test_session_rejects_bad_arguments(native, torch):
    s = native.GcooSession()
    with pytest.raises(ValueError):
        s.multiply(torch.zeros(4, 4, device="cuda"), torch.zeros(4, 4))
    L = native.lib()
    assert L.gcoo_session_multiply(s._s, None, 4, 4, None, 4, None, None) == 1
    assert L.gcoo_session_multiply(s._s, 1, 0, 4, 1, 4, 1, None) == 1
    s.close()
    import ctypes
    out = ctypes.c_void_p()
    assert L.gcoo_session_create(ctypes.byref(out), None, -1) == 1


def test_session_full_size_matches_multiply_by(native, torch):
    """The headline workload from host buffers, same bits as the device path."""
    from gcoospdm_gb300 import datagen as dg
    n = 8192
    A = dg.bernoulli_dense_torch(0x6C02, n, n, 0.01, device="cuda")
    B = dg.dense_pm1_torch(0x6C02, 5, n, n, device="cuda")
    Cd = torch.empty(n, n, device="cuda")
    native.GcooHandle(A).multiply_by(B, Cd)
    Ah, Bh = A.cpu().pin_memory(), B.cpu().pin_memory()
    s = native.GcooSession()
    Ch = s.multiply(Ah, Bh, Cout=torch.empty(n, n).pin_memory())
    assert torch.equal(Ch.view(torch.int32), Cd.cpu().view(torch.int32))
    assert s.stats()["panels"] == 11  # 6 full 1024-row panels, then 1024, 512, 256, 128, 128
    s.close()


def test_session_refuses_panels_beyond_int32(native, torch):
    """k = 2^26 + 1 columns in 32-row groups: a one-group panel could hold
    more than 2^31 - 1 entries, which a panel (scattered without a readback
    of its total) cannot take. Refused with GCOO_ERROR_UNSUPPORTED before any
    allocation or copy; the host buffers are allocated but never touched."""
    k = (1 << 26) + 1
    A = torch.empty((32, k), dtype=torch.float32)
    B = torch.empty((k, 1), dtype=torch.float32)
    s = native.GcooSession(rows_per_group=32)
    with pytest.raises(native.GcooError) as e:
        s.multiply(A, B)
    assert e.value.status == 5
    s.close()


def test_session_error_after_enqueue_drains_and_recovers(native, torch):
    """B wider than 65535 column tiles (n odd: 64-column tiles): the first
    panel's multiply is refused on the host after the copies of A and B were
    enqueued. The call drains its streams before it returns
    GCOO_ERROR_CUDA, and the session then multiplies normally."""
    from gcoospdm_gb300 import datagen as dg
    A = torch.from_numpy(dg.bernoulli_dense(41, 8, 4, 0.6))
    n = 65535 * 64 + 1
    s = native.GcooSession()
    with pytest.raises(native.GcooError) as e:
        s.multiply(A, torch.ones((4, n), dtype=torch.float32))
    assert e.value.status == 3
    B = torch.from_numpy(dg.dense_pm1(41, 5, 4, 33))
    C = s.multiply(A, B)
    assert same_bits(torch, C, device_result(native, torch, A, B))
    s.close()
