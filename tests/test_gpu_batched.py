"""GPU: the persistent batched engine (one graph-replayed launch over a
device work queue) and the autotuner. Each problem's FP32 result is
bit-identical to its own gcoo_spdm; BF16 to gcoo_spdm_ex(BF16) on the FMA
engine."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def problems(native, torch):
    from gcoospdm_gb300 import datagen as dg
    shapes = dg.batched_shapes(777, 48)
    out = []
    for i, (m, k, n, s) in enumerate(shapes):
        m, k = m // 4, k // 4  # same distribution, quarter size (test speed)
        A = dg.bernoulli_dense_torch(1000 + i, m, k, 1.0 - s, device="cuda")
        B = dg.dense_pm1_torch(1000 + i, 5, k, n, device="cuda")
        h = native.GcooHandle(A).build()
        out.append((h, A, B))
    return out


def test_batched_fp32_bit_identical(native, torch, problems):
    native.autotune_clear()
    Cs = [torch.full((h.m, B.shape[1]), float("nan"), device="cuda") for h, A, B in problems]
    batch = native.GcooBatch([(h, B, Cb) for (h, A, B), Cb in zip(problems, Cs)], prec="fp32")
    assert batch.launches == 1
    for C in Cs:
        C.fill_(float("nan"))
    batch.run()
    batch.run()  # graph replay is repeatable
    torch.cuda.synchronize()
    for (h, A, B), C in zip(problems, Cs):
        ref = h.spdm(B)
        assert torch.equal(C, ref)


def test_batched_bf16_matches_fma_form(native, torch, problems):
    Cs = [torch.empty((h.m, B.shape[1]), device="cuda") for h, A, B in problems]
    batch = native.GcooBatch([(h, B, Cb) for (h, A, B), Cb in zip(problems, Cs)], prec="bf16")
    assert batch.launches == 2
    batch.run()
    torch.cuda.synchronize()
    for (h, A, B), C in zip(problems, Cs):
        h2 = native.GcooHandle(A, engine="cuda_core").build()
        n = B.shape[1]
        if n % 8:
            continue
        ref = h2.spdm(B, prec="bf16")
        assert torch.equal(C, ref)


def test_autotune_table_round_trip(native, torch, problems, tmp_path):
    h, A, B = problems[0]
    best = h.autotune(B)
    assert best["vec"] in (1, 2, 4) and best["warps"] >= 1
    C1 = h.spdm(B)
    path = str(tmp_path / "tune.json")
    native.autotune_save(path)
    text = open(path).read()
    assert '"bucket": "m' in text and "batch_n" in text
    native.autotune_clear()
    native.autotune_load(path)
    C2 = h.spdm(B)
    assert torch.equal(C1, C2)


def test_batch_rejects_unbuilt(native, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(5, 64, 64, 0.1, device="cuda")
    h = native.GcooHandle(A)
    B = torch.zeros(64, 32, device="cuda")
    C = torch.zeros(64, 32, device="cuda")
    with pytest.raises(native.GcooError) as e:
        native.GcooBatch([(h, B, C)])
    assert e.value.status == 4


def test_irregular_zipf_rows(native, oracle_mod, torch):
    """Zipf(2) row counts capped at 4096 (heavy rows spill over many chunks)."""
    from gcoospdm_gb300 import datagen as dg
    m = k = 8192
    rows, cols, vals = dg.zipf_coo(91, m, k, 150_000, alpha=2.0, cap=4096)
    assert np.bincount(rows, minlength=m).max() <= 4096
    A = torch.zeros(m, k, device="cuda")
    A[torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda()] = torch.from_numpy(vals).cuda()
    B = dg.dense_pm1_torch(91, 5, k, 256, device="cuda")
    h = native.GcooHandle(A).build()
    assert h.nnz == 150_000
    C = h.spdm(B)
    assert h.error_norm(B, C) <= 1e-5
    # bit-for-bit against the oracle on the heaviest rows and a sample
    counts = np.bincount(rows, minlength=m)
    pick = np.unique(np.concatenate([np.argsort(counts)[-8:], np.arange(0, m, 997)]))
    sub = A[torch.from_numpy(pick).cuda()].cpu().numpy()
    ref = oracle_mod.spdm(oracle_mod.convert(sub, 1), B.cpu().numpy())
    got = C[torch.from_numpy(pick).cuda()].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
