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


def test_batched_odd_widths_every_item_shape(native, torch):
    """Widths that are not multiples of 4 or 8 (and unaligned C) take the
    narrower item shapes -- 2 or 1 values per lane, 16 or 32 lanes per row --
    in both forms: FP32 bit-identical to gcoo_spdm, BF16 to the FMA form."""
    from gcoospdm_gb300 import datagen as dg
    out = []
    for i, (m, k, n) in enumerate([(77, 64, 1), (130, 96, 3), (64, 200, 6), (300, 128, 20), (91, 64, 40),
                                   (257, 100, 100), (40, 64, 130)]):
        A = dg.bernoulli_dense_torch(2000 + i, m, k, 0.1, device="cuda")
        B = dg.dense_pm1_torch(2000 + i, 5, k, n, device="cuda")
        out.append((native.GcooHandle(A).build(), A, B))
    Cs = [torch.full((h.m, B.shape[1]), float("nan"), device="cuda") for h, A, B in out]
    batch = native.GcooBatch([(h, B, C) for (h, A, B), C in zip(out, Cs)], prec="fp32")
    batch.run()
    torch.cuda.synchronize()
    for (h, A, B), C in zip(out, Cs):
        assert torch.equal(C, h.spdm(B))
    # BF16 needs k * n % 4 == 0 (true for every k above)
    Cb = [torch.full((h.m, B.shape[1]), float("nan"), device="cuda") for h, A, B in out]
    batch = native.GcooBatch([(h, B, C) for (h, A, B), C in zip(out, Cb)], prec="bf16")
    batch.run()
    torch.cuda.synchronize()
    for (h, A, B), C in zip(out, Cb):
        ref = native.GcooHandle(A, engine="cuda_core").build()
        n = B.shape[1]
        if n % 8 == 0:  # the single-problem BF16 FMA form's width rule
            assert torch.equal(C, ref.spdm(B, prec="bf16"))
        Bq = B.to(torch.bfloat16).double()
        Aq = A.to(torch.bfloat16).double()
        exact = Aq @ Bq
        assert float(torch.linalg.norm(C.double() - exact) / torch.linalg.norm(exact)) <= 1e-5


def test_l2_read_peak_probe(native, torch):
    """The roofline denominator bench.py measures live: an L2-resident gather
    (512-byte warp loads) between 5 and 60 TB/s on a GB300."""
    gbs = native.measure_l2_read_gbs()
    assert 5000.0 < gbs < 60000.0, gbs
