"""GPU: the tensor-core engine at the precision-form size -- A 8192 x 8192
with a 16 x 16 block mask (blocks active with probability 1 - s, dense
inside), B 8192 x 1024 -- where every CTA's ring wraps around hundreds of
K-tiles, two CTAs share an SM and the grid takes several waves. Sampled rows
(64 spread over all 64 row panels) are checked against FP64 products computed
on the GPU:
  * BF16: within 1e-5 of the exact product of the BF16-rounded operands and
    within 1e-2 of the exact product;
  * split-BF16 (three BF16 terms per operand, six products): within 5e-6
    of the exact product (the FP32-level bar is 1e-5);
  * FP8-B: within 1e-5 of the exact product of A rounded to BF16 and B
    quantized to E4M3 in units of its per-column power-of-two scale.
"""
from __future__ import annotations

import numpy as np
import pytest

from fp8_emu import e4m3_round, fp8_scales

pytestmark = pytest.mark.gpu

M = K = 8192
N = 1024
ROWS = list(range(5, M, 128))  # one row per 128-row panel, at varying offsets within it


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def bf16_round_t(torch, x):
    return x.to(torch.bfloat16).to(torch.float64)


def rel_fro_t(torch, got, ref):
    return float(torch.linalg.norm(got.double() - ref) / torch.linalg.norm(ref))


@pytest.fixture(scope="module")
def operands(torch):
    from gcoospdm_gb300 import datagen as dg
    B = dg.dense_pm1_torch(9100, 5, K, N, device="cuda")
    return B


@pytest.mark.parametrize("s", [0.5, 0.75])
def test_tensor_engine_at_precision_form_size(native, torch, operands, s):
    from gcoospdm_gb300 import datagen as dg
    B = operands
    A = dg.block_dense_torch(9100 + int(s * 1000), M, K, 1.0 - s, device="cuda")
    h = native.GcooHandle(A, engine="tensor").build()
    idx = torch.tensor(ROWS, device="cuda")
    Ar = A[idx].double()
    exact = Ar @ B.double()
    C = torch.empty(M, N, device="cuda")
    errs = {}
    # BF16
    h.spdm(B, C, prec="bf16")
    assert h.query_engine("bf16")
    rounded = bf16_round_t(torch, A[idx]) @ bf16_round_t(torch, B)
    errs["bf16_vs_rounded"] = rel_fro_t(torch, C[idx], rounded)
    errs["bf16_vs_exact"] = rel_fro_t(torch, C[idx], exact)
    # split-BF16
    h.spdm(B, C, prec="split_bf16")
    errs["split_vs_exact"] = rel_fro_t(torch, C[idx], exact)
    # FP8-B: B quantized to E4M3 in units of its column's power-of-two scale
    h.spdm(B, C, prec="fp8_b")
    Bh = B.cpu().numpy()
    sc = fp8_scales(Bh)
    Bq = torch.from_numpy(e4m3_round(Bh / sc) * sc).cuda().double()
    errs["fp8_vs_quantized"] = rel_fro_t(torch, C[idx], bf16_round_t(torch, A[idx]) @ Bq)
    print(f"s={s}: " + ", ".join(f"{k} {v:.3e}" for k, v in errs.items()))
    assert h.device_status() == 0
    assert errs["bf16_vs_rounded"] <= 1e-5
    assert errs["bf16_vs_exact"] <= 1e-2
    assert errs["split_vs_exact"] <= 5e-6
    assert errs["fp8_vs_quantized"] <= 1e-5


def test_tensor_engine_ragged_panels_and_columns(native, torch):
    """m = 8000 (the last 256-row panel partly filled) and n = 528 (two full
    256-column accumulators and a 16-column one): two accumulators per CTA
    (32 panels x 3 column tiles exceed one wave of one-accumulator pairs),
    the second cluster column with one accumulator, masked to n. BF16 and
    FP8-B on sampled rows, the last panel's rows included, against FP64 of
    the rounded / quantized operands."""
    from gcoospdm_gb300 import datagen as dg
    m, k, n = 8000, 8192, 528
    A = dg.block_dense_torch(9300, m, k, 0.25, device="cuda")
    B = dg.dense_pm1_torch(9301, 5, k, n, device="cuda")
    rows = list(range(3, m, 125)) + [m - 1]
    idx = torch.tensor(rows, device="cuda")
    h = native.GcooHandle(A, engine="tensor").build()
    C = torch.empty(m, n, device="cuda")
    h.spdm(B, C, prec="bf16")
    assert h.query_engine("bf16")
    err = rel_fro_t(torch, C[idx], bf16_round_t(torch, A[idx]) @ bf16_round_t(torch, B))
    h.spdm(B, C, prec="fp8_b")
    Bh = B.cpu().numpy()
    sc = fp8_scales(Bh)
    Bq = torch.from_numpy(e4m3_round(Bh / sc) * sc).cuda().double()
    err8 = rel_fro_t(torch, C[idx], bf16_round_t(torch, A[idx]) @ Bq)
    print(f"ragged: bf16 {err:.3e}, fp8_b {err8:.3e}")
    assert h.device_status() == 0
    assert err <= 1e-5 and err8 <= 1e-5
