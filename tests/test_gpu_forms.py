"""GPU: the reduced-precision forms (BF16, split-BF16, FP8-B), each checked
against the oracle: bit-identical for BF16 and FP8-B on the FMA engine (the
same fmaf chain on BF16-rounded, or E4M3-quantized and column-scaled,
inputs), within stated relative Frobenius bounds of FP64 for split-BF16
(1e-5) and FP8-B (5e-2), and FP8-B on the tensor engine within FP32 error of
the product of its quantized operands."""
from __future__ import annotations

import numpy as np
import pytest

from fp8_emu import e4m3_round, fp8_scales

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def bf16_round(x):
    """Round-to-nearest-even FP32 -> BF16, returned as FP32 (finite inputs)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def rel_fro(Cm, C64):
    C64 = np.asarray(C64, np.float64)
    return float(np.linalg.norm(np.asarray(Cm, np.float64) - C64) / np.linalg.norm(C64))


@pytest.fixture(scope="module")
def problem(oracle_mod):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(31, 600, 520, 0.02)
    B = dg.dense_pm1(31, 5, 520, 512)
    g = oracle_mod.convert(A)
    return A, B, g, oracle_mod.spdm_f64(g, B)


def test_bf16_fma_engine_bit_identical_to_rounded_chain(native, oracle_mod, torch, problem):
    A, B, g, C64 = problem
    h = native.GcooHandle(dev(torch, A), engine="cuda_core").build()
    Cg = h.spdm(dev(torch, B), prec="bf16").cpu().numpy()
    gr = oracle_mod.Gcoo(g.m, g.k, g.cpg, g.groupIndex, g.nnzPerGroup, bf16_round(g.vals), g.rows, g.cols)
    ref = oracle_mod.spdm(gr, bf16_round(B))
    assert np.array_equal(Cg.view(np.uint32), ref.view(np.uint32))
    assert rel_fro(Cg, C64) <= 1e-2
    assert not h.query_engine("bf16")


@pytest.mark.parametrize("n", [512, 1000, 2048])
def test_group_walk_of_reduced_forms_identical_to_row_walk(native, oracle_mod, torch, n):
    """BF16 and FP8-B on the FMA engine over a block-clustered A: the GCOO-order
    walk (chosen automatically there) and the row walk give the same bits, and
    BF16 equals the oracle's rounded chain."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(33, 1003, 768, 0.3)
    B = dg.dense_pm1(33, 5, 768, n)
    dA, dB = dev(torch, A), dev(torch, B)
    g = oracle_mod.convert(A)
    C64 = oracle_mod.spdm_f64(g, B)
    for prec in ("bf16", "fp8_b"):
        if prec == "fp8_b" and n % 16:
            continue  # the FP8-B form wants n % 16 == 0
        got = {}
        for order in ("auto", "groups", "rows"):
            h = native.GcooHandle(dA, engine="cuda_core", fp32_order=order).build()
            got[order] = h.spdm(dB, prec=prec).cpu().numpy()
        assert np.array_equal(got["auto"].view(np.uint32), got["rows"].view(np.uint32)), prec
        assert np.array_equal(got["groups"].view(np.uint32), got["rows"].view(np.uint32)), prec
        assert rel_fro(got["groups"], C64) <= (1e-2 if prec == "bf16" else 5e-2)
        if prec == "bf16":
            gr = oracle_mod.Gcoo(g.m, g.k, g.cpg, g.groupIndex, g.nnzPerGroup, bf16_round(g.vals), g.rows, g.cols)
            ref = oracle_mod.spdm(gr, bf16_round(B))
            assert np.array_equal(got["groups"].view(np.uint32), ref.view(np.uint32))


def test_split_bf16_fma_engine_fp32_level(native, torch, problem):
    A, B, g, C64 = problem
    h = native.GcooHandle(dev(torch, A), engine="cuda_core").build()
    Cg = h.spdm(dev(torch, B), prec="split_bf16").cpu().numpy()
    assert rel_fro(Cg, C64) <= 1e-5


def test_fp8_b_fma_engine(native, torch, problem):
    A, B, g, C64 = problem
    h = native.GcooHandle(dev(torch, A)).build()
    Cg = h.spdm(dev(torch, B), prec="fp8_b").cpu().numpy()
    err = rel_fro(Cg, C64)
    assert err <= 5e-2
    assert err > 1e-4  # it really is the 3-bit-mantissa form


def test_fp8_b_fma_engine_bit_identical_to_quantized_chain(native, oracle_mod, torch, problem):
    """FP8-B on the FMA engine is the FP32 chain over B quantized to E4M3 in
    units of a power-of-two column scale, times that scale: bit for bit the
    oracle's chain over the quantized B, scaled afterwards (exact)."""
    A, B, g, C64 = problem
    B = B.copy()
    B[:, :64] *= 1e-3  # columns of very different magnitude
    B[:, 64:128] *= 1e3
    s = fp8_scales(B)
    Bq = e4m3_round(B / s)
    ref = (oracle_mod.spdm(g, Bq) * s).astype(np.float32)
    h = native.GcooHandle(dev(torch, A), engine="cuda_core").build()
    Cg = h.spdm(dev(torch, B), prec="fp8_b").cpu().numpy()
    assert np.array_equal(Cg.view(np.uint32), ref.view(np.uint32))


def test_fp8_b_tensor_engine_matches_quantized_product(native, torch):
    """FP8-B on the tensor engine: the same quantized B (exact in BF16), A in
    BF16, FP32 accumulation in the tensor pipe -- within FP32 summation error
    of the FP64 product of the quantized operands."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(65, 384, 320, 0.3)
    B = dg.dense_pm1(65, 5, 320, 256)
    B[:, :32] *= 1e-3
    s = fp8_scales(B)
    ref = bf16_round(A).astype(np.float64) @ (e4m3_round(B / s).astype(np.float64) * s)
    h = native.GcooHandle(dev(torch, A)).build()
    assert h.query_engine("fp8_b")
    Cg = h.spdm(dev(torch, B), prec="fp8_b").cpu().numpy()
    assert rel_fro(Cg, ref) <= 1e-5


def test_fp8_per_column_scales(native, torch, oracle_mod):
    """Columns of very different magnitude keep their relative accuracy."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(32, 200, 256, 0.05)
    B = dg.dense_pm1(32, 5, 256, 64)
    B[:, :16] *= 1e-3
    B[:, 16:32] *= 1e3
    g = oracle_mod.convert(A)
    C64 = oracle_mod.spdm_f64(g, B)
    h = native.GcooHandle(dev(torch, A)).build()
    Cg = h.spdm(dev(torch, B), prec="fp8_b").cpu().numpy()
    for lo, hi in ((0, 16), (16, 32), (32, 64)):
        assert rel_fro(Cg[:, lo:hi], C64[:, lo:hi]) <= 5e-2


def test_form_rejects_unsupported_width(native, torch, problem):
    A, B, g, C64 = problem
    h = native.GcooHandle(dev(torch, A)).build()
    Bo = dev(torch, B[:, :13].copy())
    with pytest.raises(native.GcooError) as e:
        h.spdm(Bo, prec="fp8_b")
    assert e.value.status == 5


def test_prepare_then_graph_capture(native, torch, problem):
    """After gcoo_prepare, a reduced-precision multiply replays from a CUDA graph."""
    A, B, g, C64 = problem
    h = native.GcooHandle(dev(torch, A)).build()
    dB = dev(torch, B)
    Cd = torch.empty(A.shape[0], B.shape[1], device="cuda")
    h.prepare(B.shape[1], "bf16")
    ref = h.spdm(dB, prec="bf16").clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        h.spdm(dB, Cd, prec="bf16", stream=s)
    Cd.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(Cd, ref)
