"""GPU: the tcgen05 tensor-core engine on block-clustered matrices (16 x 16
blocks), BF16 and split-BF16, against FP64: BF16 within 1e-2 of the exact
product and within FP32-accumulation error (1e-5) of the exact product of the
BF16-rounded inputs; split-BF16 within 1e-5 of the exact product."""
from __future__ import annotations

import numpy as np
import pytest

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
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def rel_fro(Cm, C64):
    C64 = np.asarray(C64, np.float64)
    return float(np.linalg.norm(np.asarray(Cm, np.float64) - C64) / np.linalg.norm(C64))


def exact(A, B):
    return np.asarray(A, np.float64) @ np.asarray(B, np.float64)


@pytest.mark.parametrize("m,k,n,p", [(128, 16, 128, 1.0), (256, 128, 128, 0.5), (300, 200, 256, 0.3),
                                     (512, 384, 384, 0.25), (1024, 1024, 512, 0.1)])
def test_tc_bf16_block_matrix(native, torch, m, k, n, p):
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(40 + m, m, k, p)
    B = dg.dense_pm1(40 + m, 5, k, n)
    h = native.GcooHandle(dev(torch, A), engine="tensor").build()
    Cg = h.spdm(dev(torch, B), prec="bf16").cpu().numpy()
    assert h.device_status() == 0
    assert rel_fro(Cg, exact(bf16_round(A), bf16_round(B))) <= 1e-5
    assert rel_fro(Cg, exact(A, B)) <= 1e-2


@pytest.mark.parametrize("m,k,n,p", [(256, 128, 128, 0.5), (640, 512, 256, 0.2)])
def test_tc_split_bf16_block_matrix(native, torch, m, k, n, p):
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(50 + m, m, k, p)
    B = dg.dense_pm1(50 + m, 5, k, n)
    h = native.GcooHandle(dev(torch, A), engine="tensor").build()
    Cg = h.spdm(dev(torch, B), prec="split_bf16").cpu().numpy()
    assert h.device_status() == 0
    assert rel_fro(Cg, exact(A, B)) <= 1e-5


def test_tc_empty_panels_are_zero(native, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(61, 512, 256, 0.4)
    A[128:384] = 0.0
    B = dg.dense_pm1(61, 5, 256, 128)
    h = native.GcooHandle(dev(torch, A), engine="tensor").build()
    Cg = h.spdm(dev(torch, B), prec="bf16").cpu().numpy()
    assert np.all(Cg[128:384] == 0.0)
    assert rel_fro(Cg, exact(A, B)) <= 1e-2


def test_auto_engine_choice(native, torch):
    from gcoospdm_gb300 import datagen as dg
    blk = native.GcooHandle(dev(torch, dg.block_dense(62, 512, 512, 0.1))).build()
    assert blk.query_engine("bf16")
    rnd = native.GcooHandle(dev(torch, dg.bernoulli_dense(62, 512, 512, 0.01))).build()
    assert not rnd.query_engine("bf16")
    assert not blk.query_engine("fp32") and blk.query_engine("fp8_b")
    assert not rnd.query_engine("fp8_b")


def test_tc_fp8_b(native, torch):
    """FP8-B on the tensor engine: B quantized to E4M3 with power-of-two
    column scales (the FMA engine's quantization), multiplied as exact BF16
    values; columns of very different magnitude keep their accuracy, and the
    two engines agree up to the BF16 rounding of A (the FMA engine keeps A in
    FP32)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(64, 384, 320, 0.3)
    B = dg.dense_pm1(64, 5, 320, 256)
    B[:, :32] *= 1e-3
    B[:, 32:64] *= 1e3
    dA, dB = dev(torch, A), dev(torch, B)
    ht = native.GcooHandle(dA).build()
    assert ht.query_engine("fp8_b")
    t = ht.spdm(dB, prec="fp8_b").cpu().numpy()
    f = native.GcooHandle(dA, engine="cuda_core").build().spdm(dB, prec="fp8_b").cpu().numpy()
    ref = exact(A, B)
    for lo, hi in ((0, 32), (32, 64), (64, 256)):
        err = rel_fro(t[:, lo:hi], ref[:, lo:hi])
        assert 1e-4 < err <= 5e-2
        assert rel_fro(t[:, lo:hi], f[:, lo:hi].astype(np.float64)) <= 1e-2


def test_tc_matches_fma_engine_bf16(native, torch):
    """Both engines compute the same BF16 product (up to FP32 summation order)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(63, 384, 320, 0.3)
    B = dg.dense_pm1(63, 5, 320, 256)
    t = native.GcooHandle(dev(torch, A), engine="tensor").build().spdm(dev(torch, B), prec="bf16").cpu().numpy()
    f = native.GcooHandle(dev(torch, A), engine="cuda_core").build().spdm(dev(torch, B), prec="bf16").cpu().numpy()
    assert rel_fro(t, f.astype(np.float64)) <= 1e-5
