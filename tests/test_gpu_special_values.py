"""GPU: special values in both operands, through every FP32 entry point.

The reference's zero test keeps NaN, +-inf and subnormal entries of A and
drops -0.0 (src/gcoo_spdm_kernels.cu:4-90, `v != 0`). Its multiply starts
every output at 0.0f and adds the products with fmaf in GCOO order
(src/gcoo_spdm_kernels.cu:92-158). So an output whose products are all -0
comes out +0, NaN and inf propagate, inf - inf gives NaN, and the product
of two values near FLT_MAX overflows to inf.

Here B holds signed zeros, NaN, +-inf, subnormals and values near FLT_MAX
in chosen rows, and A reaches them from short rows and, in the skewed
case, from long rows (the long-row kernel beside the short-row one). Every
path gives the oracle's bits, with NaN compared as NaN."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M, K, N = 203, 700, 132          # N % 4 == 0: 16-byte B pieces, long-row kernel eligible
ZP, ZN, NAN_ROW, INF_ROW, SUB_ROW, BIG_ROW = 11, 12, 13, 14, 15, 16   # special rows of B


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def same_bits(x, y):
    """Bitwise equality, NaNs compared as NaN (payloads differ across ISAs)."""
    x, y = np.asarray(x, np.float32), np.asarray(y, np.float32)
    nx, ny = np.isnan(x), np.isnan(y)
    return bool(np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint32), y[~ny].view(np.uint32)))


def operands(skewed: bool):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(95, M, K, 0.02)
    B = dg.dense_pm1(96, 5, K, N)
    B[ZP] = 0.0
    B[ZN] = -0.0
    B[NAN_ROW, ::3] = np.nan
    B[INF_ROW, ::2] = np.inf
    B[INF_ROW, 1::4] = -np.inf
    B[SUB_ROW] *= np.float32(1e-38)                      # subnormal magnitudes
    B[BIG_ROW] = np.where(B[BIG_ROW] < 0, np.float32(-3e38), np.float32(3e38))
    special = [ZP, ZN, NAN_ROW, INF_ROW, SUB_ROW, BIG_ROW]
    A[:, special] = 0.0
    # rows whose only products are -0: the outputs are +0 (0.0f + -0)
    A[0] = 0.0
    A[0, ZP] = -0.75
    A[1] = 0.0
    A[1, ZN] = 0.5
    A[2] = 0.0
    A[2, ZP], A[2, ZN] = -1.0, 1.0
    # special entries of A
    A[3, 40] = np.nan
    A[4, 41], A[4, 42] = np.inf, -np.inf                # inf - inf wherever B's row entries agree in sign
    A[5, 43], A[5, 44] = np.float32(1e-40), np.float32(-1e-45)
    A[6] = 0.0
    A[6, 45] = -0.0                                      # dropped: an empty row, +0 outputs
    A[7, BIG_ROW] = np.float32(3e38)                     # overflow to +-inf
    A[8, BIG_ROW], A[8, INF_ROW] = np.float32(-3e38), 1.0
    # short rows reaching each special row of B
    A[20:40, NAN_ROW] = 0.5
    A[40:60, INF_ROW] = -0.25
    A[60:80] = 0.0
    A[60:80, SUB_ROW] = 2.0                              # subnormal outputs
    A[80:100, BIG_ROW] = 1.5
    A[100:110, ZN] = -2.0
    if skewed:
        rng = np.random.default_rng(97)
        for r, length in ((120, 400), (150, 690), (202, 300)):
            cols = np.union1d(rng.choice(K, size=length, replace=False), special)
            v = rng.uniform(-1.0, 1.0, size=cols.size).astype(np.float32)
            A[r] = 0.0
            A[r, cols] = np.where(v == 0.0, np.float32(0.5), v)
        A[150, 333] = np.nan
        A[202, 334] = np.float32(2e-44)
    return A, B


@pytest.mark.parametrize("skewed", [False, True])
def test_special_values_every_fp32_path(native, oracle_mod, torch, skewed):
    A, B = operands(skewed)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    assert np.all(ref[[0, 1, 2, 6]].view(np.uint32) == 0)   # +0.0, never -0.0
    assert np.isnan(ref).any() and np.isposinf(ref).any() and np.isneginf(ref).any()
    sub = np.abs(ref[60:80])
    assert np.any((sub > 0) & (sub < np.float32(1.1754944e-38)))  # subnormal outputs too
    dA, dB = dev(torch, A), dev(torch, B)
    out = {}

    h = native.GcooHandle(dA).build()
    out["build + spdm"] = h.spdm(dB)
    h.build()                                        # the staged rebuild
    out["staged rebuild + spdm"] = h.spdm(dB)
    Cd = torch.full((M, N), float("nan"), device="cuda")
    h.multiply_by(dB, Cd)
    out["multiply_by"] = Cd
    out["GCOO-order walk"] = native.GcooHandle(dA, fp32_order="groups").build().spdm(dB)
    r, c = torch.nonzero(dA, as_tuple=True)          # NaN is a nonzero, -0.0 is not
    out["COO input"] = native.GcooHandle.from_coo(r.int().contiguous(), c.int().contiguous(),
                                                  dA[r, c].contiguous(), M, K).build().spdm(dB)
    g = oracle_mod.convert(A)
    out["reference-layout view"] = native.spdm_view(g.m, g.k, 4, dev(torch, g.groupIndex),
                                                    dev(torch, g.nnzPerGroup), dev(torch, g.vals),
                                                    dev(torch, g.rows), dev(torch, g.cols), dB)
    Cb = torch.full((M, N), float("nan"), device="cuda")
    batch = native.GcooBatch([(h, dB, Cb)], prec="fp32")
    batch.run()
    torch.cuda.synchronize()
    out["batched launch"] = Cb
    session = native.GcooSession(panel_rows=64)
    out["host-buffer session"] = session.multiply(torch.from_numpy(A).pin_memory(), torch.from_numpy(B).pin_memory())

    for name, C in out.items():
        assert same_bits(C.cpu().numpy(), ref), name
    assert h.device_status() == 0 and h.check_arrays() == 0
    assert h.nnz == int(np.count_nonzero(A != 0))
    batch.close()
    session.close()


def test_special_values_left_orientation(native, oracle_mod, torch):
    """C = D x A with the special values in D's columns (they meet A's
    rows): the oracle's chain on the transposed problem, bit for bit."""
    from gcoospdm_gb300 import datagen as dg
    A, _ = operands(False)
    D = dg.dense_pm1(98, 5, 64, M)
    D[:, 20] = 0.0
    D[:, 21] = -0.0
    D[::3, 22] = np.nan
    D[::2, 40] = np.inf
    D[1::4, 41] = -np.inf
    D[:, 60] *= np.float32(1e-38)
    D[:, 80] = np.float32(3e38)
    ref_t = oracle_mod.spdm(oracle_mod.convert(np.ascontiguousarray(A.T)), np.ascontiguousarray(D.T))
    ref = np.ascontiguousarray(ref_t.T)
    assert np.isnan(ref).any() and np.isinf(ref).any()
    h = native.GcooHandle(dev(torch, A)).build()
    assert same_bits(h.spdm_left(dev(torch, D)).cpu().numpy(), ref)
    assert h.device_status() == 0
