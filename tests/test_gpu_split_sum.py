"""GPU: the FP32 multiply with gcoo_params.fp32_sum = split (GCOO_SUM_SPLIT).

In a skewed matrix the rows of at least 256 entries are summed as 32-entry
pieces whose partial sums are added in piece order. Checked against the
oracle on a Zipf(2) matrix whose rows reach 4096 entries:
  * relative Frobenius error against the oracle's FP64 product <= 1e-5 (the
    bar the FP32 mode is held to; the sequential chain reaches ~5e-7);
  * every row of fewer than 256 entries bit-identical to the sequential
    chain (the oracle's FP32 multiply, the reference's order);
  * the same bits on every run, after a rebuild, and from a CUDA graph;
  * n % 4 != 0 (no 16-byte B pieces) keeps every row on the chain.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def same_bits(x, y):
    x, y = np.asarray(x, np.float32), np.asarray(y, np.float32)
    nx, ny = np.isnan(x), np.isnan(y)
    return bool(np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint32), y[~ny].view(np.uint32)))


@pytest.fixture(scope="module")
def zipf_case():
    from gcoospdm_gb300 import datagen as dg
    m, k = 4096, 8192
    rows, cols, vals = dg.zipf_coo(7100, m, k, 100_000, alpha=2.0, cap=4096)
    A = np.zeros((m, k), np.float32)
    A[rows, cols] = vals
    counts = np.count_nonzero(A, axis=1)
    assert counts.max() == 4096 and (counts >= 256).sum() >= 5  # the long rows this test is about
    return A, counts


@pytest.mark.parametrize("n", [256, 200, 520, 1040])  # 1040: B of 34 MB, the short rows walk tile-major
def test_split_sum_within_tolerance_and_short_rows_exact(native, oracle_mod, torch, zipf_case, n):
    from gcoospdm_gb300 import datagen as dg
    A, counts = zipf_case
    m, k = A.shape
    B = dg.dense_pm1(7101, 1, k, n)
    g = oracle_mod.convert(A)
    chain = oracle_mod.spdm(g, B)
    c64 = oracle_mod.spdm_f64(g, B)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    h = native.GcooHandle(dA, fp32_sum="split").build()
    C1 = h.spdm(dB).cpu().numpy()
    err = oracle_mod.rel_fro(C1, c64)
    assert err <= TOL, err
    short = counts < 256
    assert same_bits(C1[short], chain[short])
    long_rows = np.nonzero(~short)[0]
    assert not same_bits(C1[long_rows], chain[long_rows])  # the long rows really were regrouped
    # deterministic: again, after a rebuild, and on the chain handle the chain's bits
    assert same_bits(h.spdm(dB).cpu().numpy(), C1)
    h.build()
    assert same_bits(h.spdm(dB).cpu().numpy(), C1)
    hc = native.GcooHandle(dA).build()
    assert same_bits(hc.spdm(dB).cpu().numpy(), chain)
    assert h.device_status() == 0


def test_split_sum_from_coo_and_graph_replay(native, oracle_mod, torch, zipf_case):
    """COO input, the partial-sum buffer made by gcoo_prepare, then the
    multiply (side stream fork and join included) captured and replayed."""
    from gcoospdm_gb300 import datagen as dg
    A, counts = zipf_case
    m, k = A.shape
    n = 256
    B = dg.dense_pm1(7102, 1, k, n)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    ref = native.GcooHandle(dA, fp32_sum="split").build().spdm(dB)
    r, c = torch.nonzero(dA, as_tuple=True)
    h = native.GcooHandle.from_coo(r.int().contiguous(), c.int().contiguous(), dA[r, c].contiguous(), m, k,
                                   fp32_sum="split").build()
    h.prepare(n, "fp32")
    Cd = torch.empty(m, n, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        h.spdm(dB, Cd, stream=s)
    Cd.fill_(float("nan"))
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(Cd, ref)


def test_split_sum_without_16_byte_pieces_keeps_the_chain(native, oracle_mod, torch, zipf_case):
    from gcoospdm_gb300 import datagen as dg
    A, _ = zipf_case
    m, k = A.shape
    B = dg.dense_pm1(7103, 1, k, 98)  # n % 4 != 0: every row on the row kernel
    chain = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(torch.from_numpy(A).cuda(), fp32_sum="split").build()
    assert same_bits(h.spdm(torch.from_numpy(B).cuda()).cpu().numpy(), chain)


def test_split_sum_leaves_uniform_matrices_on_the_chain(native, oracle_mod, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(7104, 600, 900, 0.05)  # not skewed: no long-row list
    B = dg.dense_pm1(7104, 5, 900, 128)
    h = native.GcooHandle(torch.from_numpy(A).cuda(), fp32_sum="split").build()
    assert same_bits(h.spdm(torch.from_numpy(B).cuda()).cpu().numpy(), oracle_mod.spdm(oracle_mod.convert(A), B))
