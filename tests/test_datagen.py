"""CPU: the seeded input generator every test, fixture and benchmark draws
from. The hash is SplitMix64 (known answers below); the torch form, which
generates full-size inputs on the device, gives the NumPy form's bytes; and
each workload has the shape, sparsity and value distribution it claims."""
from __future__ import annotations

import numpy as np
import pytest

from gcoospdm_gb300 import datagen as dg

GOLD = 0x9E3779B97F4A7C15
M64 = (1 << 64) - 1


def test_splitmix64_known_answers():
    """SplitMix64 from state 0 (Steele, Lea and Flood; Vigna's published
    generator): the state steps by the golden-ratio constant and each output
    is the finaliser of the new state."""
    want = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    states = np.array([(i * GOLD) & M64 for i in range(3)], dtype=np.uint64)
    assert [int(v) for v in dg.splitmix64_np(states)] == want


def test_torch_form_gives_the_numpy_bytes():
    torch = pytest.importorskip("torch")
    for seed, m, k, p in ((5, 37, 29, 0.35), (6, 64, 130, 0.01), (7, 3, 1, 1.0), (8, 16, 16, 0.0)):
        a = dg.bernoulli_dense(seed, m, k, p)
        t = dg.bernoulli_dense_torch(seed, m, k, p, device="cpu", chunk=97).numpy()
        assert np.array_equal(a.view(np.uint32), t.view(np.uint32)), (seed, m, k, p)
    b = dg.dense_pm1(9, 5, 33, 130)
    assert np.array_equal(b.view(np.uint32), dg.dense_pm1_torch(9, 5, 33, 130, device="cpu", chunk=1000).numpy().view(np.uint32))
    c = dg.block_dense(10, 70, 45, 0.3)
    assert np.array_equal(c.view(np.uint32), dg.block_dense_torch(10, 70, 45, 0.3, device="cpu").numpy().view(np.uint32))
    h = dg.hash_np(11, 3, 1000, 64)
    ht = dg.hash_torch(11, 3, 1000, 64, "cpu").numpy().view(np.uint64)
    assert np.array_equal(h, ht)


def test_values_are_odd_multiples_of_2_pow_minus_24():
    v = dg.dense_pm1(12, 5, 256, 256).astype(np.float64)
    q = v * (1 << 24)
    assert np.all(np.abs(v) < 1.0) and np.all(v != 0.0)
    assert np.array_equal(q, np.round(q)) and np.all(np.round(q).astype(np.int64) % 2 != 0)
    assert abs(v.mean()) < 0.01 and abs(v.var() - 1.0 / 3.0) < 0.01   # U(-1, 1)


def test_bernoulli_density_and_chunking():
    p = 0.01
    a = dg.bernoulli_dense(13, 1024, 1024, p)
    nnz = int(np.count_nonzero(a))
    sd = (1024 * 1024 * p * (1 - p)) ** 0.5
    assert abs(nnz - 1024 * 1024 * p) < 6 * sd
    # the row chunking of the generator does not change a byte
    b = dg.bernoulli_dense(13, 1024, 1024, p, chunk_rows=7)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.count_nonzero(dg.bernoulli_dense(13, 50, 50, 0.0)) == 0
    assert np.count_nonzero(dg.bernoulli_dense(13, 50, 50, 1.0)) == 2500


def test_block_mask_is_whole_blocks():
    a = dg.block_dense(14, 100, 90, 0.4) != 0
    for bi in range(0, 100, 16):
        for bj in range(0, 90, 16):
            blk = a[bi:bi + 16, bj:bj + 16]
            assert blk.all() or not blk.any()


def test_zipf_rows_distinct_columns_and_total():
    m, k, target, cap = 4096, 4096, 60000, 512
    rows, cols, vals = dg.zipf_coo(15, m, k, target, alpha=2.0, cap=cap)
    assert rows.size == target and cols.size == target and vals.dtype == np.float32
    assert np.all(np.diff(rows) >= 0) and rows.min() >= 0 and rows.max() < m
    assert cols.min() >= 0 and cols.max() < k
    key = rows * k + cols
    assert np.all(np.diff(key) > 0)                  # sorted, distinct per row
    counts = np.bincount(rows, minlength=m)
    assert counts.max() <= cap and counts.max() > 8 * counts.mean()   # heavy-tailed
    assert np.all(vals != 0) and abs(float(vals.mean())) < 0.05 and abs(float(vals.std()) - 1.0) < 0.05


def test_batched_shapes_ranges():
    s = dg.batched_shapes(777, 512)
    assert len(s) == 512
    m, k, n, sp = (np.array([x[i] for x in s]) for i in range(4))
    assert m.min() >= 256 and m.max() <= 4096 and k.min() >= 256 and k.max() <= 4096
    assert set(n.tolist()) == {32, 64, 128}
    assert sp.min() >= 0.9 and sp.max() < 0.999
    assert dg.batched_shapes(777, 512) == s          # deterministic


def test_bernoulli_nnz_counts_the_mask():
    """The mask count the bench's reference arm reports without building A."""
    for seed, m, k, p in ((3, 37, 129, 0.05), (8192, 300, 8192, 0.01), (9, 1, 5000, 0.5)):
        A = dg.bernoulli_dense(seed, m, k, p)
        assert dg.bernoulli_nnz(seed, m, k, p) == int(np.count_nonzero(A))
