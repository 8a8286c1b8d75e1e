"""GPU: dense -> GCOO conversion through the C ABI, bit-identical to the
reference (golden fixtures) and to the oracle on larger seeded inputs."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu
FIELDS = ("groupIndex", "nnzPerGroup", "vals", "rows", "cols")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


GOLDEN = ["tiny", "edge_values", "empty_groups", "all_zero", "k1", "m3", "n_tail", "cpg1", "cpg2", "cpg8",
          "cpg16", "readme_800", "sweep_2048_s099", "ragged_1001x517"]


@pytest.mark.parametrize("name", GOLDEN)
def test_handle_conversion_matches_reference(native, torch, manifest, name):
    entry = manifest["cases"][name]
    A, _ = golden_inputs(entry, name)
    h = native.GcooHandle(dev(torch, A), rows_per_group=entry["cpg"]).build()
    a = h.export()
    assert a["nnz"] == entry["nnz"]
    assert a["n_group"] == entry["n_group"]
    for f in FIELDS:
        assert digest(host(a[f])) == entry["digests"][f], f
    assert h.device_status() == 0


@pytest.mark.parametrize("name", ["tiny", "edge_values", "cpg8", "readme_800", "ragged_1001x517"])
def test_caller_array_conversion_matches_reference(native, torch, manifest, name):
    entry = manifest["cases"][name]
    A, _ = golden_inputs(entry, name)
    dA = dev(torch, A)
    gi, npg, nnz = native.convert_count(dA, entry["cpg"])
    assert nnz == entry["nnz"]
    vals, rows, cols = native.convert_scatter(dA, gi, nnz, entry["cpg"])
    torch.cuda.synchronize()
    got = {"groupIndex": gi, "nnzPerGroup": npg, "vals": vals, "rows": rows, "cols": cols}
    for f in FIELDS:
        assert digest(host(got[f])) == entry["digests"][f], f


@pytest.mark.parametrize("n,s,cpg", [(2048, 0.95, 4), (4096, 0.99, 4), (4096, 0.999, 4), (3000, 0.98, 32),
                                     (2048, 0.99, 1), (2048, 0.99, 16)])
def test_conversion_matches_oracle_sweep_shapes(native, oracle_mod, torch, n, s, cpg):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(100 + n, n, n, 1.0 - s)
    g = oracle_mod.convert(A, cpg)
    h = native.GcooHandle(dev(torch, A), rows_per_group=cpg).build()
    a = h.export()
    assert a["nnz"] == g.nnz
    for f in FIELDS:
        np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)


def test_unaligned_rows_and_base(native, oracle_mod, torch):
    """k not a multiple of 4 and a base pointer off the 16-byte grid."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(77, 333, 1027, 0.07)
    buf = torch.zeros(A.size + 3, dtype=torch.float32, device="cuda")
    buf[1:1 + A.size] = dev(torch, A.ravel())
    dA = buf[1:1 + A.size].view(333, 1027)
    assert dA.data_ptr() % 16 != 0
    h = native.GcooHandle(dA).build()
    a = h.export()
    g = oracle_mod.convert(A, 4)
    for f in FIELDS:
        np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)


def test_heavy_rows_and_empty_rows(native, oracle_mod, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(5, 64, 9000, 0.001)
    A[3, :] = dg.dense_pm1(5, 9, 1, 9000)[0]      # a fully dense row (9000 entries)
    A[10:20, :] = 0.0                               # empty groups
    g = oracle_mod.convert(A, 4)
    h = native.GcooHandle(dev(torch, A)).build()
    a = h.export()
    for f in FIELDS:
        np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)


def test_rebuild_after_change(native, oracle_mod, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(41, 200, 150, 0.05)
    dA = dev(torch, A)
    h = native.GcooHandle(dA).build()
    n1 = h.nnz
    A2 = dg.bernoulli_dense(42, 200, 150, 0.2)
    dA.copy_(dev(torch, A2))
    h.build()
    g = oracle_mod.convert(A2)
    assert h.nnz == g.nnz and h.nnz != n1
    np.testing.assert_array_equal(host(h.export()["cols"]), g.cols)


@pytest.mark.parametrize("name", GOLDEN)
def test_one_pass_rebuild_matches_reference(native, oracle_mod, torch, manifest, name):
    """A second build of the same handle reads A once (each tile's entries
    staged in a slot, then placed after the scans): the same arrays as the
    fixtures, and the same FP32 product."""
    entry = manifest["cases"][name]
    A, B = golden_inputs(entry, name)
    h = native.GcooHandle(dev(torch, A), rows_per_group=entry["cpg"]).build()
    C1 = h.spdm(dev(torch, B)).cpu().numpy() if B is not None else None
    h.build()  # arrays from the first build have room: one pass
    a = h.export()
    assert a["nnz"] == entry["nnz"]
    for f in FIELDS:
        assert digest(host(a[f])) == entry["digests"][f], f
    if B is not None:
        C2 = h.spdm(dev(torch, B)).cpu().numpy()
        assert np.array_equal(np.isnan(C1), np.isnan(C2))
        assert np.array_equal(C1[~np.isnan(C1)].view(np.uint32), C2[~np.isnan(C2)].view(np.uint32))
    assert h.device_status() == 0


@pytest.mark.parametrize("m,k,p,cpg", [(1001, 516, 0.05, 4), (4099, 2048, 0.01, 4), (777, 1000, 0.3, 8),
                                       (513, 4096, 0.002, 2), (300, 64, 0.5, 1), (5, 8, 1.0, 4)])
def test_one_pass_rebuild_matches_oracle(native, oracle_mod, torch, m, k, p, cpg):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(200 + m, m, k, p)
    B = dg.dense_pm1(200 + m, 5, k, 96)
    g = oracle_mod.convert(A, cpg)
    h = native.GcooHandle(dev(torch, A), rows_per_group=cpg).build()
    h.build()
    a = h.export()
    assert a["nnz"] == g.nnz
    for f in FIELDS:
        np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)
    ref = oracle_mod.spdm(oracle_mod.convert(A, 4), B)
    assert np.array_equal(h.spdm(dev(torch, B)).cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_one_pass_capacity_fallback_and_shrink(native, oracle_mod, torch):
    """Rebuild after A got denser than the arrays allow (the staged attempt
    falls back to the two-pass path) and after it got sparser (one pass)."""
    from gcoospdm_gb300 import datagen as dg
    A1 = dg.bernoulli_dense(51, 2000, 1024, 0.01)
    A2 = dg.bernoulli_dense(52, 2000, 1024, 0.2)
    A3 = dg.bernoulli_dense(53, 2000, 1024, 0.005)
    dA = dev(torch, A1)
    h = native.GcooHandle(dA).build()
    for A in (A2, A3, A2, A1):
        dA.copy_(dev(torch, A))
        h.build()
        h.build()
        g = oracle_mod.convert(A)
        a = h.export()
        assert a["nnz"] == g.nnz
        for f in FIELDS:
            np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)
        assert h.device_status() == 0


def test_staged_rebuild_overflowed_tiles(native, oracle_mod, torch):
    """Rebuild where a few tiles (4 rows x 1024 columns) hold far more entries
    than their staging slot (sized from the last build): those tiles are
    rescanned from A, the others placed from their slots. Includes the last,
    partial group and the last, partial tile."""
    from gcoospdm_gb300 import datagen as dg
    m, k = 1030, 3000
    dA = dev(torch, dg.bernoulli_dense(61, m, k, 0.02))
    h = native.GcooHandle(dA).build()
    A2 = dg.bernoulli_dense(62, m, k, 0.004)
    rng = np.random.default_rng(63)
    for r0, r1, c0, c1 in ((0, 4, 0, 1024), (500, 504, 1024, 2048), (1028, 1030, 2048, 3000), (8, 12, 40, 1000)):
        blk = rng.uniform(-1.0, 1.0, size=(r1 - r0, c1 - c0)).astype(np.float32)
        A2[r0:r1, c0:c1] = np.where(blk == 0.0, np.float32(0.5), blk)
    dA.copy_(dev(torch, A2))
    for _ in range(2):
        h.build()
        g = oracle_mod.convert(A2)
        a = h.export()
        assert a["nnz"] == g.nnz
        for f in FIELDS:
            np.testing.assert_array_equal(host(a[f]), getattr(g, f), err_msg=f)
        assert h.device_status() == 0
        assert h.check_arrays() == 0
    B = dg.dense_pm1(64, 1, k, 40)
    ref = oracle_mod.spdm(g, B)
    assert np.array_equal(h.spdm(dev(torch, B)).cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_full_size_staged_rebuild_equals_two_pass(native, torch):
    """n=8192, s=0.99: the staged rebuild (A read once, tiles staged and
    placed) gives arrays bit-identical to the two-pass first build, also
    after A changed so that some tiles overflow their slots (rescanned) --
    compared with a fresh handle's two-pass build of the new A."""
    from gcoospdm_gb300 import datagen as dg
    dA = dg.bernoulli_dense_torch(8193, 8192, 8192, 0.01, device="cuda")
    h = native.GcooHandle(dA).build()
    first = {f: t.clone() for f, t in h.export().items() if f in FIELDS}
    h.build()
    again = h.export()
    for f in FIELDS:
        assert torch.equal(again[f], first[f]), f
    assert h.check_arrays() == 0
    # thin most rows out and fill a few tiles densely: same handle, staged path with rescans
    dA[: 4096] *= (dg.bernoulli_dense_torch(8194, 4096, 8192, 0.5, device="cuda") != 0).float()
    dA[100:104, 2048:3072] = dg.dense_pm1_torch(8195, 5, 4, 1024, device="cuda") + 2.0
    dA[8190:8192, 7168:8192] = dg.dense_pm1_torch(8196, 5, 2, 1024, device="cuda") + 2.0
    h.build()
    got = h.export()
    # a temporary handle: its exported views keep it (and its arrays) alive
    ref = native.GcooHandle(dA).build().export()
    assert got["nnz"] == ref["nnz"]
    for f in FIELDS:
        assert torch.equal(got[f], ref[f]), f
    assert h.check_arrays() == 0


def test_full_size_properties_8192(native, torch):
    """n=8192, s=0.99: counts equal the dense count, offsets are the exclusive
    prefix, every group is (column, row) sorted, values round-trip."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(8192, 8192, 8192, 0.01)
    dA = dev(torch, A)
    h = native.GcooHandle(dA).build()
    a = h.export()
    nnz = a["nnz"]
    assert nnz == int((dA != 0).sum().item())
    gi, npg = a["groupIndex"].long(), a["nnzPerGroup"].long()
    assert int(gi[0]) == 0 and int(gi[-1]) == nnz and int(npg[-1]) == 0
    assert torch.equal(gi[1:] - gi[:-1], npg[:-1])
    rows, cols = a["rows"].long(), a["cols"].long()
    grp = torch.repeat_interleave(torch.arange(a["n_group"], device="cuda"), npg[:-1])
    assert torch.equal(rows // 4, grp)
    key = grp * (1 << 40) + cols * 8192 + rows
    assert bool((key[1:] > key[:-1]).all())
    assert torch.equal(dA[rows, cols], a["vals"])


@pytest.mark.parametrize("n", [46344, 46341])
def test_nnz_beyond_int32_refused_and_handle_recovers(native, torch, n):
    """A dense n x n matrix of ones holds n*n > 2^31 - 1 nonzeros (8.6 GB),
    more than the format's int32 offsets can address. Every conversion entry
    refuses it with GCOO_ERROR_FORMAT (6) before writing an entry: the first
    two-pass build, the caller-array count, and a later one-read rebuild of
    a handle whose arrays exist (n = 46344; k odd takes the scalar count).
    The handle stays usable: a refused rebuild leaves it unbuilt, and once A
    is thinned out it builds and multiplies."""
    A = torch.ones(n, n, device="cuda")
    h = native.GcooHandle(A)
    with pytest.raises(native.GcooError) as e:
        h.build()
    assert e.value.status == 6
    ng = (n + 3) // 4
    with pytest.raises(native.GcooError) as e:
        native.convert_count(A)
    assert e.value.status == 6
    A[1:] = 0.0
    h.build()
    assert h.nnz == n and h.check_arrays() == 0 and h.device_status() == 0
    A.fill_(1.0)
    with pytest.raises(native.GcooError) as e:
        h.build()
    assert e.value.status == 6
    B = torch.ones(n, 8, device="cuda")
    with pytest.raises(native.GcooError) as e:
        h.spdm(B)
    assert e.value.status == 4  # not built: the refused build left no stale arrays in use
    A.zero_()
    A[:, 0] = 2.0
    h.build()
    a = h.export()
    assert a["nnz"] == n and a["n_group"] == ng
    assert torch.equal(a["cols"], torch.zeros(n, dtype=torch.int32, device="cuda"))
    assert torch.equal(h.spdm(B), torch.full((n, 8), 2.0, device="cuda"))
    assert h.device_status() == 0 and h.check_arrays() == 0
    h.close()
    del h, A
    torch.cuda.empty_cache()
