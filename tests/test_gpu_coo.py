"""GPU: sparse-input ingestion (gcoo_create_coo). The arrays must equal, bit
for bit, those of writing the triplets into a zero dense buffer in order (a
later duplicate overwrites, as the reference's Matrix Market reader does) and
converting it; the multiply must equal the dense-built handle's."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FIELDS = ("groupIndex", "nnzPerGroup", "vals", "rows", "cols")


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def densify(m, k, rows, cols, vals):
    A = np.zeros((m, k), np.float32)
    for r, c, v in zip(rows, cols, vals):  # file order: the last write wins
        A[r, c] = v
    return A


def triplets(seed, m, k, count, dup_frac=0.2, zero_frac=0.05):
    from gcoospdm_gb300 import datagen as dg
    h = dg.hash_np(seed, 50, 0, 4 * count)
    rows = (h[:count] % np.uint64(m)).astype(np.int32)
    cols = (h[count:2 * count] % np.uint64(k)).astype(np.int32)
    vals = dg.pm1_from_hash(h[2 * count:3 * count])
    nd = int(count * dup_frac)
    rows[-nd:], cols[-nd:] = rows[:nd], cols[:nd]  # duplicates appear later, with other values
    nz = int(count * zero_frac)
    vals[count // 2:count // 2 + nz] = 0.0
    vals[-1] = -0.0
    return rows, cols, vals


@pytest.mark.parametrize("m,k,count,cpg", [(300, 200, 5000, 4), (97, 1000, 3000, 8), (1000, 33, 9000, 1),
                                           (4096, 4096, 200_000, 4)])
def test_coo_matches_densify_then_convert(native, oracle_mod, torch, m, k, count, cpg):
    rows, cols, vals = triplets(m + count, m, k, count)
    A = densify(m, k, rows, cols, vals)
    g = oracle_mod.convert(A, cpg)
    t = [torch.from_numpy(x).cuda() for x in (rows, cols, vals)]
    h = native.GcooHandle.from_coo(*t, m=m, k=k, rows_per_group=cpg).build()
    a = h.export()
    assert a["nnz"] == g.nnz
    for f in FIELDS:
        np.testing.assert_array_equal(a[f].cpu().numpy(), getattr(g, f), err_msg=f)
    from gcoospdm_gb300 import datagen as dg
    B = dg.dense_pm1_torch(m, 5, k, 96, device="cuda")
    hd = native.GcooHandle(torch.from_numpy(A).cuda(), rows_per_group=cpg).build()
    assert torch.equal(h.spdm(B), hd.spdm(B))
    assert h.device_status() == 0


def test_coo_rejects_out_of_range(native, torch):
    rows = torch.tensor([0, 5, 2], dtype=torch.int32, device="cuda")
    cols = torch.tensor([1, 1, 9], dtype=torch.int32, device="cuda")
    vals = torch.ones(3, device="cuda")
    h = native.GcooHandle.from_coo(rows, cols, vals, m=4, k=4)
    with pytest.raises(native.GcooError) as e:
        h.build()
    assert e.value.status == 1


def test_coo_empty_and_all_zero(native, torch):
    e = torch.zeros(0, dtype=torch.int32, device="cuda")
    h = native.GcooHandle.from_coo(e, e, torch.zeros(0, device="cuda"), m=10, k=7).build()
    assert h.nnz == 0
    B = torch.ones(7, 5, device="cuda")
    assert torch.equal(h.spdm(B), torch.zeros(10, 5, device="cuda"))
    z = torch.zeros(3, dtype=torch.int32, device="cuda")
    h2 = native.GcooHandle.from_coo(z, z, torch.zeros(3, device="cuda"), m=10, k=7).build()
    assert h2.nnz == 0


def test_coo_zipf_matches_dense_build(native, torch):
    """The irregular workload's pattern at 16384^2, ingested without densifying."""
    from gcoospdm_gb300 import datagen as dg
    m = k = 16384
    rows, cols, vals = dg.zipf_coo(5, m, k, 300_000, alpha=2.0, cap=4096)
    r, c, v = (torch.from_numpy(rows.astype(np.int32)).cuda(), torch.from_numpy(cols.astype(np.int32)).cuda(),
               torch.from_numpy(vals).cuda())
    hc = native.GcooHandle.from_coo(r, c, v, m=m, k=k).build()
    A = torch.zeros(m, k, device="cuda")
    A[r.long(), c.long()] = v
    hd = native.GcooHandle(A).build()
    ac, ad = hc.export(), hd.export()
    for f in FIELDS:
        assert torch.equal(ac[f], ad[f]), f
    B = dg.dense_pm1_torch(5, 5, k, 256, device="cuda")
    assert torch.equal(hc.spdm(B), hd.spdm(B))


def test_matrix_market_file_through_the_handle_and_the_driver(native, oracle_mod, torch, tmp_path):
    """The reference driver's -file= input: C = M x M for the matrix M of a
    Matrix Market file (symmetric, lower triangle stored, with duplicates
    and explicit zeros). GcooHandle.from_matrix_market gives the oracle's
    bits on the densified M; `gcoo_main -file= -check=1` passes its FP64
    check."""
    import os
    import subprocess
    n, e = 300, 2500
    rng = np.random.default_rng(61)
    r = rng.integers(1, n + 1, size=e)
    c = rng.integers(1, n + 1, size=e)
    r, c = np.maximum(r, c), np.minimum(r, c)
    v = rng.uniform(-1.0, 1.0, size=e).astype(np.float32)
    v[::17] = 0.0
    path = tmp_path / "sym.mtx"
    path.write_text("%%MatrixMarket matrix coordinate real symmetric\n% test matrix\n"
                    f"{n} {n} {e}\n" + "".join(f"{a} {b} {x:.9g}\n" for a, b, x in zip(r, c, v)))
    rows, cols, vals, m, k = native.read_matrix_market(str(path))
    M = densify(m, k, rows, cols, vals)
    assert np.array_equal(M, M.T)
    h = native.GcooHandle.from_matrix_market(str(path)).build()
    assert h.nnz == int(np.count_nonzero(M))
    got = h.spdm(torch.from_numpy(M).cuda()).cpu().numpy()
    ref = oracle_mod.spdm(oracle_mod.convert(M), M)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    main = os.path.join(os.path.dirname(native.__file__), "_build", "gcoo_main")
    out = subprocess.run([main, f"-file={path}", "-algo=gcoospdm", "-check=1", "-reps=3"],
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "Read mtx file" in out.stdout and "Test passed" in out.stdout and "Time:" in out.stdout
