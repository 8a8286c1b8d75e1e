"""GPU: the plain FP32 multiply through the C ABI, bit-identical to the
reference's output (golden fixtures) and to the oracle; relative Frobenius
error against FP64 at the full benchmark size."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu


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


def same_bits(x, y):
    """Bitwise equality, NaNs compared as NaN (payloads differ across ISAs)."""
    x, y = np.asarray(x, np.float32), np.asarray(y, np.float32)
    nx, ny = np.isnan(x), np.isnan(y)
    return bool(np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint32), y[~ny].view(np.uint32)))


WITH_C = ["tiny", "edge_values", "empty_groups", "all_zero", "k1", "m3", "n_tail", "readme_800",
          "sweep_2048_s099", "ragged_1001x517"]


@pytest.mark.parametrize("name", WITH_C)
def test_spdm_matches_reference_output(native, oracle_mod, torch, manifest, name):
    entry = manifest["cases"][name]
    A, B = golden_inputs(entry, name)
    h = native.GcooHandle(dev(torch, A)).build()
    Cg = h.spdm(dev(torch, B)).cpu().numpy()
    if name == "edge_values":
        ref = oracle_mod.spdm(oracle_mod.convert(A), B)  # oracle == reference bit-for-bit on this case
        assert digest(ref) == entry["digests"]["C"]
        assert same_bits(Cg, ref)
    else:
        assert digest(Cg) == entry["digests"]["C"]
    assert h.device_status() == 0


@pytest.mark.parametrize("vec,warps,col_warps", [(1, 0, 0), (2, 0, 0), (4, 0, 0), (4, 4, 1), (4, 16, 4),
                                                 (2, 8, 2), (1, 32, 8)])
def test_launch_shapes_bit_identical(native, oracle_mod, torch, vec, warps, col_warps):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(21, 1000, 900, 0.03)
    B = dg.dense_pm1(21, 5, 900, 520)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A), vec=vec, warps=warps, col_warps=col_warps).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)


@pytest.mark.parametrize("cpg", [1, 2, 8, 16, 32])
def test_any_group_height_same_result(native, oracle_mod, torch, cpg):
    """The per-element fmaf chain does not depend on the group height."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(22, 777, 640, 0.02)
    B = dg.dense_pm1(22, 5, 640, 256)
    ref = oracle_mod.spdm(oracle_mod.convert(A, 4), B)
    h = native.GcooHandle(dev(torch, A), rows_per_group=cpg).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)


@pytest.mark.parametrize("n", [1, 3, 31, 33, 130, 257, 1000])
def test_odd_widths(native, oracle_mod, torch, n):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(23, 150, 120, 0.1)
    B = dg.dense_pm1(23, 5, 120, n)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A)).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)


def test_misaligned_operands(native, oracle_mod, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(24, 200, 160, 0.05)
    B = dg.dense_pm1(24, 5, 160, 128)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A)).build()
    bufB = torch.zeros(B.size + 1, device="cuda")
    bufB[1:] = dev(torch, B.ravel())
    bufC = torch.zeros(200 * 128 + 1, device="cuda")
    Bv, Cv = bufB[1:].view(160, 128), bufC[1:].view(200, 128)
    h.spdm(Bv, Cv)
    assert same_bits(Cv.cpu().numpy(), ref)


def test_heavy_group_multi_chunk(native, oracle_mod, torch):
    """A group with more entries than one shared-memory chunk (2048)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(25, 40, 6000, 0.002)
    A[1, :] = dg.dense_pm1(25, 9, 1, 6000)[0]
    A[2, ::2] = dg.dense_pm1(25, 10, 1, 3000)[0]
    B = dg.dense_pm1(25, 5, 6000, 200)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A)).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)


@pytest.mark.parametrize("density,n", [(0.06, 256), (0.12, 520), (0.3, 256)])
def test_uniformly_long_rows(native, oracle_mod, torch, density, n):
    """Rows of ~490, ~980 and ~2460 entries, not skewed: groups of four rows
    overflow one staging chunk, so the launch takes two rows or one per CTA
    (the first two) or stages in several passes (the last); the same bits
    as the oracle's chain in every case."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(26, 600, 8192, density)
    B = dg.dense_pm1(26, 5, 8192, n)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A)).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)
    assert h.device_status() == 0


@pytest.mark.parametrize("n", [256, 200, 98, 36])
def test_long_rows_of_skewed_matrices(native, oracle_mod, torch, n):
    """Skewed row lengths: rows of at least 256 entries go to the long-row
    kernel (a deep shared-memory ring of B row pieces per warp), the others to
    the row kernel. Rows at the threshold, long rows starting on odd and even
    entries, lengths that are not multiples of 32, a last column tile cut
    short; n % 4 != 0 leaves every row to the row kernel. Bit-identical to the
    oracle either way, also after a staged rebuild and from COO input."""
    from gcoospdm_gb300 import datagen as dg
    m, k = 600, 5000
    A = dg.bernoulli_dense(31, m, k, 0.002)
    rng = np.random.default_rng(32)
    for r, length in ((3, 255), (4, 256), (5, 257), (6, 4999), (7, 1000), (8, 1001), (100, 3333), (599, 300)):
        A[r, :] = 0
        cols = np.sort(rng.choice(k, size=length, replace=False))
        v = rng.uniform(-1.0, 1.0, size=length).astype(np.float32)
        A[r, cols] = np.where(v == 0.0, np.float32(0.5), v)
    B = dg.dense_pm1(33, 1, k, n)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    dA, dB = dev(torch, A), dev(torch, B)
    h = native.GcooHandle(dA).build()
    assert same_bits(h.spdm(dB).cpu().numpy(), ref)
    h.build()
    assert same_bits(h.spdm(dB).cpu().numpy(), ref)
    r, c = torch.nonzero(dA, as_tuple=True)
    hc = native.GcooHandle.from_coo(r.int().contiguous(), c.int().contiguous(), dA[r, c].contiguous(), m, k).build()
    assert same_bits(hc.spdm(dB).cpu().numpy(), ref)
    # the long rows run on a side stream forked from the caller's: captured and replayed in a graph
    Cd = torch.empty(m, n, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        h.spdm(dB, Cd, stream=s)
    Cd.zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert same_bits(Cd.cpu().numpy(), ref)


@pytest.mark.parametrize("n,vec", [(4100, 4), (4102, 2), (4099, 1), (1920, 4)])
def test_short_rows_walk_several_column_tiles(native, oracle_mod, torch, n, vec):
    """Short rows (about 2.5 entries) over many groups and a wide, ragged n:
    each warp walks several column tiles (in pairs, then one) per staging of
    its group's entries. Same bits as the oracle."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(26, 8192, 512, 0.005)
    A[5, :] = 0.0  # an empty row inside a walked group
    B = dg.dense_pm1(26, 5, 512, n)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    h = native.GcooHandle(dev(torch, A), vec=vec).build()
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), ref)
    assert h.device_status() == 0


@pytest.mark.parametrize("name", ["tiny", "edge_values", "empty_groups", "all_zero", "k1", "m3", "n_tail",
                                  "readme_800", "ragged_1001x517"])
def test_group_order_matches_reference_output(native, oracle_mod, torch, manifest, name):
    """The GCOO-order FP32 walk (forced) gives the reference's bits too."""
    entry = manifest["cases"][name]
    A, B = golden_inputs(entry, name)
    h = native.GcooHandle(dev(torch, A), fp32_order="groups").build()
    Cg = h.spdm(dev(torch, B)).cpu().numpy()
    assert same_bits(Cg, oracle_mod.spdm(oracle_mod.convert(A), B))
    if name != "edge_values":
        assert digest(Cg) == entry["digests"]["C"]


@pytest.mark.parametrize("m,k,n,vec", [(1003, 640, 1000, 0), (1003, 640, 1002, 0), (1003, 640, 999, 0),
                                       (512, 4096, 2048, 2), (64, 256, 8192, 0)])
def test_group_order_block_clustered_auto_and_forced(native, oracle_mod, torch, m, k, n, vec):
    """Block-clustered A (the rows of a group share their columns): the
    automatic choice takes the GCOO-order walk; both walks and the oracle agree
    bit for bit, with ragged m and n of every alignment."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.block_dense(31, m, k, 0.3)
    B = dg.dense_pm1(31, 5, k, n)
    ref = oracle_mod.spdm(oracle_mod.convert(A), B)
    dA, dB = dev(torch, A), dev(torch, B)
    for order in ("auto", "groups", "rows"):
        h = native.GcooHandle(dA, vec=vec, fp32_order=order).build()
        assert same_bits(h.spdm(dB).cpu().numpy(), ref), order
    # uniform random sparsity: the auto choice stays with rows; forcing groups is still exact
    A2 = dg.bernoulli_dense(32, m, k, 0.02)
    ref2 = oracle_mod.spdm(oracle_mod.convert(A2), B)
    h = native.GcooHandle(dev(torch, A2), fp32_order="groups").build()
    assert same_bits(h.spdm(dB).cpu().numpy(), ref2)


def test_group_order_needs_groups_of_four(native, torch):
    A = torch.zeros(64, 64, device="cuda")
    with pytest.raises(native.GcooError) as e:
        native.GcooHandle(A, rows_per_group=8, fp32_order="groups")
    assert e.value.status == 5


def test_reference_layout_view_entry(native, oracle_mod, torch, manifest):
    """gcoo_spdm_view on arrays in the reference's own layout."""
    for name in ("readme_800", "n_tail", "empty_groups"):
        entry = manifest["cases"][name]
        A, B = golden_inputs(entry, name)
        g = oracle_mod.convert(A)
        Cg = native.spdm_view(g.m, g.k, 4, dev(torch, g.groupIndex), dev(torch, g.nnzPerGroup),
                              dev(torch, g.vals), dev(torch, g.rows), dev(torch, g.cols), dev(torch, B))
        assert digest(Cg.cpu().numpy()) == entry["digests"]["C"], name


def test_plugin_mirror_and_builder(native, torch, manifest):
    entry = manifest["cases"]["readme_800"]
    A, B = golden_inputs(entry, "readme_800")
    dA, dB = dev(torch, A), dev(torch, B)
    C1 = torch.empty(800, 800, device="cuda")
    g = native.SpGemmBuilder.getShGemmAlgo(dA, 800, 800, "gcoospdm")
    assert g.mutiplyBy(dB, 800, 800, C1) == 0.0
    assert digest(C1.cpu().numpy()) == entry["digests"]["C"]
    g.build()
    assert g.m_nGroup == 200 and int(g.m_pGroupIndex[-1]) == entry["nnz"]
    C2 = torch.empty_like(C1)
    assert g.runKernelTest(dB, 800, 800, C2) == 0.0
    assert torch.equal(C1, C2)
    assert native.SpGemmBuilder.getShGemmAlgo(dA, 800, 800, "ell") is None
    # the reference's auxiliary "csr" plugin (a baseline): the same bits
    csr = native.SpGemmBuilder.getShGemmAlgo(dA, 800, 800, "csr")
    C3 = torch.full_like(C1, float("nan"))
    assert csr.mutiplyBy(dB, 800, 800, C3) == 0.0
    assert torch.equal(C3, C1)
    csr.build()
    C3.fill_(float("nan"))
    assert csr.runKernelTest(dB, 800, 800, C3) == 0.0
    assert torch.equal(C3, C1)
    del csr
    # the other orientation: C = B x self
    assert g.mutiply(dB, 800, 800, C2) == 0.0
    ref = (dB.double() @ dA.double()).float()
    assert float((C2 - ref).abs().max()) < 1e-4


@pytest.mark.parametrize("m,k,p,s", [(300, 200, 96, 0.9), (1000, 777, 130, 0.98), (64, 4096, 512, 0.99)])
def test_left_orientation_bit_identical(native, oracle_mod, torch, m, k, p, s):
    """C = D x A equals, bit for bit, the oracle's chain on the transposed
    problem (C^T = A^T x D^T: each C element over A's rows in order)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(80 + m, m, k, 1.0 - s)
    D = dg.dense_pm1(80 + m, 5, p, m)
    ref_t = oracle_mod.spdm(oracle_mod.convert(np.ascontiguousarray(A.T)), np.ascontiguousarray(D.T))
    h = native.GcooHandle(dev(torch, A)).build()
    Cg = h.spdm_left(dev(torch, D)).cpu().numpy()
    assert same_bits(Cg, np.ascontiguousarray(ref_t.T))
    Cg2 = h.spdm_left(dev(torch, D)).cpu().numpy()  # second call reuses the column layout
    assert same_bits(Cg2, Cg)


def test_multiply_by_steady_state_and_determinism(native, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(26, 2048, 2048, 0.01)
    B = dg.dense_pm1(26, 5, 2048, 2048)
    h = native.GcooHandle(dev(torch, A))
    dB = dev(torch, B)
    C1 = h.multiply_by(dB)
    C2 = h.multiply_by(dB)
    C3 = h.spdm(dB)
    assert torch.equal(C1, C2) and torch.equal(C1, C3)


def test_multiply_by_on_changing_matrices(native, oracle_mod, torch):
    """mutiplyBy with A's contents changing between calls: rebuilds with
    room (staged), denser than the arrays' room (the staged attempt falls
    back to the two-pass build), skewed (the long/short split), back to
    sparse. Every result is bit-identical to the oracle's."""
    from gcoospdm_gb300 import datagen as dg
    m, k, n = 1500, 2048, 256
    rng = np.random.default_rng(77)
    sparse = dg.bernoulli_dense(71, m, k, 0.01)
    dense = dg.bernoulli_dense(72, m, k, 0.2)
    skewed = dg.bernoulli_dense(73, m, k, 0.005)
    for r, length in ((5, 1500), (600, 800), (1499, 300)):
        cols = np.sort(rng.choice(k, size=length, replace=False))
        v = rng.uniform(-1.0, 1.0, size=length).astype(np.float32)
        skewed[r, :] = 0.0
        skewed[r, cols] = np.where(v == 0.0, np.float32(0.5), v)
    B = dg.dense_pm1(74, 1, k, n)
    dA, dB = dev(torch, sparse), dev(torch, B)
    h = native.GcooHandle(dA)
    Cd = torch.empty(m, n, device="cuda")
    for A in (sparse, sparse, dense, dense, skewed, skewed, sparse):
        dA.copy_(dev(torch, A))
        Cd.fill_(float("nan"))
        h.multiply_by(dB, Cd)
        ref = oracle_mod.spdm(oracle_mod.convert(A), B)
        assert same_bits(Cd.cpu().numpy(), ref)
        assert h.device_status() == 0



def test_width_beyond_grid_limit_is_refused(native, oracle_mod, torch):
    """Column tiles lie along the grid's y dimension: B wider than 65535
    tiles of the chosen shape is refused with GCOO_ERROR_CUDA before any
    launch, and the handle stays usable. With the launch shape given (two
    warps per row, which also keeps four rows per CTA), groups of 4 rows of
    600 entries (more than one staging chunk) take one column tile per CTA
    (groups that fit one chunk walk several, which widens the reach), n odd
    one column per lane: 64-column tiles. B (10 GB) is never read."""
    from gcoospdm_gb300 import datagen as dg
    native.autotune_clear()  # the given shape, not a tuned wider one
    A = dg.bernoulli_dense(42, 8, 600, 1.0)
    h = native.GcooHandle(dev(torch, A), fp32_order="rows", col_warps=2).build()
    n = 65535 * 64 + 1
    wide = torch.empty(600, n, device="cuda")
    with pytest.raises(native.GcooError) as e:
        h.spdm(wide)
    assert e.value.status == 3
    del wide
    B = dg.dense_pm1(42, 5, 600, 33)
    assert same_bits(h.spdm(dev(torch, B)).cpu().numpy(), oracle_mod.spdm(oracle_mod.convert(A), B))
    assert h.device_status() == 0

def test_error_norm_kernel_matches_oracle(native, oracle_mod, torch):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(27, 500, 400, 0.05)
    B = dg.dense_pm1(27, 5, 400, 300)
    h = native.GcooHandle(dev(torch, A)).build()
    Cg = h.spdm(dev(torch, B))
    e_gpu = h.error_norm(dev(torch, B), Cg)
    C64 = oracle_mod.dense_gemm_f64(A, B)
    e_cpu = oracle_mod.rel_fro(Cg.cpu().numpy(), C64)
    assert e_gpu == pytest.approx(e_cpu, rel=1e-6, abs=1e-12)
    assert e_gpu < 1e-6
    # a planted error is seen
    Cbad = Cg.clone()
    Cbad[3, 7] += 1.0
    assert h.error_norm(dev(torch, B), Cbad) > 1e-4


def test_full_size_fp32_within_tolerance(native, torch):
    """n=8192, s=0.99 (the headline point): ||C - C64||_F / ||C64||_F <= 1e-5."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(8192, 8192, 8192, 0.01)
    B = dg.dense_pm1(8192, 5, 8192, 8192)
    h = native.GcooHandle(dev(torch, A)).build()
    dB = dev(torch, B)
    Cg = h.spdm(dB)
    err = h.error_norm(dB, Cg)
    assert err <= 1e-5
    # and equal, bit for bit, to the oracle on a slice of rows
    rows = slice(4096, 4096 + 64)
    sub = A[rows]
    from oracle import convert, spdm
    ref = spdm(convert(sub), B)
    assert np.array_equal(Cg[rows].cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_fp32_multiply_replays_from_a_cuda_graph(native, torch):
    """The persistent-handle path: build once, capture the multiply, replay it
    with new B contents (no allocation or synchronisation inside gcoo_spdm)."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(29, 1024, 768, 0.02, device="cuda")
    h = native.GcooHandle(A).build()
    B = dg.dense_pm1_torch(29, 5, 768, 512, device="cuda")
    Cd = torch.empty(1024, 512, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        h.spdm(B, Cd, stream=s)
    for seed in (30, 31):
        B.copy_(dg.dense_pm1_torch(seed, 5, 768, 512, device="cuda"))
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(Cd, h.spdm(B))
