"""GPU: the reference's own GCOO kernels (its kernel file compiled for sm_103a
into a cubin by the oracle recipe, launched with the reference plugin's
shapes) against this library on the same device buffers.

Two pins in one place: the reference's GPU code reproduces the recorded golden
fixtures (which were made by running the same kernel file under the host
emulator), and this library's conversion arrays and FP32 products are
bit-identical to the reference's, also at the full headline size. The cubin
exists only where the reference tree was available when the oracle was
built; without it these tests skip."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu
FIELDS = ("groupIndex", "nnzPerGroup", "vals", "rows", "cols")
GOLDEN = ["tiny", "edge_values", "empty_groups", "all_zero", "k1", "m3", "n_tail", "cpg1", "cpg2", "cpg8",
          "cpg16", "readme_800", "sweep_2048_s099", "ragged_1001x517"]


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def refgpu(torch):
    import oracle
    if not oracle.refgpu_available():
        pytest.skip("reference cubin not built on this machine (needs the reference tree at build time)")
    torch.zeros(1, device="cuda")  # make the runtime's context current before the driver-API loader runs
    oracle.refgpu()
    return oracle


def digest_np(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def digest(t):
    return digest_np(t.cpu().numpy())


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def same_bits(torch, x, y):
    """Equal bit patterns (NaN payloads and -0.0 included)."""
    x, y = x.cuda(), y.cuda()
    if x.dtype == torch.float32:
        x, y = x.view(torch.int32), y.view(torch.int32)
    return x.shape == y.shape and bool(torch.equal(x, y))


def test_reference_cubin_constants(refgpu):
    assert refgpu.refgpu_column_per_group() == 4
    assert refgpu.refgpu().refgpu_bs() == 128


@pytest.mark.parametrize("name", GOLDEN)
def test_reference_gpu_kernels_reproduce_fixtures_and_match_library(native, torch, refgpu, manifest, name):
    entry = manifest["cases"][name]
    A, B = golden_inputs(entry, name)
    dA = dev(torch, A)
    r = refgpu.refgpu_convert(dA, entry["cpg"])
    assert r["nnz"] == entry["nnz"]
    for f in FIELDS:
        assert digest(r[f]) == entry["digests"][f], f"reference GPU {f} differs from the fixture"
    ours = native.GcooHandle(dA, rows_per_group=entry["cpg"]).build()
    a = ours.export()
    for f in FIELDS:
        assert same_bits(torch, a[f], r[f]), f
    if entry["cpg"] == 4 and B is not None:
        dB = dev(torch, B)
        Cr = torch.full((A.shape[0], B.shape[1]), float("nan"), device="cuda")
        refgpu.refgpu_spdm(r, dB, Cr)
        if name == "edge_values":
            # NaN results carry the host ISA's payload in the fixture and the GPU's canonical NaN here:
            # compare NaN as NaN against the oracle, which reproduces the fixture bit for bit.
            ref = refgpu.spdm(refgpu.convert(A), B)
            assert digest_np(ref) == entry["digests"]["C"]
            x, y = Cr.cpu().numpy(), ref
            nx, ny = np.isnan(x), np.isnan(y)
            assert np.array_equal(nx, ny) and np.array_equal(x[~nx].view(np.uint32), y[~ny].view(np.uint32))
        else:
            assert digest(Cr) == entry["digests"]["C"], "reference GPU product differs from the fixture"
        Co = ours.spdm(dB)
        assert torch.equal(Co.view(torch.int32), Cr.view(torch.int32))  # same ISA: every bit, NaNs included


@pytest.mark.parametrize("size,sparsity", [(8192, 0.99), (16384, 0.995), (4096, 0.95)])
def test_full_size_bit_identical_to_reference_kernels(native, torch, refgpu, size, sparsity):
    """The headline workload (and a larger and a denser one): conversion arrays
    and the FP32 product, bit for bit, this library vs the reference's kernels."""
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense_torch(0x6C02, size, size, 1.0 - sparsity, device="cuda")
    B = dg.dense_pm1_torch(0x6C02, 5, size, size, device="cuda")
    r = refgpu.refgpu_convert(A, 4)
    h = native.GcooHandle(A).build()
    for _ in range(2):  # the first build sizes the arrays; the rebuild reads A once
        a = h.export()
        assert a["nnz"] == r["nnz"]
        for f in FIELDS:
            assert same_bits(torch, a[f], r[f]), f
        h.build()
    Cr = torch.empty(size, size, device="cuda")
    refgpu.refgpu_spdm(r, B, Cr)
    Co = h.spdm(B)
    assert torch.equal(Co.view(torch.int32), Cr.view(torch.int32))
    del r, Cr
    C2 = torch.empty_like(Co)
    h.multiply_by(B, C2)  # the end-to-end call gives the same bits
    assert torch.equal(C2.view(torch.int32), Co.view(torch.int32))
