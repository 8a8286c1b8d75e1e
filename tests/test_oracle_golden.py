"""CPU: the oracle against the reference's own outputs (golden fixtures made by
running src/gcoo_spdm_kernels.cu under the host emulator), bit for bit."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_arrays, golden_inputs

FIELDS = ("groupIndex", "nnzPerGroup", "vals", "rows", "cols")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _cases(manifest):
    return sorted(manifest["cases"].items())


def test_manifest_pins_reference_constants(manifest):
    # src/constants.h:4-5 of the reference
    assert manifest["column_per_group"] == 4
    assert manifest["bs"] == 128
    assert len(manifest["cases"]) >= 14


@pytest.mark.parametrize("name", ["tiny", "edge_values", "empty_groups", "all_zero", "k1", "m3", "n_tail",
                                  "cpg1", "cpg2", "cpg8", "cpg16", "readme_800", "sweep_2048_s099",
                                  "ragged_1001x517"])
def test_oracle_matches_reference(oracle_mod, manifest, name):
    entry = manifest["cases"][name]
    A, B = golden_inputs(entry, name)
    g = oracle_mod.convert(A, entry["cpg"])
    assert g.nnz == entry["nnz"]
    for f in FIELDS:
        assert digest(getattr(g, f)) == entry["digests"][f], f
    if "C" in entry["digests"]:
        Cm = oracle_mod.spdm(g, B)
        assert digest(Cm) == entry["digests"]["C"]


def test_edge_values_semantics(oracle_mod, manifest):
    """-0.0 dropped, NaN / inf / denormals kept (the `v != 0.0` test)."""
    arr = golden_arrays("edge_values")
    A = arr["A"]
    g = oracle_mod.convert(A, 4)
    assert g.nnz == int(np.count_nonzero(A != 0))  # NaN != 0 is True, -0.0 != 0 is False
    assert not np.any((g.vals == 0))
    assert np.isnan(g.vals).sum() == 1
    assert np.isinf(g.vals).sum() == 2
    np.testing.assert_array_equal(g.vals.view(np.uint32), arr["vals"].view(np.uint32))


def test_small_fixture_arrays_match_digests(manifest):
    for name, entry in _cases(manifest):
        arr = golden_arrays(name)
        if entry["spec"]["kind"] == "hand" or name in ("tiny", "n_tail") or name.startswith("cpg"):
            for f in FIELDS:
                assert digest(arr[f]) == entry["digests"][f], (name, f)


def test_group_order_is_column_then_row(oracle_mod):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(3, 23, 17, 0.4)
    for cpg in (1, 2, 4, 8):
        g = oracle_mod.convert(A, cpg)
        for gg in range(g.n_group):
            s, e = g.groupIndex[gg], g.groupIndex[gg + 1]
            key = g.cols[s:e].astype(np.int64) * 1000 + g.rows[s:e]
            assert np.all(np.diff(key) > 0)
            assert np.all(g.rows[s:e] // cpg == gg)
        assert g.nnzPerGroup[-1] == 0
        assert g.groupIndex[-1] == g.nnz


def test_fp32_chain_close_to_fp64(oracle_mod):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(6, 300, 280, 0.1)
    B = dg.dense_pm1(6, 5, 280, 96)
    g = oracle_mod.convert(A)
    C32 = oracle_mod.spdm(g, B)
    C64 = oracle_mod.dense_gemm_f64(A, B)
    assert oracle_mod.rel_fro(C32, C64) < 1e-6
    np.testing.assert_allclose(oracle_mod.spdm_f64(g, B), C64, rtol=1e-12, atol=1e-12)


def test_multiply_by_equals_convert_then_spdm(oracle_mod):
    from gcoospdm_gb300 import datagen as dg
    A = dg.bernoulli_dense(9, 77, 65, 0.2)
    B = dg.dense_pm1(9, 5, 65, 33)
    C1 = oracle_mod.multiply_by(A, B, 4, 2)
    C2 = oracle_mod.spdm(oracle_mod.convert(A), B)
    np.testing.assert_array_equal(C1.view(np.uint32), C2.view(np.uint32))


def test_planted_mistake_is_caught(oracle_mod, manifest):
    """A wrong order (row, then column) inside the group must not match."""
    A, B = golden_inputs(manifest["cases"]["tiny"], "tiny")
    g = oracle_mod.convert(A)
    order = np.lexsort((g.cols, g.rows))
    assert digest(g.cols[order]) != manifest["cases"]["tiny"]["digests"]["cols"]
