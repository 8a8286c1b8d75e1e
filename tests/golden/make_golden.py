"""Record the reference's own outputs as golden fixtures.

Runs the reference kernel file (hclhkbu/gcoospdm src/gcoo_spdm_kernels.cu)
compiled for the host under the fiber emulator (oracle/ref_emu, built by
oracle/Makefile from the reference tree) on seeded and hand-made inputs, and
writes what it produced:

* ``<case>.npz`` -- inputs (for the hand-made cases) and the full outputs of
  small cases: groupIndex, nnzPerGroup, vals, rows, cols and C;
* ``manifest.json`` -- for every case its shape, seeds, nnz and the SHA-256 of
  each output array, so that large cases need no stored arrays.

Only runs where the reference tree is present (it is read through the
emulator library); the fixtures it writes are committed and are what the
tests compare against everywhere else.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from gcoospdm_gb300 import datagen as dg  # noqa: E402

FIELDS = ("groupIndex", "nnzPerGroup", "vals", "rows", "cols")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def edge_matrix() -> np.ndarray:
    """9 x 13 with -0.0 (dropped), NaN (kept), +-inf, denormals, huge values."""
    A = dg.bernoulli_dense(11, 9, 13, 0.45)
    A[0, 0] = -0.0
    A[0, 1] = np.float32(np.nan)
    A[1, 2] = np.float32(np.inf)
    A[2, 3] = np.float32(-np.inf)
    A[3, 4] = np.float32(1e-40)  # FP32 denormal
    A[4, 5] = np.float32(-1e-45)
    A[5, 6] = np.float32(3.0e38)
    A[6, 7] = -0.0
    A[8, 12] = np.float32(-3.0e38)
    return A


def cases():
    """(name, A, B or None, cpg, spec, store_full)."""
    out = []
    out.append(("tiny", dg.bernoulli_dense(1, 10, 7, 0.5), dg.dense_pm1(1, 5, 7, 5), 4,
                {"kind": "bernoulli", "seed": 1, "m": 10, "k": 7, "p": 0.5, "b_seed": 1, "b_stream": 5, "n": 5}, True))
    out.append(("edge_values", edge_matrix(), dg.dense_pm1(12, 5, 13, 3), 4, {"kind": "hand", "m": 9, "k": 13, "n": 3}, True))
    A = dg.bernoulli_dense(13, 16, 8, 0.6)
    A[4:8] = 0
    A[12:16] = 0
    out.append(("empty_groups", A, dg.dense_pm1(13, 5, 8, 4), 4, {"kind": "hand", "m": 16, "k": 8, "n": 4}, True))
    out.append(("all_zero", np.zeros((5, 6), np.float32), dg.dense_pm1(14, 5, 6, 3), 4, {"kind": "hand", "m": 5, "k": 6, "n": 3}, True))
    out.append(("k1", dg.bernoulli_dense(15, 9, 1, 0.7), dg.dense_pm1(15, 5, 1, 7), 4, {"kind": "hand", "m": 9, "k": 1, "n": 7}, True))
    out.append(("m3", dg.bernoulli_dense(16, 3, 5, 0.7), dg.dense_pm1(16, 5, 5, 1), 4, {"kind": "hand", "m": 3, "k": 5, "n": 1}, True))
    out.append(("n_tail", dg.bernoulli_dense(17, 12, 33, 0.3), dg.dense_pm1(17, 5, 33, 130), 4,
                {"kind": "bernoulli", "seed": 17, "m": 12, "k": 33, "p": 0.3, "b_seed": 17, "b_stream": 5, "n": 130}, True))
    A = dg.bernoulli_dense(18, 37, 29, 0.35)
    for cpg in (1, 2, 8, 16):
        out.append((f"cpg{cpg}", A, None, cpg, {"kind": "bernoulli", "seed": 18, "m": 37, "k": 29, "p": 0.35}, True))
    out.append(("readme_800", dg.bernoulli_dense(6, 800, 800, 0.1), dg.dense_pm1(6, 5, 800, 800), 4,
                {"kind": "bernoulli", "seed": 6, "m": 800, "k": 800, "p": 0.1, "b_seed": 6, "b_stream": 5, "n": 800}, False))
    out.append(("sweep_2048_s099", dg.bernoulli_dense(7, 2048, 2048, 0.01), dg.dense_pm1(7, 5, 2048, 256), 4,
                {"kind": "bernoulli", "seed": 7, "m": 2048, "k": 2048, "p": 0.01, "b_seed": 7, "b_stream": 5, "n": 256}, False))
    out.append(("ragged_1001x517", dg.bernoulli_dense(8, 1001, 517, 0.05), dg.dense_pm1(8, 5, 517, 333), 4,
                {"kind": "bernoulli", "seed": 8, "m": 1001, "k": 517, "p": 0.05, "b_seed": 8, "b_stream": 5, "n": 333}, False))
    return out


def main() -> None:
    if not oracle.ref_available():
        oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference emulation not built (reference tree absent)")
    manifest = {"generator": "tests/golden/make_golden.py",
                "source": "hclhkbu/gcoospdm src/gcoo_spdm_kernels.cu under oracle/ref_emu",
                "column_per_group": int(oracle.ref().ref_emu_column_per_group()),
                "bs": int(oracle.ref().ref_emu_bs()), "cases": {}}
    for name, A, B, cpg, spec, full in cases():
        g = oracle.ref_convert(A, cpg)
        entry = {"spec": spec, "cpg": cpg, "nnz": g.nnz, "n_group": g.n_group,
                 "digests": {f: digest(getattr(g, f)) for f in FIELDS}}
        arrays = {f: getattr(g, f) for f in FIELDS}
        if B is not None:
            Cm = oracle.ref_spdm(g, B)
            entry["digests"]["C"] = digest(Cm)
            arrays["C"] = Cm
        if full:
            if spec["kind"] == "hand":
                arrays["A"] = A
                if B is not None:
                    arrays["B"] = B
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        else:
            # keep the first entries of each output to make a mismatch readable
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                                **{f: a.ravel()[:256] for f, a in arrays.items()})
        manifest["cases"][name] = entry
        print(name, "nnz", g.nnz)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
