"""Shared test setup: the `gpu` marker, the in-tree builds, golden fixtures."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native():
    import gcoospdm_gb300 as g
    g.build()
    return g


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden_arrays(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def golden_inputs(entry, name):
    """Regenerate (A, B) of a golden case from its seeds (or load hand-made ones)."""
    from gcoospdm_gb300 import datagen as dg
    spec = entry["spec"]
    if spec["kind"] == "hand":
        arr = golden_arrays(name)
        return arr["A"], arr.get("B")
    A = dg.bernoulli_dense(spec["seed"], spec["m"], spec["k"], spec["p"])
    B = None
    if "n" in spec:
        B = dg.dense_pm1(spec["b_seed"], spec["b_stream"], spec["k"], spec["n"])
    return A, B
