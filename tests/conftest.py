"""Shared test set-up.

Markers: ``gpu`` -- needs an sm_103 GPU (GB300); everything else runs on CPU.
The golden fixtures under tests/golden/ were dumped from the reference's own
openmp-threading build by tests/golden/make_golden.py.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")

# name -> (size, grid, lookups, gridpoints, hash_bins); the same table as make_golden.py
CONFIGS = {
    "tiny_unionized": dict(size="small", grid="unionized", gridpoints=1000, lookups=200000),
    "tiny_hash": dict(size="small", grid="hash", gridpoints=1000, lookups=200000, hash_bins=500),
    "tiny_nuclide": dict(size="small", grid="nuclide", gridpoints=1000, lookups=200000),
    "small_unionized": dict(size="small", grid="unionized"),
    "small_hash": dict(size="small", grid="hash"),
    "small_nuclide": dict(size="small", grid="nuclide"),
    "large_unionized": dict(size="large", grid="unionized"),
    "large_hash": dict(size="large", grid="hash"),
    "large_nuclide": dict(size="large", grid="nuclide"),
    "xl_hash": dict(size="XL", grid="hash", lookups=100000000),
    "xl_nuclide": dict(size="XL", grid="nuclide", lookups=100000000),
}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) GPU")


def golden_json(name: str) -> dict:
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def golden_npz(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).data).hexdigest()


def oracle_config(name: str):
    import oracle
    c = CONFIGS[name]
    return oracle.Config(size=c["size"], grid=c["grid"], lookups=c.get("lookups"),
                         n_gridpoints=c.get("gridpoints"), hash_bins=c.get("hash_bins", 10000))


def product_inputs(name: str, **over):
    import xsbench_gb300 as X
    c = dict(CONFIGS[name])
    c.update(over)
    return X.make_inputs(method="event", **c)


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (both in-tree)."""
    import oracle
    from xsbench_gb300 import build as B
    B.build()
    oracle.build()
    yield
