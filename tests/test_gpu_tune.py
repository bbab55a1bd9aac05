"""The autotuner (xs_autotune): it keeps the hash bit-exact whatever grid and
shapes it picks, caches its choice by (device, problem) and reinstalls a
cached choice without timing."""
import json
import time

import pytest

import xsbench_gb300 as X
from conftest import golden_json, product_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_nuclide"])
def test_autotune_keeps_results_and_caches(tmp_path, name):
    g = golden_json("full_" + name)
    cache = str(tmp_path / "tune.json")
    inp = product_inputs(name)
    with X.grid_init(inp) as p:
        with X.Context(inp, p) as ctx:
            best = ctx.autotune(cache)
            assert best["kernel"] in ("plain", "batched")
            assert best["grid"] in ("unionized", "nuclide", "hash")
            for kernel in ("plain", "batched"):
                assert ctx.run_event(kernel=kernel).verification == g["verification"]
            r = ctx.run_event(kernel=best["kernel"])
            assert r.verification == g["verification"]
        entries = json.load(open(cache))
        assert len(entries) == 1
        (key, val), = entries.items()
        assert "GB300" in key or "|grid=" in key
        assert val["lookups_per_s"] > 0
        assert val["fuel_lanes"] in (1, 2, 4)
        with X.Context(inp, p) as ctx2:
            t0 = time.perf_counter()
            best2 = ctx2.autotune(cache)
            assert time.perf_counter() - t0 < 5.0
            assert best2 == best
            assert ctx2.run_event(kernel=best2["kernel"]).verification == g["verification"]
