"""The autotuner (xs_autotune): it keeps the hash bit-exact whatever grid and
shapes it picks, caches its choice by (device, problem) and reinstalls a
cached choice without timing."""
import json
import time

import pytest

import xsbench_gb300 as X
from conftest import golden_json, product_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_nuclide", "tiny_hash"])
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
        assert val["block"] == best["block"] in (128, 256, 512)
        assert val["guided"] in (0, 1) and val["tile_sort"] in (-1, 0, 1)
        with X.Context(inp, p) as ctx2:
            t0 = time.perf_counter()
            best2 = ctx2.autotune(cache)
            assert time.perf_counter() - t0 < 5.0
            assert best2 == best
            assert ctx2.run_event(kernel=best2["kernel"]).verification == g["verification"]


@pytest.mark.parametrize("block", [128, 256, 512])
def test_every_block_shape_keeps_the_hash(block):
    """The block shapes the tuner chooses among (threads per block of the
    plain kernel and of the persistent list kernel, the threads per SM kept):
    each gives the reference's verification sum and argmax vector."""
    import numpy as np
    from conftest import sha
    name = "tiny_hash"
    g = golden_json("full_" + name)
    inp = product_inputs(name)
    with X.grid_init(inp) as p, X.Context(inp, p) as ctx:
        for kernel in ("plain", "batched"):
            for arith in ("fast", "exact"):
                idx = np.empty(g["lookups"], np.uint8)
                r = ctx.run_event(kernel=kernel, arith=arith, block=block, max_idx_out=idx)
                assert r.verification == g["verification"], (kernel, arith)
                assert sha(idx) == g["sha256_max_idx"], (kernel, arith)
        with pytest.raises(X.XSError):
            ctx.run_event(block=64)
        with pytest.raises(X.XSError):   # the plain kernel's block must divide its tile
            ctx.run_event(block=512, tile=256)
