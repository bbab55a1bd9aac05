"""Problem setup on the GPU (xs_ctx_create_on_device) against the reference.

The context built on the device is read back with xs_ctx_download and every
setup array is compared by sha256 with the arrays the reference's
grid_init_do_not_profile built (openmp-threading/GridInit.c:3; digests in
tests/golden/setup_*.json): the bar is bit-identical.  A full event run on the
device-built context must then give the reference's verification sum
(openmp-threading/Simulation.c:15-114; tests/golden/full_*.json).
"""
import numpy as np
import pytest

import xsbench_gb300 as X
from conftest import golden_json, product_inputs, sha

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide",
                                  "small_unionized", "small_hash", "small_nuclide",
                                  "large_hash", "large_nuclide", "large_unionized"])
def test_device_setup_matches_reference(name):
    g = golden_json("setup_" + name)
    inp = product_inputs(name)
    with X.Context(inp) as ctx:
        with ctx.download() as p:
            a = p.arrays()
            assert set(a) == set(g["sha256"])
            for k, v in a.items():
                assert sha(v) == g["sha256"][k], k
            assert p.sd.max_num_nucs == g["max_num_nucs"]
            assert p.sd.length_index_grid == g["length_index_grid"]
            del a
        f = golden_json("full_" + name)
        r = ctx.run_event()
        assert r.verification == f["verification"]


def test_device_setup_equals_host_setup_memcmp():
    """Same arrays as the host setup, element by element (tiny problem)."""
    inp = product_inputs("tiny_unionized")
    with X.grid_init(inp) as host, X.Context(inp) as ctx, ctx.download() as dev:
        a, b = host.arrays(), dev.arrays()
        assert set(a) == set(b)
        for k in a:
            assert np.array_equal(a[k], b[k]), k


def test_device_setup_ragged_gridpoints():
    """Gridpoint counts that are not a multiple of any block or bucket size:
    the device setup equals the host setup."""
    for gp, grid in ((3, "unionized"), (37, "unionized"), (1001, "hash"), (257, "nuclide")):
        inp = product_inputs("tiny_unionized", gridpoints=gp, grid=grid)
        with X.grid_init(inp) as host, X.Context(inp) as ctx, ctx.download() as dev:
            a, b = host.arrays(), dev.arrays()
            for k in a:
                assert np.array_equal(a[k], b[k]), (gp, grid, k)


def test_device_setup_rejects_bad_inputs():
    inp = product_inputs("tiny_hash")
    inp.hash_bins = 0
    with pytest.raises(X.XSError) as e:
        X.Context(inp)
    assert e.value.status == 1
    inp = product_inputs("tiny_unionized")
    inp.n_isotopes = 50                      # the material lists name nuclide 67
    with pytest.raises(X.XSError) as e:
        X.Context(inp)
    assert e.value.status == 1
