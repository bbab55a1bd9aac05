"""GPU parity: the sm_103a kernels through the C ABI against the reference.

Bars (the reference: openmp-threading built from source, tests/golden/):
  * verification sum and the whole per-lookup argmax vector: bit-exact;
  * EXACT arithmetic: every macro_xs bit-identical (sha256 of the N x 5 array);
  * FAST arithmetic: each lookup's macro_xs vector within 1e-12 relative of the
    reference's, in the max norm: max_k |a_k - b_k| <= 1e-12 * max_k |b_k|.
    The vector norm is the meaningful one: a channel whose terms cancel
    (extrapolated, negative micro xs; e.g. a sum of 5.6 in absolute terms that
    lands on -2e-4) carries the reference's own rounding error of ~1e-16 of the
    terms, so its element-wise relative difference can exceed 1e-12 while the
    absolute difference is half an ulp of the terms.  The worst vector
    relative difference observed is ~6e-16.
"""
import numpy as np
import pytest

import oracle
import xsbench_gb300 as X
from conftest import golden_json, golden_npz, oracle_config, product_inputs, sha

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
_CACHE = {}


def ctx_for(name):
    if name not in _CACHE:
        for k in list(_CACHE):          # keep one large problem resident at a time
            if not k.startswith("tiny"):
                _CACHE.pop(k)[1].close()
        inp = product_inputs(name)
        prob = X.grid_init(inp)
        ctx = X.Context(inp, prob)
        _CACHE[name] = (prob, ctx)
    return _CACHE[name][1]


@pytest.fixture(scope="module", autouse=True)
def _cleanup():
    yield
    for prob, ctx in _CACHE.values():
        ctx.close()
        prob.close()
    _CACHE.clear()


def rel_err(a, b):
    """Largest per-lookup relative difference of the macro_xs vectors (max norm)."""
    num = np.max(np.abs(a - b), axis=1)
    den = np.maximum(np.max(np.abs(b), axis=1), 1e-300)
    return float(np.max(num / den))


def run(ctx, n, **kw):
    macro = np.empty((n, 5), np.float64)
    idx = np.empty(n, np.uint8)
    r = ctx.run_event(macro_out=macro, max_idx_out=idx, **kw)
    return r, macro, idx


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide"])
@pytest.mark.parametrize("kernel", ["plain", "batched"])
@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_tiny_against_reference(name, kernel, arith):
    g = golden_json("full_" + name)
    ctx = ctx_for(name)
    r, macro, idx = run(ctx, g["lookups"], kernel=kernel, arith=arith)
    assert r.verification == g["verification"]
    assert sha(idx) == g["sha256_max_idx"]
    if arith == "exact":
        assert sha(macro) == g["sha256_macro_xs"]
    else:
        with oracle.Problem(oracle_config(name)) as o:
            ref = o.run_event(want_macro=True)["macro"]
        assert rel_err(macro, ref) <= REL_TOL


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide"])
@pytest.mark.parametrize("lanes", ["1", "2", "4"])
@pytest.mark.parametrize("table", ["1", "0"])
def test_fuel_lane_split(monkeypatch, name, lanes, table):
    """The plain and batched kernels with the fuel nuclides split over 1, 2 or
    4 lanes per lookup (FAST arithmetic; the partial sums are added in a fixed
    tree), with and without the union table (unionized grid): the same argmax
    vector and hash as the reference, macro_xs within REL_TOL, and
    bit-identical results run to run."""
    monkeypatch.setenv("XSGB_FUEL_LANES", lanes)
    monkeypatch.setenv("XSGB_BATCHED_FUEL_LANES", lanes)
    monkeypatch.setenv("XSGB_UNION_TABLE", table)
    g = golden_json("full_" + name)
    inp = product_inputs(name)
    with oracle.Problem(oracle_config(name)) as o:
        ref = o.run_event(want_macro=True)["macro"]
    with X.grid_init(inp) as prob, X.Context(inp, prob) as ctx:
        assert (ctx.union_table_bytes > 0) == (table == "1" and name == "tiny_unionized")
        for kernel in ("plain", "batched"):
            r, macro, idx = run(ctx, g["lookups"], kernel=kernel, arith="fast")
            r2, macro2, _ = run(ctx, g["lookups"], kernel=kernel, arith="fast")
            assert r.verification == g["verification"] == r2.verification, kernel
            assert sha(idx) == g["sha256_max_idx"], kernel
            assert np.array_equal(macro, macro2), kernel
            assert rel_err(macro, ref) <= REL_TOL, kernel


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide"])
def test_staged_material_rows(monkeypatch, name):
    """The plain kernel reading the materials' nuclide lists and concentrations
    from shared memory (staged by each block) or through the read-only cache:
    bit-identical macro_xs either way and the reference's hash, with the
    overflow pass (200,000 lookups) and without it (4,096 lookups)."""
    g = golden_json("full_" + name)
    got = {}
    for stage in ("0", "1"):
        monkeypatch.setenv("XSGB_STAGE_ROWS", stage)
        for n in (g["lookups"], 4096):
            inp = product_inputs(name, lookups=n)
            with X.grid_init(inp) as prob, X.Context(inp, prob) as ctx:
                for arith in ("fast", "exact"):
                    r, macro, _ = run(ctx, n, kernel="plain", arith=arith)
                    if n == g["lookups"]:
                        assert r.verification == g["verification"], (stage, arith)
                    got[stage, arith, n] = (r.verification, macro)
    for key in [k[1:] for k in got if k[0] == "0"]:
        v0, m0 = got[("0",) + key]
        v1, m1 = got[("1",) + key]
        assert v0 == v1 and np.array_equal(m0, m1), key


@pytest.mark.parametrize("name", ["small_unionized", "small_hash", "small_nuclide",
                                  "large_unionized", "large_hash", "large_nuclide"])
def test_full_size_against_reference(name):
    g = golden_json("full_" + name)
    gl = golden_npz("lookups_" + name)
    ctx = ctx_for(name)
    n = g["lookups"]
    r_exact, m_exact, i_exact = run(ctx, n, kernel="plain", arith="exact")
    assert r_exact.verification == g["verification"]
    assert r_exact.hash == g["hash"]
    assert sha(i_exact) == g["sha256_max_idx"]
    assert sha(m_exact) == g["sha256_macro_xs"]
    assert np.array_equal(m_exact[gl["index"]], gl["macro_xs"])
    for kernel in ("plain", "batched"):
        r, m, i = run(ctx, n, kernel=kernel, arith="fast")
        assert r.verification == g["verification"], kernel
        assert sha(i) == g["sha256_max_idx"], kernel
        assert rel_err(m, m_exact) <= REL_TOL, kernel
        del m
    r, _, i = run(ctx, n, kernel="batched", arith="exact")
    assert r.verification == g["verification"]


@pytest.mark.parametrize("name", ["xl_hash", "xl_nuclide"])
def test_xl_against_reference(name):
    """XL (355 x 238,847 points, 100M lookups).  The reference has no XL
    constant (io.c:85-106); the digests come from its own build.  The nuclide
    grid gives the same interval as the hash grid for every lookup, so both
    are held to the hash-grid digests: EXACT bit for bit, FAST by the argmax
    digest and 1e-12 of the EXACT macro_xs."""
    import torch
    g = golden_json("full_xl_hash")
    gl = golden_npz("lookups_xl_hash")
    ctx = ctx_for(name)
    n = g["lookups"]
    r, m, i = run(ctx, n, kernel="batched", arith="exact")
    assert r.verification == g["verification"] and r.hash == 156835
    assert sha(i) == g["sha256_max_idx"]
    assert sha(m) == g["sha256_macro_xs"]
    assert np.array_equal(m[gl["index"]], gl["macro_xs"])
    # FAST, both kernels: the whole argmax vector against the reference's
    # digest, and every lookup's macro_xs vector within 1e-12 (max norm) of
    # the EXACT (reference-identical) run, compared on the device
    m_exact = torch.from_numpy(m).cuda()
    del m
    den = m_exact.abs().amax(dim=1).clamp_min(1e-300)
    for kernel in ("plain", "batched"):
        md = torch.empty((n, 5), dtype=torch.float64, device="cuda")
        idd = torch.empty(n, dtype=torch.uint8, device="cuda")
        r = ctx.run_event(kernel=kernel, arith="fast", macro_out=md, max_idx_out=idd)
        assert r.verification == g["verification"], kernel
        assert sha(idd.cpu().numpy()) == g["sha256_max_idx"], kernel
        err = float(((md - m_exact).abs().amax(dim=1) / den).max())
        assert err <= REL_TOL, (kernel, err)
        del md, idd


def test_verification_only_runs_match():
    g = golden_json("full_tiny_hash")
    ctx = ctx_for("tiny_hash")
    for kernel in ("plain", "batched"):
        for tile, buckets in ((256, 1), (1024, 256), (4096, 65536)):
            r = ctx.run_event(kernel=kernel, tile=tile, buckets=buckets)
            assert r.verification == g["verification"], (kernel, tile, buckets)
            assert r.kernel_launches >= 1


def test_shards_add_up():
    g = golden_json("full_tiny_unionized")
    ctx = ctx_for("tiny_unionized")
    n = g["lookups"]
    cuts = [0, 1, 777, 65536, 131071, n]
    total = 0
    parts = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        r, _, idx = run(ctx, b - a, first=a, count=b - a, kernel="plain", arith="exact")
        total += r.verification
        parts.append(idx)
    assert total == g["verification"]
    assert sha(np.concatenate(parts)) == g["sha256_max_idx"]


@pytest.mark.parametrize("kernel", ["plain", "batched"])
def test_caller_samples_host_and_device(kernel):
    import torch
    name = "tiny_nuclide"
    g = golden_json("full_" + name)
    ctx = ctx_for(name)
    with oracle.Problem(oracle_config(name)) as o:
        s = o.run_event(want_samples=True, want_macro=True)
    E, M = s["energy"], s["mat"]
    n = E.shape[0]
    macro = np.empty((n, 5))
    idx = np.empty(n, np.uint8)
    r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel=kernel, arith="exact")
    assert r.verification == g["verification"]
    assert sha(macro) == g["sha256_macro_xs"]
    dE = torch.from_numpy(E).cuda()
    dM = torch.from_numpy(M).cuda()
    dmacro = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    didx = torch.empty(n, dtype=torch.uint8, device="cuda")
    r2 = ctx.lookup_samples(dE, dM, macro_out=dmacro, max_idx_out=didx, kernel=kernel,
                            arith="exact")
    torch.cuda.synchronize()
    assert r2.verification == g["verification"]
    assert sha(dmacro.cpu().numpy()) == g["sha256_macro_xs"]
    assert sha(didx.cpu().numpy()) == g["sha256_max_idx"]


@pytest.mark.parametrize("name", ["small_unionized", "small_hash", "large_unionized"])
def test_host_sample_pipeline_full_size(name):
    """The host-sample pipeline over the whole 17,000,000-lookup batch (13
    chunks on four streams, the plain kernel's overflow passes on a fifth;
    the large problem is the bench's end-to-end configuration):
    the reference's hash and argmax digest in both arithmetics, EXACT macro_xs
    bit for bit, FAST bit-identical to the device-resident plain run (the
    overflow pass repeats the tiles' arithmetic lookup for lookup), and the
    batched kernel's chunks by the same digests."""
    import torch
    g = golden_json("full_" + name)
    ctx = ctx_for(name)
    n = g["lookups"]
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    E, M = pin((n,), torch.float64), pin((n,), torch.int32)
    ctx.sample_event(0, n, E, M)
    macro, idx = pin((n, 5), torch.float64), pin((n,), torch.uint8)
    r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel="plain", arith="exact")
    assert r.hash == g["hash"] and r.verification == g["verification"]
    assert sha(idx) == g["sha256_max_idx"]
    assert sha(macro) == g["sha256_macro_xs"]
    _, m_dev, _ = run(ctx, n, kernel="plain", arith="fast")
    r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel="plain", arith="fast")
    assert r.verification == g["verification"]
    assert sha(idx) == g["sha256_max_idx"]
    assert np.array_equal(macro, m_dev)
    del m_dev
    r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel="batched", arith="fast")
    assert r.verification == g["verification"]
    assert sha(idx) == g["sha256_max_idx"]


@pytest.mark.parametrize("n", [1, 31, 262145, 2097153, 5767169, 11534337])
def test_host_pipeline_chunk_edges(n):
    """The host-sample pipeline at batch sizes around its chunk schedule
    (whole chunks of 2^21 lookups plain, 2^22 batched; ramps of 1/8, 1/4, 1/2
    chunk at both ends above 2.75 chunks): one lookup, under one warp, a ramp
    chunk plus one, a plain chunk plus one, the plain ramp with ragged middle
    chunks, and the batched ramp.  Against the same samples
    from device arrays (one launch): EXACT bit for bit, the batched kernel bit
    for bit in both arithmetics, the plain kernel's FAST within REL_TOL (a short
    device-resident batch runs a material's partial warp of lookups split over
    lanes, the pipeline's chunks send it to the overflow pass), the argmax
    vector and the verification sum identical."""
    import torch
    ctx = ctx_for("tiny_hash")
    E, M = np.empty(n), np.empty(n, np.int32)
    ctx.sample_event(0, n, E, M)
    dE, dM = torch.from_numpy(E).cuda(), torch.from_numpy(M).cuda()
    for kernel in ("plain", "batched"):
        for arith in ("exact", "fast"):
            dmacro = torch.empty((n, 5), dtype=torch.float64, device="cuda")
            didx = torch.empty(n, dtype=torch.uint8, device="cuda")
            rd = ctx.lookup_samples(dE, dM, macro_out=dmacro, max_idx_out=didx, kernel=kernel,
                                    arith=arith)
            macro, idx = np.empty((n, 5)), np.empty(n, np.uint8)
            rh = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel=kernel,
                                    arith=arith)
            key = (kernel, arith)
            assert rh.verification == rd.verification, key
            assert np.array_equal(idx, didx.cpu().numpy()), key
            if kernel == "plain" and arith == "fast":
                assert rel_err(macro, dmacro.cpu().numpy()) <= REL_TOL, key
            else:
                assert np.array_equal(macro, dmacro.cpu().numpy()), key


def test_async_runs_then_sync():
    import torch
    g = golden_json("full_tiny_hash")
    ctx = ctx_for("tiny_hash")
    n = g["lookups"]
    out = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(3):
        ctx.run_event(macro_out=out, async_=True, stream=s, arith="exact")
    r = ctx.sync()
    assert r.verification == g["verification"]
    torch.cuda.synchronize()
    assert sha(out.cpu().numpy()) == g["sha256_macro_xs"]


def test_history_small_particles():
    g = golden_json("history_small")
    inp = X.make_inputs(size="small", grid="unionized", method="history", lookups=34,
                        particles=2000)
    with X.grid_init(inp) as p, X.Context(inp, p) as ctx:
        for kernel in ("plain", "batched"):
            for arith in ("exact", "fast"):
                r = ctx.run_history(kernel=kernel, arith=arith)
                assert r.verification == g["particles_2000_verification"], (kernel, arith)
        # a range of particles, stepped, adds up with the rest
        a = ctx.run_history(kernel="batched", first=0, count=777).verification
        b = ctx.run_history(kernel="batched", first=777, count=2000 - 777).verification
        assert a + b == g["particles_2000_verification"]


@pytest.mark.parametrize("size", ["small", "large"])
def test_history_full_published_hash(size):
    """History-based mode at the reference's default size (500,000 particles x
    34 lookups): the published hashes 941535 / 954318 (io.c:94-95)."""
    g = golden_json("history_" + size)
    inp = X.make_inputs(size=size, grid="unionized", method="history")
    assert inp.particles == g["particles"] and inp.lookups == g["lookups"]
    with X.grid_init(inp) as p, X.Context(inp, p) as ctx:
        for kernel in ("plain", "batched"):
            for arith in ("fast", "exact"):
                r = ctx.run_history(kernel=kernel, arith=arith)
                assert r.verification == g["verification"], (kernel, arith)
                assert r.verification % 999983 == g["hash"]


def test_c_driver_dataset_file_round_trip(tmp_path):
    """The C host program writes the problem to XS_data.dat (-b write) and a
    second run reads it back (-b read) instead of building it (Main.c:50-58);
    both report the published hash, and the file is the reference's own
    binary_write output for the problem (masked digest from the reference
    build, io.c:456-474)."""
    import subprocess
    from xsbench_gb300 import build as B
    args = ["-m", "event", "-s", "small", "-G", "unionized"]
    for mode in ("write", "read"):
        out = subprocess.run([B.EXE_PATH, *args, "-b", mode], cwd=str(tmp_path),
                             capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "945990" in out.stdout, mode
    rec = golden_json("datafile")["small_unionized"]
    assert oracle.datafile_digest(str(tmp_path / "XS_data.dat")) == (rec["bytes"],
                                                                      rec["sha256_masked"])


@pytest.mark.parametrize("method,expect", [("event", 945990), ("history", 941535)])
@pytest.mark.parametrize("grid", ["unionized", "nuclide", "hash"])
@pytest.mark.parametrize("kid", ["0", "1", "2", "3"])
def test_c_driver_reports_the_published_hash(method, expect, grid, kid):
    """The reference's CI matrix (.travis.yml:21-28: history / event x the three
    grid types, small problem) through the C host program (the reference's main
    over the C ABI), for every kernel id: exit status 0 and the published
    verification value (io.c:89-95)."""
    args = ["-m", method, "-s", "small", "-G", grid, "-k", kid]
    import subprocess
    from xsbench_gb300 import build as B
    out = subprocess.run([B.EXE_PATH, *args], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert str(expect) in out.stdout


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_nuclide", "tiny_hash"])
@pytest.mark.parametrize("kernel", ["plain", "batched"])
@pytest.mark.parametrize("arith", ["fast", "exact"])
def test_edge_energies_against_oracle(name, kernel, arith):
    """Caller samples at the edges the searches must get right: zero and
    subnormal energies, energies equal to gridpoints, the hash grid's bin
    edges and the doubles just below them, 1 - 2^-53; on the unionized and
    nuclide grids also energies outside [0, 1) and NaN (on the hash grid the
    reference indexes outside its table for those, Simulation.c:350).  The
    argmax vector and the verification sum bit-exact; macro_xs bit-identical
    (EXACT) or within REL_TOL (FAST), NaN where the reference gives NaN."""
    rng = np.random.default_rng(11)
    with oracle.Problem(oracle_config(name)) as o:
        grid = np.array(o.arrays()["nuclide_grid"]).reshape(-1, 6)[:, 0]
        edges = np.arange(500) / 500.0
        E = [np.array([0.0, 5e-324, 1e-300, 1.0 - 2.0 ** -53]),
             grid[rng.integers(0, grid.size, 3000)],
             edges, np.nextafter(edges[1:], 0.0),
             rng.random(2000)]
        if name != "tiny_hash":
            E.append(np.array([1.0, 1.5, -0.25, 1e10, -1e10, np.nan, np.inf]))
        E = np.concatenate(E)
        M = rng.integers(0, 12, E.size).astype(np.int32)
        ref = o.run_samples(E, M)
    ctx = ctx_for(name)
    macro = np.empty((E.size, 5))
    idx = np.empty(E.size, np.uint8)
    r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=idx, kernel=kernel, arith=arith)
    assert r.verification == ref["verification"]
    assert np.array_equal(idx, ref["max_idx"])
    fin = np.isfinite(ref["macro"])
    assert np.array_equal(np.isfinite(macro), fin)
    assert np.array_equal(macro[~fin], ref["macro"][~fin], equal_nan=True)   # same inf / NaN
    if arith == "exact":
        assert np.array_equal(macro[fin], ref["macro"][fin])
    else:
        rows = fin.all(axis=1)
        assert rel_err(macro[rows], ref["macro"][rows]) <= REL_TOL


_EDGE_CACHE = {}


def edge_samples(name):
    """Edge energies of the hash / nuclide problem (as above, without the
    out-of-range ones on the hash grid) and the oracle's results for them."""
    if name not in _EDGE_CACHE:
        rng = np.random.default_rng(23)
        with oracle.Problem(oracle_config(name)) as o:
            grid = np.array(o.arrays()["nuclide_grid"]).reshape(-1, 6)[:, 0]
            edges = np.arange(500) / 500.0
            k = 2.0 ** -12   # the guide's bin edges for 1,000 points per nuclide
            gedges = np.arange(1, 4096) * k
            E = [np.array([0.0, 5e-324, 1e-300, 1.0 - 2.0 ** -53]),
                 grid[rng.integers(0, grid.size, 3000)], edges, np.nextafter(edges[1:], 0.0),
                 gedges[rng.integers(0, gedges.size, 500)],
                 np.nextafter(gedges[rng.integers(0, gedges.size, 500)], 0.0), rng.random(2000)]
            if name != "tiny_hash":
                E.append(np.array([1.0, 1.5, -0.25, 1e10, -1e10, np.nan, np.inf]))
            E = np.concatenate(E)
            M = rng.integers(0, 12, E.size).astype(np.int32)
            _EDGE_CACHE[name] = (E, M, o.run_samples(E, M))
    return _EDGE_CACHE[name]


GUIDED_VARIANTS = [
    {"XSGB_GUIDE": "1"},
    {"XSGB_GUIDE": "1", "XSGB_GUIDE_LOG2": "6"},
    {"XSGB_GUIDE": "1", "XSGB_BIN_RECORDS": "0"},
    {"XSGB_GUIDE": "1", "XSGB_BIN_RECORDS": "0", "XSGB_GUIDE_LOG2": "6"},
    {"XSGB_GUIDE": "1", "XSGB_TILE_SORT": "0", "XSGB_OVERFLOW": "0", "XSGB_BIN_PREFETCH": "0"},
    {"XSGB_GUIDE": "1", "XSGB_OVERFLOW": "1", "XSGB_BIN_PREFETCH": "4", "XSGB_FUEL_LANES": "4"},
    {"XSGB_GUIDE": "0", "XSGB_TILE_SORT": "1"},
]


@pytest.mark.parametrize("name", ["tiny_hash", "tiny_nuclide"])
@pytest.mark.parametrize("variant", range(len(GUIDED_VARIANTS)))
def test_guided_search_variants(monkeypatch, name, variant):
    """The plain kernel's interval searches in every configuration the
    switches select -- the guide with and without bin records, with 64 bins
    per nuclide (about 16 gridpoints per bin, so most lookups take the walk
    past the bin's first interval), the in-tile energy order and the overflow
    pass on and off, prefetch distances, lanes per fuel lookup, the grids'
    own searches -- on the hash and nuclide grids: the event batch's
    verification sum and argmax vector against the reference's digests, and
    the edge energies (gridpoints, hash-bin and guide-bin edges, zero,
    subnormals) against the oracle, in both arithmetics."""
    for k, v in GUIDED_VARIANTS[variant].items():
        monkeypatch.setenv(k, v)
    g = golden_json("full_" + name)
    E, M, ref = edge_samples(name)
    inp = product_inputs(name)
    with X.grid_init(inp) as prob, X.Context(inp, prob) as ctx:
        for arith in ("fast", "exact"):
            r, _, idx = run(ctx, g["lookups"], kernel="plain", arith=arith)
            assert r.verification == g["verification"], arith
            assert sha(idx) == g["sha256_max_idx"], arith
            macro = np.empty((E.size, 5))
            mi = np.empty(E.size, np.uint8)
            r = ctx.lookup_samples(E, M, macro_out=macro, max_idx_out=mi, kernel="plain", arith=arith)
            assert r.verification == ref["verification"], arith
            assert np.array_equal(mi, ref["max_idx"]), arith
            fin = np.isfinite(ref["macro"])
            assert np.array_equal(macro[~fin], ref["macro"][~fin], equal_nan=True)
            if arith == "exact":
                assert np.array_equal(macro[fin], ref["macro"][fin])
            else:
                rows = fin.all(axis=1)
                assert rel_err(macro[rows], ref["macro"][rows]) <= REL_TOL
        # checked runs (every table index bounds-checked) and the batched kernel
        for kernel in ("plain", "batched"):
            assert ctx.run_event(kernel=kernel, checked=True).verification == g["verification"]
            assert ctx.run_event(kernel=kernel).verification == g["verification"]


def test_drop_in_seam():
    g = golden_json("full_tiny_unionized")
    inp = product_inputs("tiny_unionized")
    with X.grid_init(inp) as p:
        assert X.run_event_based_simulation(inp, p) == g["verification"]


def test_bad_material_sample_is_reported():
    ctx = ctx_for("tiny_hash")
    E = np.full(1000, 0.5)
    M = np.zeros(1000, np.int32)
    M[517] = 12
    for kernel in ("plain", "batched"):
        with pytest.raises(X.XSError) as e:
            ctx.lookup_samples(E, M, kernel=kernel)
        assert e.value.status == 6
    # the context stays usable
    assert ctx.lookup_samples(E, np.zeros(1000, np.int32)).verification > 0


def test_corrupt_index_grid_is_rejected():
    inp = product_inputs("tiny_hash")
    with X.grid_init(inp) as p:
        p.sd.index_grid[12345] = 999999          # beyond the nuclide grid
        with pytest.raises(X.XSError) as e:
            X.Context(inp, p)
        assert e.value.status == 6
        p.sd.mats[3] = 68                        # nuclide id beyond n_isotopes
        p.sd.index_grid[12345] = 0
        with pytest.raises(X.XSError) as e:
            X.Context(inp, p)
        assert e.value.status == 6


def test_checked_runs_pass_on_valid_tables():
    for name in ("tiny_unionized", "tiny_hash", "tiny_nuclide"):
        g = golden_json("full_" + name)
        ctx = ctx_for(name)
        for kernel in ("plain", "batched"):
            assert ctx.run_event(kernel=kernel, checked=True).verification == g["verification"]
