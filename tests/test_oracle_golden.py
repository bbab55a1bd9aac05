"""The oracle (oracle/xs_oracle.c) against the reference's own outputs.

These pin the checker before it is trusted: published hashes
(openmp-threading/io.c:89-95), and per-lookup values, full-run argmax and
macro_xs digests and setup-array digests dumped from the reference built from
source (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

import oracle
from conftest import golden_json, golden_npz, oracle_config, sha


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide"])
def test_oracle_full_digest_tiny(name):
    g = golden_json("full_" + name)
    with oracle.Problem(oracle_config(name)) as p:
        r = p.run_event(want_macro=True)
    assert r["verification"] == g["verification"]
    assert sha(r["max_idx"]) == g["sha256_max_idx"]
    assert sha(r["macro"]) == g["sha256_macro_xs"]   # bit-identical to the reference


def test_oracle_small_unionized_full_17m():
    g = golden_json("full_small_unionized")
    with oracle.Problem(oracle_config("small_unionized")) as p:
        r = p.run_event(want_macro=True)
    assert r["verification"] % oracle.HASH_MODULUS == oracle.HASH_SMALL_EVENT == g["hash"]
    assert sha(r["max_idx"]) == g["sha256_max_idx"]
    assert sha(r["macro"]) == g["sha256_macro_xs"]


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide",
                                  "small_unionized", "small_hash", "small_nuclide",
                                  "large_hash", "large_nuclide", "large_unionized"])
def test_oracle_setup_and_sampled_lookups(name):
    gs = golden_json("setup_" + name)
    gl = golden_npz("lookups_" + name)
    with oracle.Problem(oracle_config(name)) as p:
        arrs = p.arrays()
        for k, v in arrs.items():
            assert sha(v) == gs["sha256"][k], k
        for i, e, m, mx, mi in zip(gl["index"], gl["energy"], gl["mat"], gl["macro_xs"],
                                   gl["max_idx"]):
            r = p.run_event(first=int(i), n=1, nthreads=1, want_macro=True, want_samples=True)
            assert r["energy"][0] == e and r["mat"][0] == m
            assert np.array_equal(r["macro"][0], mx)
            assert r["max_idx"][0] == mi


def test_oracle_history_small():
    g = golden_json("history_small")
    cfg = oracle.Config(size="small", grid="unionized", method="history", lookups=34,
                        particles=2000)
    with oracle.Problem(cfg) as p:
        assert p.run_history() == g["particles_2000_verification"]
    assert g["hash"] == oracle.HASH_SMALL_HISTORY


def test_published_hashes_in_fixtures():
    assert golden_json("full_small_unionized")["hash"] == oracle.HASH_SMALL_EVENT
    assert golden_json("full_large_unionized")["hash"] == oracle.HASH_LARGE_EVENT
    assert golden_json("history_large")["hash"] == oracle.HASH_LARGE_HISTORY
    for g in ("hash", "nuclide"):
        assert golden_json(f"full_large_{g}")["hash"] == oracle.HASH_LARGE_EVENT
        assert golden_json(f"full_small_{g}")["hash"] == oracle.HASH_SMALL_EVENT


def test_oracle_planted_mistake_is_caught():
    """A change of one concentration in the oracle's tables changes the digest:
    the digest comparison above is sensitive to single-value errors."""
    g = golden_json("full_tiny_unionized")
    with oracle.Problem(oracle_config("tiny_unionized")) as p:
        p.sd.concs[0] = p.sd.concs[0] * (1 + 1e-15) + 1e-16
        r = p.run_event(n=20000, want_macro=True)
    ref = golden_npz("lookups_tiny_unionized")
    # the planted error shows in macro_xs of fuel lookups
    sel = ref["index"] < 20000
    diff = [not np.array_equal(r["macro"][i], mx)
            for i, mx, m in zip(ref["index"][sel], ref["macro_xs"][sel], ref["mat"][sel]) if m == 0]
    assert any(diff)
    assert g["lookups"] == 200000


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide", "small_hash"])
def test_oracle_optimisation_1_port(name):
    """The port of the reference's optimisation 1 (Simulation.c:698-871:
    sampling split from the lookups, sorts by material and energy) gives the
    reference's verification sum, on every grid; where the reference build is
    present, its own optimisation 1 gives the same sum."""
    import ctypes as C
    import os
    g = golden_json("full_" + name)
    cfg = oracle_config(name)
    with oracle.Problem(cfg) as p:
        L = oracle.lib()
        ph = (C.c_double * 4)()
        v = L.or_run_event_k1(C.byref(p.inp), C.byref(p.sd), 0, g["lookups"], 4, ph)
        assert v == g["verification"]
        assert ph[3] > 0
        if os.path.exists(oracle.REF_LIB_PATH) and name.startswith("tiny"):
            ref = C.CDLL(oracle.REF_LIB_PATH)
            ref.refh_event_k1.restype = C.c_ulonglong
            ref.refh_event_k1.argtypes = [C.POINTER(oracle.Inputs), C.POINTER(oracle.SimData)]
            inp = cfg.inputs()
            inp.lookups = g["lookups"]
            assert ref.refh_event_k1(C.byref(inp), C.byref(p.sd)) == g["verification"]
