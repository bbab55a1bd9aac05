"""bench.py's host-side logic, on the CPU: the material probabilities and
algorithmic bytes behind its roofline figures, the clock sampler's parsing
and timed-region filter, the profile summaries its side measurements read,
and the reference arm's JSON line (the reference's CPU path on a small
workload)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import xsbench_gb300 as X
from conftest import ROOT, oracle_config

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_material_probabilities_match_sampled_materials():
    """P(material) of pick_mat (Simulation.c:447-459) against the materials of
    200,000 sampled lookups of the oracle (3-sigma binomial bounds)."""
    p = bench.material_probabilities()
    assert abs(sum(p) - 1.0) < 1e-12
    with oracle.Problem(oracle_config("tiny_unionized")) as o:
        r = o.run_event(want_samples=True)
    counts = np.bincount(r["mat"], minlength=12)
    n = counts.sum()
    for m in range(12):
        sd = np.sqrt(n * p[m] * (1 - p[m]))
        assert abs(counts[m] - n * p[m]) <= 4 * sd + 1, (m, counts[m], n * p[m])


@pytest.mark.parametrize("size,grid,expect", [("large", "unionized", 5714.3),
                                              ("large", "hash", 7532.1),
                                              ("large", "nuclide", 11520.0),
                                              ("XL", "hash", 8861.3),
                                              ("XL", "nuclide", 13291.9)])
def test_algorithmic_bytes(size, grid, expect):
    """The algorithmic bytes per lookup of the reference's searches that the
    roofline fractions divide by (8 per search probe, 4 or 8 per index entry,
    16 for the hash bracket energies, 96 per gridpoint pair)."""
    inp = X.make_inputs(size=size, grid=grid, method="event")
    nn = [34 if inp.n_isotopes == 68 else 321, 5, 4, 4, 27, 21, 21, 21, 21, 21, 9, 9]
    assert abs(bench.algorithmic_bytes_per_lookup(inp, nn) - expect) < 0.5


def test_clock_sampler_keeps_the_timed_region(tmp_path):
    """Samples stamped inside [mark_begin, mark_end] are the ones reported;
    throttle reasons are collected from them."""
    import datetime
    c = bench.ClockSampler(0)
    base = datetime.datetime(2026, 12, 4, 12, 0, 0)
    rows = []
    for i, (mhz, thermal) in enumerate([(1500, "Not Active"), (2070, "Not Active"),
                                        (2070, "Active"), (2070, "Not Active"),
                                        (900, "Not Active")]):
        ts = (base + datetime.timedelta(seconds=i)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        rows.append(f"{ts}, 0, {mhz}, 2070, 500.0, 0x0, Not Active, {thermal}, Not Active, Not Active")
    f = tmp_path / "clk.csv"
    f.write_text("\n".join(rows) + "\n")

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    c.proc = Done()
    c.f = open(f, "r+")
    c.t0 = (base + datetime.timedelta(seconds=1)).timestamp()
    c.t1 = (base + datetime.timedelta(seconds=3)).timestamp()
    r = c.stop()
    assert r["samples"] == 3 and r["in_timed_region"]
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070
    assert r["reasons"] == ["hw_thermal_slowdown"]


@pytest.mark.parametrize("kernel,workload", [("k_plain", "large_unionized"),
                                             ("k_plain", "large_hash"),
                                             ("k_plain", "xl_hash"),
                                             ("k_plain", "xl_nuclide"),
                                             ("k_plain", "large_nuclide"),
                                             ("k_batched_lookup", "large_hash"),
                                             ("k_batched_lookup", "large_nuclide"),
                                             ("k_batched_lookup", "xl_hash"),
                                             ("k_batched_lookup", "xl_nuclide"),
                                             ("k_batched_lookup", "large_unionized_records")])
def test_profiles_the_bench_reads(kernel, workload):
    """Every DRAM figure the bench line quotes comes from a committed ncu
    summary that states its command."""
    v, src = bench.profiled_dram(kernel, workload)
    assert v and v > 0 and src.startswith("profiles/")
    text = open(os.path.join(ROOT, src)).read()
    assert "ncu " in text and "--clock-control none" in text


def test_reference_arm_line():
    """--impl reference on the small unionized problem: one JSON line with the
    contract's keys, the reference's CPU path timed on this host's cores."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "small_unionized", "--steps", "1", "--warmup", "1"],
                         capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "lookups/s"
    assert d["cpu_baseline"]["kind"] in ("reference", "port")
    assert d["cpu_baseline"]["k1"]["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
