#!/usr/bin/env python3
"""Benchmark of the event-based macroscopic cross-section lookup on GB300.

One step = one pass of the lookup over the whole event batch of the workload
(default: the large problem on the unionized grid, 17,000,000 lookups, the
plain kernel).  Prints one JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                    [--kernel plain|batched] [--arith fast|exact]
    python bench.py --impl reference ...   # the reference's CPU path on the host cores

Timing: W untimed steps, then K steps bracketed by a barrier and
cudaStreamSynchronize, timed with CUDA events on the stream the kernels run
on; the tables (5.7 GB index grid) are larger than L2, so no flush is needed.
Multi-GPU: one process per GPU; rank r takes event indices
[r*N, (r+1)*N) (weak scaling, no data-path collective); value = all ranks'
lookups / max over ranks of the timed span.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "lookups/s device-timed, large unionized; batched & fwd+adjoint vs plain, FP64"
UNIT = "lookups/s"

WORKLOADS = {
    "large_unionized": dict(size="large", grid="unionized"),
    "large_hash": dict(size="large", grid="hash"),
    "large_nuclide": dict(size="large", grid="nuclide"),
    "small_unionized": dict(size="small", grid="unionized"),
    "small_hash": dict(size="small", grid="hash"),
    "small_nuclide": dict(size="small", grid="nuclide"),
    "xl_hash": dict(size="XL", grid="hash", lookups=100000000),
    "xl_nuclide": dict(size="XL", grid="nuclide", lookups=100000000),
}
# openmp-threading/Simulation.c:433-445
DIST = [0.140, 0.052, 0.275, 0.134, 0.154, 0.064, 0.066, 0.055, 0.008, 0.015, 0.025, 0.013]


def material_probabilities():
    """P(material) of pick_mat (Simulation.c:447-459): cumulative sums skip dist[0]."""
    run = [sum(DIST[j] for j in range(i, 0, -1)) for i in range(12)]
    p = [0.0] * 12
    prev = 0.0
    for i in range(1, 12):
        p[i] = run[i] - prev
        prev = run[i]
    p[0] = 1.0 - prev
    return p


def algorithmic_bytes_per_lookup(inputs, num_nucs) -> float:
    """Bytes one lookup must move from the tables (the reference algorithm):
    union search 8 B per probe, then per nuclide its index entry and the
    96-byte pair of bracketing gridpoints (hash: the two bracket energies and
    the in-bin search; nuclide: the full per-nuclide search)."""
    nbar = sum(p * n for p, n in zip(material_probabilities(), num_nucs))
    n_gp = inputs.n_gridpoints
    if inputs.grid_type == 0:
        n_union = inputs.n_isotopes * n_gp
        return 8 * math.ceil(math.log2(n_union)) + nbar * (4 + 96)
    if inputs.grid_type == 2:
        probes = math.ceil(math.log2(n_gp / inputs.hash_bins + 2))
        return nbar * (8 + 16 + 8 * probes + 96)
    return nbar * (8 * math.ceil(math.log2(n_gp)) + 96)


def nbar_of(inputs, problem) -> float:
    """Expected nuclides per lookup (material probabilities x list lengths)."""
    nn = list(problem.arrays()["num_nucs"])
    return sum(p * n for p, n in zip(material_probabilities(), nn))


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(workload, kernel):
    """DRAM read+write bytes per lookup of one step of the path (for the plain
    path: the tiled kernel plus its overflow pass), from the ncu summary
    committed under profiles/ (line 'dram_bytes_per_lookup: X')."""
    name = os.path.join(ROOT, "profiles", f"{'k_plain' if kernel == 'plain' else 'k_batched_lookup'}_{workload}.md")
    try:
        for line in open(name):
            if line.strip().startswith("dram_bytes_per_lookup:"):
                return float(line.split(":", 1)[1].split()[0]), os.path.relpath(name, ROOT)
    except OSError:
        pass
    return None, None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from
    start() (before the end of the warm-up, so that the sampler is running
    when the timed region begins) to stop(); only the samples stamped inside
    the timed region [mark_begin(), mark_end()] are reported (all of them if
    none is)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.f = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def mark_begin(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    @staticmethod
    def _stamp(text):
        import datetime
        try:
            return datetime.datetime.strptime(text.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        samples = []
        for r in rows:
            try:
                samples.append((self._stamp(r[0]), float(r[2]), float(r[3]),
                                {n for n, v in zip(names, r[6:10]) if v.strip().lower() == "active"}))
            except (ValueError, IndexError):
                continue
        inside = [x for x in samples if x[0] is not None and self.t0 is not None
                  and self.t1 is not None and self.t0 - 0.05 <= x[0] <= self.t1 + 0.05]
        used = inside or samples
        if not used:
            return None
        return {"sm_mhz": statistics.median(x[1] for x in used),
                "sm_max_mhz": max(x[2] for x in used), "samples": len(used),
                "in_timed_region": bool(inside),
                "reasons": sorted(set().union(*(x[3] for x in used)))}


def cpu_k1(L, inp, sd, lookups, cores, budget_s):
    """The port of the reference's optimisation 1 (Simulation.c:698-871:
    sampling, sorts by material and energy, lookups by material) over the
    first n lookups, n sized to about budget_s seconds; (rate, record)."""
    ph = (C.c_double * 4)()
    n = min(lookups, 1000000)
    t0 = time.perf_counter()
    L.or_run_event_k1(C.byref(inp), sd, 0, n, cores, ph)
    dt = time.perf_counter() - t0
    n2 = int(min(lookups, max(n, n * budget_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    L.or_run_event_k1(C.byref(inp), sd, 0, n2, cores, ph)
    dt2 = time.perf_counter() - t0
    return n2 / dt2, {"value": n2 / dt2, "unit": UNIT,
                      "sample": f"lookups [0, {n2}) sampled, sorted and looked up in one call, "
                                f"{dt2:.2f} s on {cores} threads",
                      "phases_s": {"sample": round(ph[0], 3), "sort": round(ph[1], 3),
                                   "lookup": round(ph[2], 3)}}


def cpu_baseline_oracle(inputs_x, problem, workload, budget_s=10.0):
    """The oracle port of the reference's CPU path timed on this host's cores
    over bounded samples of the same workload, reusing the (bit-identical)
    setup arrays: the event loop (k0, Simulation.c:15-114; the line's value)
    and optimisation 1 (k1, Simulation.c:698-871)."""
    import oracle
    L = oracle.lib()
    oin = oracle.Inputs()
    C.memmove(C.byref(oin), C.byref(inputs_x), C.sizeof(oin))
    sd = C.cast(C.byref(problem.sd), C.POINTER(oracle.SimData))
    cores = os.cpu_count() or 1
    n = 200000
    t0 = time.perf_counter()
    L.or_run_event(C.byref(oin), sd, 0, n, cores, None, None, None, None)
    dt = time.perf_counter() - t0
    n2 = int(min(inputs_x.lookups, max(n, n * budget_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    L.or_run_event(C.byref(oin), sd, 0, n2, cores, None, None, None, None)
    dt2 = time.perf_counter() - t0
    k0 = {"value": n2 / dt2, "unit": UNIT,
          "sample": f"lookups [0, {n2}) of {workload} ({n2 / inputs_x.lookups:.1%} of the batch), "
                    f"{dt2:.2f} s on {cores} threads"}
    _, k1 = cpu_k1(L, oin, sd, inputs_x.lookups, cores, budget_s * 0.6)
    return {"value": k0["value"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": k0["sample"] + " (k0, the event loop)", "k0": k0, "k1": k1}


# ---------------------------------------------------------- side measurements
XL_HASH = 156835   # the reference build's XL event value (no published constant; io.c:85-106)


def expected_hash(wl):
    if wl["size"] == "XL":
        return XL_HASH if wl.get("lookups") == 100000000 else None
    return {"large": 952131, "small": 945990}.get(wl["size"])


def profiled_dram(kernel_file, workload):
    """DRAM bytes per lookup from a committed ncu summary (profiles/<kernel>_<workload>.md)."""
    name = os.path.join(ROOT, "profiles", f"{kernel_file}_{workload}.md")
    try:
        for line in open(name):
            if line.strip().startswith("dram_bytes_per_lookup:"):
                return float(line.split(":", 1)[1].split()[0]), os.path.relpath(name, ROOT)
    except OSError:
        pass
    return None, None


def time_kernel(ctx, stream, n, steps, warmup, **kw):
    """(lookups/s, ms per step, last Result) of `steps` event runs, device-timed."""
    import torch
    for _ in range(warmup):
        ctx.run_event(async_=True, stream=stream, count=n, **kw)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        ctx.run_event(async_=True, stream=stream, count=n, **kw)
    e1.record(stream)
    torch.cuda.synchronize()
    r = ctx.sync()
    t = e0.elapsed_time(e1) / 1e3
    return n * steps / t, t / steps * 1e3, r


def side_measurements(stream, steps, warmup, fp64_peak, peak_gbs):
    """The other configurations of the benchmark set on this GPU, one problem
    at a time (built on the device): the large hash grid (plain, batched,
    forward + adjoint), the XL problem on the hash and nuclide grids (plain
    and batched, 100,000,000 lookups), the large unionized grid batched
    without its union table (the sort's own gain), and the reference's own
    CUDA kernels (baseline and optimisation 6) through oracle/ref_cuda_harness."""
    import torch
    import xsbench_gb300 as X
    out = {}
    # the practical DRAM ceiling of the plain kernels' access pattern: whole
    # 128-byte lines gathered at random, a warp's 32 lanes inside one window
    # (xsbench_gb300/_lib/xsgb_gather_ceiling, 8 GB buffer, about 2 s)
    ceiling = None
    probe = os.path.join(ROOT, "xsbench_gb300", "_lib", "xsgb_gather_ceiling")
    if os.path.exists(probe):
        try:
            p = subprocess.run([probe, "33"], capture_output=True, text=True, timeout=120)
            g = json.loads(p.stdout.strip().splitlines()[-1])
            if p.returncode == 0 and "windows" in g:
                out["gather_ceiling"] = g
                ceiling = max(w["gbs"] for w in g["windows"] if w["window_bytes"] == 1 << 24)
        except (subprocess.SubprocessError, ValueError, IndexError) as e:
            out["gather_ceiling"] = {"unavailable": str(e)[:200]}

    def plain_key(wl_name, wl, ctx, inputs, nn):
        exp = expected_hash(wl)
        v, ms, r = time_kernel(ctx, stream, inputs.lookups, steps, warmup, kernel="plain")
        bpl = algorithmic_bytes_per_lookup(inputs, nn)
        nbar = sum(p * k for p, k in zip(material_probabilities(), nn))
        rec = {"value": v, "unit": UNIT, "ms_per_step": ms, "hash": r.hash,
               "hash_ok": exp is None or r.hash == exp,
               "roofline": {"bound": "hbm", "achieved": v * bpl / 1e9, "peak": peak_gbs,
                            "unit": "GB/s", "frac": v * bpl / 1e9 / peak_gbs,
                            "algorithmic_bytes_per_lookup": round(bpl, 1)},
               "fp64": {"ops_per_lookup": round(11 * nbar, 1),
                        "frac": v * 11 * nbar / fp64_peak}}
        dram, src = profiled_dram("k_plain", wl_name)
        if dram:
            rec["dram"] = {"bytes_per_lookup": dram, "achieved_gbs": v * dram / 1e9,
                           "frac": v * dram / 1e9 / peak_gbs, "source": src}
            if ceiling:
                rec["dram"]["frac_of_gather_ceiling"] = v * dram / 1e9 / ceiling
        return rec

    def batched_key(wl_name, wl, ctx, inputs, nn, ops_per_nuclide=11):
        exp = expected_hash(wl)
        v, ms, r = time_kernel(ctx, stream, inputs.lookups, steps, warmup, kernel="batched")
        nbar = sum(p * k for p, k in zip(material_probabilities(), nn))
        rec = {"value": v, "unit": UNIT, "ms_per_step": ms, "hash": r.hash,
               "hash_ok": exp is None or r.hash == exp,
               "fp64": {"ops_per_lookup": round(ops_per_nuclide * nbar, 1),
                        "frac": v * ops_per_nuclide * nbar / fp64_peak}}
        dram, src = profiled_dram("k_batched_lookup", wl_name)
        if dram:
            rec["dram"] = {"bytes_per_lookup": dram, "achieved_gbs": v * dram / 1e9,
                           "frac": v * dram / 1e9 / peak_gbs, "source": src}
        return rec

    def open_ctx(wl):
        inputs = X.make_inputs(method="event", **wl)
        ctx = X.Context(inputs)   # built on the device
        nn = [34 if inputs.n_isotopes == 68 else 321, 5, 4, 4, 27, 21, 21, 21, 21, 21, 9, 9]
        return inputs, ctx, nn

    # large hash grid: plain, batched, forward + adjoint
    wl = WORKLOADS["large_hash"]
    inputs, ctx, nn = open_ctx(wl)
    try:
        out["large_hash_plain"] = plain_key("large_hash", wl, ctx, inputs, nn)
        out["large_hash_batched"] = batched_key("large_hash", wl, ctx, inputs, nn)
        N = inputs.lookups
        g = torch.randn((N, 5), dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(1234))
        d_e = torch.empty(N, dtype=torch.float64, device="cuda")
        d_c = torch.zeros((12, 321), dtype=torch.float64, device="cuda")
        d_x = torch.zeros((inputs.n_isotopes, inputs.n_gridpoints, 5), dtype=torch.float64,
                          device="cuda")
        macro = torch.empty((N, 5), dtype=torch.float64, device="cuda")
        akw = dict(count=N, stream=stream, macro_out=macro, d_concs=d_c, d_xs=d_x, d_energy=d_e)
        for _ in range(2):
            ctx.adjoint(g, **akw)
        times = [ctx.adjoint(g, **akw) for _ in range(max(3, steps // 2))]
        t_adj = statistics.median(r.device_ms for r in times) / 1e3
        out["large_hash_forward_adjoint"] = {
            "value": N / t_adj, "unit": UNIT, "ms_per_step": t_adj * 1e3,
            "vs_forward": (N / t_adj) / out["large_hash_plain"]["value"],
            "hash_ok": times[-1].hash == 952131,
            "what": "forward macro_xs + dL/dE + dL/dconcs + dL/dxs, device arrays, N(0,1) upstream"}
        del g, d_e, d_c, d_x, macro
        # the autotuner's choice for this context (xs_autotune: grid type,
        # guided searches, kernel shapes, block size, in-tile order, on 4M of
        # its lookups), then the whole batch timed with it
        t0 = time.perf_counter()
        best = ctx.autotune()
        t_tune = time.perf_counter() - t0
        v, ms, r = time_kernel(ctx, stream, inputs.lookups, steps, warmup, kernel=best["kernel"])
        out["large_hash_autotuned"] = {"value": v, "unit": UNIT, "ms_per_step": ms,
                                       "hash_ok": r.hash == 952131, "choice": best,
                                       "tuning_s": round(t_tune, 1)}
    finally:
        ctx.close()
    # the XL problem on both grids
    for name in ("xl_hash", "xl_nuclide"):
        wl = WORKLOADS[name]
        inputs, ctx, nn = open_ctx(wl)
        try:
            out[name + "_plain"] = plain_key(name, wl, ctx, inputs, nn)
            out[name + "_batched"] = batched_key(name, wl, ctx, inputs, nn)
        finally:
            ctx.close()
    # batched on the large unionized grid without the union table
    os.environ["XSGB_UNION_TABLE"] = "0"
    try:
        wl = WORKLOADS["large_unionized"]
        inputs, ctx, nn = open_ctx(wl)
        try:
            out["large_unionized_batched_no_union_table"] = batched_key(
                "large_unionized_records", wl, ctx, inputs, nn)
            out["large_unionized_batched_no_union_table"]["union_table"] = ctx.union_table_bytes > 0
        finally:
            ctx.close()
        # history mode on the same problem (500,000 particles x 34 lookups,
        # Simulation.c:116-238): the particles stepped in lockstep as event
        # batches, and one thread per particle as the reference runs it
        hin = X.make_inputs(size="large", grid="unionized", method="history")
        ctx = X.Context(hin)
        try:
            n = hin.particles * hin.lookups
            hist = {}
            for kernel, reps in (("batched", 5), ("plain", 2)):
                ctx.run_history(kernel=kernel)
                runs = [ctx.run_history(kernel=kernel) for _ in range(reps)]
                t = statistics.median(r.device_ms for r in runs) / 1e3
                hist[kernel] = {"value": n / t, "unit": UNIT, "ms_per_run": t * 1e3,
                                "hash": runs[-1].hash, "hash_ok": runs[-1].hash == 954318}
            out["large_unionized_history"] = {
                "particles": hin.particles, "lookups_per_particle": hin.lookups,
                "stepped": hist["batched"], "per_particle": hist["plain"]}
        finally:
            ctx.close()
    finally:
        del os.environ["XSGB_UNION_TABLE"]
    out["reference_cuda"] = reference_cuda_kernels()
    return out


def reference_cuda_kernels():
    """The reference's cuda/Simulation.cu kernels (baseline, k0, and
    optimisation 6, k6) on this GPU, large unionized problem: its sm_103a
    cubin built from its sources (oracle/_ref) and launched by
    oracle/ref_cuda_harness (device time of the lookup launches)."""
    cubin = os.path.join(ROOT, "oracle", "_ref", "xsbench_cuda_sim.cubin")
    if not os.path.exists(cubin):
        return {"unavailable": "the reference's CUDA cubin (oracle/_ref) was not built for this run"}
    exe = os.path.join(ROOT, "oracle", "_build", "ref_cuda_harness")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "harness"],
                       capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(exe):
        return {"unavailable": "oracle/ref_cuda_harness did not build: " + (r.stderr or r.stdout)[-200:]}
    res = {}
    for k in (0, 6):
        r = subprocess.run([exe, "-m", "event", "-s", "large", "-G", "unionized", "-k", str(k),
                            "--reps", "3", "--cubin", cubin], capture_output=True, text=True,
                           cwd=ROOT, timeout=600)
        try:
            d = json.loads(r.stdout.strip().splitlines()[-1])
            res[f"k{k}"] = {"value": d["lookups_per_s"], "unit": UNIT, "ms": d["ms"],
                            "what": d["what"], "hash_ok": d["hash"] == 952131}
        except Exception:
            res[f"k{k}"] = {"unavailable": (r.stderr or r.stdout)[-200:]}
    return res


# ------------------------------------------------------------- reference arm
def reference_arm(args, rank):
    """The reference's own CPU implementation of the path on the host cores:
    the reference library built from its sources (oracle/_ref) where it was
    built for this machine, else the oracle port of it."""
    if rank != 0:
        return 0
    import oracle
    wl = WORKLOADS[args.workload]
    cfg = oracle.Config(size=wl["size"], grid=wl["grid"], lookups=wl.get("lookups"))
    inp = cfg.inputs()
    cores = os.cpu_count() or 1
    kind = "port"
    ref = None
    if os.path.exists(oracle.REF_LIB_PATH):
        try:
            ref = C.CDLL(oracle.REF_LIB_PATH)
            ref.refh_grid_init.restype = C.POINTER(oracle.SimData)
            ref.refh_grid_init.argtypes = [C.POINTER(oracle.Inputs)]
            ref.refh_run_event.restype = C.c_ulonglong
            ref.refh_run_event.argtypes = [C.POINTER(oracle.Inputs), C.POINTER(oracle.SimData),
                                           C.c_long, C.c_long] + [C.c_void_p] * 4
            ref.refh_set_threads.argtypes = [C.c_int]
            ref.refh_set_threads(cores)
            kind = "reference"
        except OSError:
            ref = None
    if ref is not None:
        sdp = ref.refh_grid_init(C.byref(inp))
        run = lambda a, n: ref.refh_run_event(C.byref(inp), sdp, a, n, None, None, None, None)  # noqa: E731
    else:
        prob = oracle.Problem(cfg)
        L = oracle.lib()
        run = lambda a, n: L.or_run_event(C.byref(prob.inp), C.byref(prob.sd), a, n, cores,  # noqa: E731
                                          None, None, None, None)
    # each step the whole batch when the run (warm-up + timed steps) fits in
    # about 150 s at the measured rate -- the same workload as the GPU arm's
    # step -- else a bounded sample of about 2 s of work per step
    t0 = time.perf_counter()
    run(0, 100000)
    rate0 = 100000 / (time.perf_counter() - t0)
    if inp.lookups * (args.steps + args.warmup) / rate0 <= 150.0:
        per_step = inp.lookups
    else:
        per_step = int(min(inp.lookups // max(1, args.steps), max(100000, rate0 * 2.0)))
    for s in range(args.warmup):
        run(s * per_step % max(1, inp.lookups - per_step), per_step)
    t0 = time.perf_counter()
    for s in range(args.steps):
        run((s * per_step) % max(1, inp.lookups - per_step), per_step)
    t = time.perf_counter() - t0
    value = per_step * args.steps / t
    # the reference's sorted CPU path (optimisation 1, Simulation.c:698-871),
    # reported beside the event loop; the line's value stays the event loop's
    if ref is not None:
        ref.refh_event_k1.restype = C.c_ulonglong
        ref.refh_event_k1.argtypes = [C.POINTER(oracle.Inputs), C.POINTER(oracle.SimData)]
        t0 = time.perf_counter()
        ref.refh_event_k1(C.byref(inp), sdp)
        dt = time.perf_counter() - t0
        k1 = {"value": inp.lookups / dt, "unit": UNIT,
              "sample": f"all {inp.lookups} lookups in one call, {dt:.2f} s on {cores} threads"}
    else:
        _, k1 = cpu_k1(oracle.lib(), prob.inp, C.byref(prob.sd), inp.lookups, cores, 6.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (the reference's LCG generators)",
        "config": {"workload": args.workload, "kernel": "openmp-threading event loop (k0)",
                   "sample_lookups_per_step": per_step,
                   "whole_batch_per_step": per_step == inp.lookups},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{per_step} consecutive lookups of {args.workload} per step "
                                   "(k0, the event loop)",
                         "k1": k1},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- our arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large_unionized", choices=sorted(WORKLOADS))
    ap.add_argument("--kernel", default="plain", choices=["plain", "batched"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"])
    ap.add_argument("--tile", type=int, default=0, help="plain kernel: lookups per block tile")
    ap.add_argument("--gridpoints", type=int, default=0,
                    help="override gridpoints per nuclide (a smaller case of the workload, for profiling)")
    ap.add_argument("--buckets", type=int, default=0, help="batched: energy buckets per material")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end measurement through xs_lookup_samples (host buffers)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the forward+adjoint side measurement (xs_run_adjoint, device arrays)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the side measurement of the other kernel on the same workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the other configurations (large hash, XL, no union table, reference CUDA)")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank)

    import torch
    import xsbench_gb300 as X
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    wl = dict(WORKLOADS[args.workload])
    if args.gridpoints:
        wl["gridpoints"] = args.gridpoints
    inputs = X.make_inputs(method="event", **wl)
    N = inputs.lookups
    t_setup = time.perf_counter()
    problem = X.grid_init(inputs)
    ctx = X.Context(inputs, problem, device=local)
    t_setup = time.perf_counter() - t_setup
    from xsbench_gb300.shard import reduce_time_max, shard_range
    first, N = shard_range(rank, world, N, "weak")
    # a non-default stream: its handle goes to the library and the events
    # below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    kw = dict(kernel=args.kernel, arith=args.arith, first=first, count=N, stream=stream,
              tile=args.tile, buckets=args.buckets)

    # correctness of this very configuration (rank 0 holds lookups [0, N))
    r = ctx.run_event(**kw)
    # the published hash holds for the workload as defined (not for a resized one)
    expected = None if args.gridpoints else X.EXPECTED_HASH.get(("event", wl["size"].lower()))
    hash_ok = (expected is None or rank != 0 or N != 17000000 or r.hash == expected)
    # W warm-up steps, continued until the GPU has been busy for about a
    # second: a freshly started GPU ran the first ~20 steps measurably slower
    # (3 warm-up steps: 849-863 M lookups/s in the first process on a box,
    # 893 M in the next; 60 warm-up steps: 893 M in the first)
    clocks = ClockSampler(local)
    clocks.start()   # past its start-up by the time the timed region begins
    warm, t_warm = 0, time.perf_counter()
    while warm < args.warmup or (time.perf_counter() - t_warm < 1.0 and warm < 200):
        ctx.run_event(async_=True, **kw)
        ctx.sync()
        warm += 1

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark_begin()
    launches = 0
    ev0.record(stream)
    for _ in range(args.steps):
        launches += ctx.run_event(async_=True, **kw).kernel_launches
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks.mark_end()
    clk = clocks.stop()
    last = ctx.sync()
    if dist:
        dist.barrier()
    t = ev0.elapsed_time(ev1) / 1e3
    t_max = reduce_time_max(t, dist)
    value = world * N * args.steps / t_max
    hash_ok = hash_ok and (rank != 0 or expected is None or N != 17000000
                           or last.hash == expected)

    # end to end through the C ABI with host buffers: samples in, macro_xs out
    e2e = None
    if not args.no_e2e:
        pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
        hE, hM = pin((N,), torch.float64), pin((N,), torch.int32)
        ctx.sample_event(first, N, hE, hM)
        hmacro, hidx = pin((N, 5), torch.float64), pin((N,), torch.uint8)
        ekw = dict(kernel=args.kernel, arith=args.arith, tile=args.tile, buckets=args.buckets)
        ctx.lookup_samples(hE, hM, macro_out=hmacro, max_idx_out=hidx, **ekw)  # warm
        e2e_t = []
        for _ in range(max(1, args.e2e_steps)):
            t0 = time.perf_counter()
            re = ctx.lookup_samples(hE, hM, macro_out=hmacro, max_idx_out=hidx, **ekw)
            e2e_t.append(time.perf_counter() - t0)
        e2e = {"value": world * N / statistics.median(e2e_t), "unit": UNIT,
               "h2d_bytes_per_step": N * 12, "d2h_bytes_per_step": N * 41 + 8,
               "api": "xs_lookup_samples (host pinned)",
               "verification_matches": bool(re.verification == last.verification)}
        del hE, hM, hmacro, hidx

    # the other lookup kernel on the same workload and context (same hash)
    other = None
    if not args.no_batched:
        okind = "batched" if args.kernel == "plain" else "plain"
        okw = dict(kw, kernel=okind, tile=0, buckets=0)
        for _ in range(max(3, args.warmup)):
            ctx.run_event(async_=True, **okw)
        ctx.sync()
        o0 = torch.cuda.Event(enable_timing=True)
        o1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        o0.record(stream)
        for _ in range(args.steps):
            ctx.run_event(async_=True, **okw)
        o1.record(stream)
        torch.cuda.synchronize()
        ro = ctx.sync()
        t_o = o0.elapsed_time(o1) / 1e3
        other = {"kernel": okind, "value": N * args.steps / t_o, "unit": UNIT,
                 "ms_per_step": t_o / args.steps * 1e3,
                 "vs_value": (N * args.steps / t_o) / (N * args.steps / t),
                 "hash_ok": ro.hash == last.hash,
                 "union_table": bool(okind == "batched" and ctx.union_table_bytes > 0)}

    adj = None
    if not args.no_adjoint:
        g = torch.randn((N, 5), dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(1234))
        d_e = torch.empty(N, dtype=torch.float64, device="cuda")
        d_c = torch.zeros((12, problem.sd.max_num_nucs), dtype=torch.float64, device="cuda")
        d_x = torch.zeros((inputs.n_isotopes, inputs.n_gridpoints, 5), dtype=torch.float64,
                          device="cuda")
        macro = torch.empty((N, 5), dtype=torch.float64, device="cuda")
        akw = dict(first=first, count=N, stream=stream, macro_out=macro, d_concs=d_c, d_xs=d_x,
                   d_energy=d_e)
        for _ in range(2):
            ctx.adjoint(g, **akw)
        times = []
        launches_adj = 0
        for _ in range(max(3, args.steps // 4)):
            ra = ctx.adjoint(g, **akw)
            times.append(ra.device_ms)
            launches_adj = ra.kernel_launches
        t_adj = statistics.median(times) / 1e3
        adj = {"value": N / t_adj, "unit": UNIT, "ms_per_step": t_adj * 1e3,
               "vs_forward": (N / t_adj) / (N * args.steps / t), "kernel_launches": launches_adj,
               "hash_ok": ra.hash == last.hash,
               "what": "forward macro_xs + dL/dE + dL/dconcs + dL/dxs, device arrays"}

    line = None
    if rank == 0:
        sm_mhz = (clk or {}).get("sm_max_mhz") or 2070.0
        fp64_peak = 2.0 * torch.cuda.get_device_properties(local).multi_processor_count * sm_mhz * 1e6
        bpl = algorithmic_bytes_per_lookup(inputs, list(problem.arrays()["num_nucs"]))
        peak, peak_kind = measured_peak_gbs()
        per_launch_s = t / args.steps
        achieved = N * bpl / per_launch_s / 1e9
        traffic_pl, traffic_src = (None, None) if args.gridpoints else \
            profiled_traffic(args.workload, args.kernel)
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cpu = cpu_baseline_oracle(inputs, problem, args.workload, args.cpu_budget)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": warm,
            "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the reference's own LCG problem generators)",
            "config": {"workload": args.workload, "kernel": args.kernel, "arith": args.arith,
                       "tile": args.tile, "buckets": args.buckets,
                       "n_isotopes": inputs.n_isotopes, "n_gridpoints": inputs.n_gridpoints,
                       "grid": wl["grid"], "lookups_per_gpu": N,
                       "l2": "inputs larger than L2 (tables > 129 MB), no flush",
                       "parallelism": f"shards x{world} (event index ranges)",
                       "hash_ok": bool(hash_ok), "hash": last.hash,
                       "setup_s": round(t_setup, 2),
                       "union_table_gb": round(ctx.union_table_bytes / 1e9, 1),
                       "device_gb": round(ctx.device_bytes / 1e9, 1)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_lookup": bpl,
                         "traffic": (traffic_pl * N if traffic_pl else None),
                         "traffic_source": traffic_src},
            # the other bound of this FP64 path: 11 FP64 instructions per nuclide
            # (FAST records: one subtraction, five interpolations, five
            # accumulations) against the FP64 pipe's rate, 2 per SM per clock
            # (ncu's peak_sustained for DFMA) x SMs x the maximum SM clock
            "fp64": ({"ops_per_lookup": round(11 * nbar_of(inputs, problem), 1),
                      "achieved_gops": value * 11 * nbar_of(inputs, problem) / 1e9,
                      "peak_gops": fp64_peak / 1e9,
                      "peak_source": "2 FP64 ops per SM per clock x SMs x max SM clock",
                      "frac": value * 11 * nbar_of(inputs, problem) / fp64_peak}
                     if args.arith == "fast" and args.kernel == "plain" else None),
            "e2e": e2e,
            "gpu_launches": launches,
            "other_kernel": other,
            "forward_adjoint": adj,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
    ctx.close()   # frees the device for the side configurations
    if rank == 0 and world == 1 and not args.no_side and not args.gridpoints \
            and args.workload == "large_unionized":
        side_clocks = ClockSampler(local)
        side_clocks.start()
        side_clocks.mark_begin()
        line["side"] = side_measurements(stream, max(3, min(args.steps, 5)), 3, fp64_peak, peak)
        side_clocks.mark_end()
        # clocks over the whole side section (set-ups included)
        line["side"]["clocks"] = side_clocks.stop()
    if rank == 0:
        print(json.dumps(line), flush=True)
    problem.close()
    if dist:
        dist.destroy_process_group()
    return 0 if hash_ok else 1


if __name__ == "__main__":
    sys.exit(main())
