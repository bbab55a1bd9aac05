"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference sources exist (it builds oracle/_ref/ from them
with oracle/Makefile); the fixtures it writes are committed, so nothing that
runs on a GPU machine needs the reference.

What it records, per configuration:
  setup_<cfg>.json   lengths and sha256 of every setup array the reference's
                     grid_init_do_not_profile (openmp-threading/GridInit.c:3)
                     builds (mats/concs: only the valid prefix of each row,
                     the rest is uninitialised memory in the reference)
  full_<cfg>.json    for lookups [0, N): un-modded verification sum, the hash
                     (sum % 999983), sha256 of the per-lookup argmax vector
                     (uint8) and of the macro_xs vector (N x 5 float64, little
                     endian) -- all from the reference's calculate_macro_xs
                     (openmp-threading/Simulation.c:326) called by
                     oracle/ref_harness.c
  lookups_<cfg>.npz  a sample of lookups: index, energy, material, macro_xs[5]
                     and argmax, for tests that compare values directly
  history_<size>.json  the reference's run_history_based_simulation sum
  layout.json        sizeof / offsetof of NuclideGridPoint, Inputs and
                     SimulationData as the reference header lays them out

Usage:  python tests/golden/make_golden.py [--xl]
"""
from __future__ import annotations

import argparse
import dataclasses
import ctypes as C
import hashlib
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(oracle.REFERENCE_DIR, "openmp-threading")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).data).hexdigest()


def ref_lib() -> C.CDLL:
    if not oracle.build_reference(cuda=False):
        raise SystemExit(f"the reference checkout is missing: {oracle.REFERENCE_DIR}")
    L = C.CDLL(oracle.REF_LIB_PATH)
    P = C.POINTER
    L.refh_grid_init.argtypes = [P(oracle.Inputs)]
    L.refh_grid_init.restype = P(oracle.SimData)
    L.refh_free.argtypes = [P(oracle.SimData)]
    L.refh_run_event.argtypes = [P(oracle.Inputs), P(oracle.SimData), C.c_long, C.c_long,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.refh_run_event.restype = C.c_ulonglong
    L.refh_event_simulation.argtypes = [P(oracle.Inputs), P(oracle.SimData)]
    L.refh_event_simulation.restype = C.c_ulonglong
    L.refh_history_simulation.argtypes = [P(oracle.Inputs), P(oracle.SimData)]
    L.refh_history_simulation.restype = C.c_ulonglong
    L.refh_set_threads.argtypes = [C.c_int]
    return L


def sample_indices(n: int) -> np.ndarray:
    head = np.arange(min(n, 200), dtype=np.int64)
    spread = np.unique(np.linspace(0, n - 1, 300).astype(np.int64))
    return np.unique(np.concatenate([head, spread]))


def p(x):
    return None if x is None else x.ctypes.data_as(C.c_void_p)


def one_config(L, name, cfg: oracle.Config, full=True):
    inp = cfg.inputs()
    t0 = time.time()
    sdp = L.refh_grid_init(C.byref(inp))
    sd = sdp.contents
    arrs = oracle.simdata_arrays(sd, inp)
    setup = dict(config=dataclasses.asdict(cfg), n_isotopes=inp.n_isotopes, n_gridpoints=inp.n_gridpoints,
                 max_num_nucs=sd.max_num_nucs, length_index_grid=sd.length_index_grid,
                 length_unionized_energy_array=sd.length_unionized_energy_array,
                 num_nucs=arrs["num_nucs"].tolist(),
                 sha256={k: sha(v) for k, v in arrs.items()})
    with open(os.path.join(OUT, f"setup_{name}.json"), "w") as f:
        json.dump(setup, f, indent=1)
    print(f"[{name}] setup {time.time() - t0:.1f}s", flush=True)

    # sampled lookups (one call per lookup range keeps it simple)
    idx = sample_indices(inp.lookups)
    rows = []
    for i in idx:
        macro = np.empty((1, 5), np.float64)
        mi = np.empty(1, np.uint8)
        e = np.empty(1, np.float64)
        m = np.empty(1, np.int32)
        L.refh_run_event(C.byref(inp), sdp, int(i), 1, p(macro), p(mi), p(e), p(m))
        rows.append((e[0], m[0], macro[0], mi[0]))
    np.savez_compressed(os.path.join(OUT, f"lookups_{name}.npz"), index=idx,
                        energy=np.array([r[0] for r in rows]),
                        mat=np.array([r[1] for r in rows], np.int32),
                        macro_xs=np.stack([r[2] for r in rows]),
                        max_idx=np.array([r[3] for r in rows], np.uint8))

    if full:
        t0 = time.time()
        n = inp.lookups
        macro = np.empty((n, 5), np.float64)
        mi = np.empty(n, np.uint8)
        v = L.refh_run_event(C.byref(inp), sdp, 0, n, p(macro), p(mi), None, None)
        v_sim = L.refh_event_simulation(C.byref(inp), sdp)
        assert v == v_sim, (v, v_sim)
        full_rec = dict(config=dataclasses.asdict(cfg), lookups=n, verification=int(v),
                        hash=int(v) % oracle.HASH_MODULUS, sha256_max_idx=sha(mi),
                        sha256_macro_xs=sha(macro),
                        argmax_counts=np.bincount(mi, minlength=5).tolist())
        with open(os.path.join(OUT, f"full_{name}.json"), "w") as f:
            json.dump(full_rec, f, indent=1)
        print(f"[{name}] full run {time.time() - t0:.1f}s hash={full_rec['hash']}", flush=True)
        del macro, mi
    L.refh_free(sdp)


def history(L, size):
    cfg = oracle.Config(size=size, grid="unionized", method="history")
    inp = cfg.inputs()
    sdp = L.refh_grid_init(C.byref(inp))
    v = L.refh_history_simulation(C.byref(inp), sdp)
    small_cfg = oracle.Config(size=size, grid="unionized", method="history", lookups=34,
                              particles=2000)
    inp2 = small_cfg.inputs()
    v2 = L.refh_history_simulation(C.byref(inp2), sdp)
    rec = dict(config=dataclasses.asdict(cfg), particles=inp.particles, lookups=inp.lookups,
               verification=int(v), hash=int(v) % oracle.HASH_MODULUS,
               particles_2000_verification=int(v2))
    with open(os.path.join(OUT, f"history_{size}.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(f"[history {size}] hash={rec['hash']}", flush=True)
    L.refh_free(sdp)


LAYOUT_FIELDS = {
    "NuclideGridPoint": ["energy", "total_xs", "elastic_xs", "absorbtion_xs", "fission_xs",
                         "nu_fission_xs"],
    "Inputs": ["nthreads", "n_isotopes", "n_gridpoints", "lookups", "HM", "grid_type",
               "hash_bins", "particles", "simulation_method", "binary_mode", "kernel_id"],
    "SimulationData": ["num_nucs", "concs", "mats", "unionized_energy_array", "index_grid",
                       "nuclide_grid", "length_num_nucs", "length_concs", "length_mats",
                       "length_unionized_energy_array", "length_index_grid",
                       "length_nuclide_grid", "max_num_nucs", "p_energy_samples",
                       "length_p_energy_samples", "mat_samples", "length_mat_samples"],
}


def layout():
    """Compile a probe against the reference header and record its struct layout."""
    import tempfile
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "XSbench_header.h"',
             'int main(void){ printf("{");']
    first = True
    for st, fields in LAYOUT_FIELDS.items():
        sep = "" if first else ","
        first = False
        lines.append(f'printf("{sep}\\"{st}\\": {{\\"sizeof\\": %zu", sizeof({st}));')
        for f in fields:
            lines.append(f'printf(", \\"{f}\\": %zu", offsetof({st}, {f}));')
        lines.append('printf("}");')
    lines.append('printf("}\\n"); return 0; }')
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        with open(src, "w") as f:
            f.write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-std=gnu99", f"-I{REF_DIR}", src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    rec = json.loads(out)
    with open(os.path.join(OUT, "layout.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print("[layout]", rec, flush=True)


# The dataset file of binary_write (openmp-threading/io.c:456-474), digested
# with the bytes the reference leaves undefined zeroed (oracle.datafile_digest).
DATAFILE_CASES = {
    "tiny_unionized": ["-s", "small", "-g", "1000", "-G", "unionized"],
    "tiny_hash": ["-s", "small", "-g", "1000", "-G", "hash", "-h", "500"],
    "small_unionized": ["-s", "small", "-G", "unionized"],
}


def datafile():
    """Digests of the dataset files the reference's own binary_write makes
    (oracle/_ref/XSBench ... -b write, in a scratch directory)."""
    import tempfile
    rec = {}
    for name, args in DATAFILE_CASES.items():
        with tempfile.TemporaryDirectory() as d:
            # exit status 1 = "invalid checksum" for the reduced problems (no
            # published value); the file is written before the lookups run
            out = subprocess.run([oracle.REF_EXE_PATH, *args, "-m", "event", "-l", "1000",
                                  "-t", "1", "-b", "write"], cwd=d, capture_output=True, text=True)
            assert "Writing all data structures" in out.stdout, out.stdout + out.stderr
            n, h = oracle.datafile_digest(os.path.join(d, "XS_data.dat"))
        rec[name] = {"args": args, "bytes": n, "sha256_masked": h}
        print("[datafile]", name, n, h, flush=True)
    with open(os.path.join(OUT, "datafile.json"), "w") as f:
        json.dump(rec, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--xl", action="store_true", help="also the XL hash-grid config (slow)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if args.only == "layout":
        layout()
        return
    if args.only == "datafile":
        ref_lib()   # builds oracle/_ref
        datafile()
        return
    L = ref_lib()
    L.refh_set_threads(os.cpu_count() or 1)
    configs = {
        # reduced problem for fast CPU tests: 68 nuclides x 1000 points, 200k lookups
        "tiny_unionized": oracle.Config(size="small", grid="unionized", n_gridpoints=1000, lookups=200000),
        "tiny_hash": oracle.Config(size="small", grid="hash", n_gridpoints=1000, lookups=200000, hash_bins=500),
        "tiny_nuclide": oracle.Config(size="small", grid="nuclide", n_gridpoints=1000, lookups=200000),
        "small_unionized": oracle.Config(size="small", grid="unionized"),
        "small_hash": oracle.Config(size="small", grid="hash"),
        "small_nuclide": oracle.Config(size="small", grid="nuclide"),
        "large_unionized": oracle.Config(size="large", grid="unionized"),
        "large_hash": oracle.Config(size="large", grid="hash"),
        "large_nuclide": oracle.Config(size="large", grid="nuclide"),
    }
    if args.xl:
        configs["xl_hash"] = oracle.Config(size="XL", grid="hash", lookups=100000000)
    for name, cfg in configs.items():
        if args.only and args.only != name:
            continue
        one_config(L, name, cfg)
    if not args.only:
        layout()
        datafile()
        history(L, "small")
        history(L, "large")


if __name__ == "__main__":
    main()
