"""In-tree build of the GB300 library and its C driver.

    python -m xsbench_gb300.build            # -> xsbench_gb300/_lib/libxsgb.so, xsgb,
                                             #    xsgb_gather_ceiling
    python -m xsbench_gb300.build --ptxas-v  # also print registers / spills

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, with nvcc; the host
driver is plain C compiled with the system C compiler.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libxsgb.so")
EXE_PATH = os.path.join(LIB_DIR, "xsgb")
PROBE_PATH = os.path.join(LIB_DIR, "xsgb_gather_ceiling")

CU_SOURCES = ["capi.cu", "setup_host.cu", "tables.cu", "lookup.cu", "lookup_unionized.cu",
              "lookup_nuclide.cu", "lookup_hash.cu", "static_scratch.cu", "adjoint.cu", "tune.cu",
              "setup_device.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return p.returncode, " ".join(cmd), p.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_v: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "xsgb.h"))
    nv = nvcc()
    flags = ["-O3", "-std=c++17", "-lineinfo", *GENCODE, "-Xcompiler", "-fPIC",
             "-Xcompiler", "-Wall", "-I", os.path.join(ROOT, "include")]
    if ptxas_v:
        flags += ["-Xptxas", "-v"]
    flags += os.environ.get("XSGB_NVCC_FLAGS", "").split()
    jobs = []
    objs = []
    # the gather-ceiling probe: a standalone binary, built beside the library
    probe = os.path.join(CSRC, "gather_ceiling.cu")
    if force or _stale(PROBE_PATH, [probe]):
        jobs.append([nv, "-O3", "-std=c++17", *GENCODE, "-o", PROBE_PATH, probe])
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or ptxas_v or _stale(o, [s, *headers]):
            jobs.append([nv, *flags, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for rc, cmd, out in ex.map(_run, jobs):
                if verbose or ptxas_v or rc:
                    print(cmd, "\n", out, file=sys.stderr)
                if rc:
                    raise RuntimeError(f"nvcc failed ({rc}): {cmd}\n{out}")
    if jobs or not os.path.exists(LIB_PATH):
        rc, cmd, out = _run([nv, "-shared", *GENCODE, "-o", LIB_PATH, *objs, "-lpthread"])
        if rc:
            raise RuntimeError(f"link failed: {cmd}\n{out}")
    drv = os.path.join(CSRC, "xsgb_main.c")
    if _stale(EXE_PATH, [drv, LIB_PATH, os.path.join(ROOT, "include", "xsgb.h")]):
        cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
        rc, cmd, out = _run([cc, "-std=gnu99", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                             "-o", EXE_PATH, drv, "-L", LIB_DIR, "-lxsgb",
                             "-Wl,-rpath,$ORIGIN", "-lm"])
        if rc:
            raise RuntimeError(f"driver build failed: {cmd}\n{out}")
    return LIB_PATH


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ptxas-v", action="store_true")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.verbose, ptxas_v=a.ptxas_v, force=a.force))


if __name__ == "__main__":
    main()
