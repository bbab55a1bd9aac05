"""Register and spill budgets of the hot lookup kernels, read from ptxas's
report when the three lookup units are compiled for sm_103a (no GPU needed).

The kernels' speed rests on their occupancy: the plain kernel runs four
256-thread blocks per SM (64 registers), the persistent list kernel four
(three on the hash grid, 80 registers), and a change in the shared device
code can raise a kernel's registers and drop it a block per SM without any
result changing (the hash-grid list kernel at 96 registers ran 11-17 %
slower).  These budgets catch that at build time."""
import concurrent.futures as cf
import os
import re
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "xsbench_gb300", "csrc")


def ptxas_report(unit, out_dir):
    from xsbench_gb300 import build as B
    cmd = [B.nvcc(), "-O3", "-std=c++17", *B.GENCODE, "-Xptxas", "-v", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, unit),
           "-o", os.path.join(out_dir, unit + ".o")]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-2000:]
    res = {}
    name = None
    for line in p.stderr.splitlines():
        m = re.search(r"Compiling entry function '(\w+)'", line)
        if m:
            name = m.group(1)
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and name:
            res.setdefault(name, {})["spill"] = int(m.group(1)) + int(m.group(2))
        m = re.search(r"Used (\d+) registers", line)
        if m and name:
            res.setdefault(name, {})["regs"] = int(m.group(1))
    return res


@pytest.fixture(scope="module")
def reports(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("ptxas"))
    units = ["lookup_unionized.cu", "lookup_nuclide.cu", "lookup_hash.cu"]
    with cf.ThreadPoolExecutor(3) as ex:
        out = {}
        for r in ex.map(lambda u: ptxas_report(u, d), units):
            out.update(r)
    return out


def entry(reports, pattern):
    hits = [v for k, v in reports.items() if re.search(pattern, k)]
    assert hits, pattern
    return hits[0]


# (mangled-name pattern, register budget, spill budget in bytes)
BUDGETS = [
    # plain kernel, FAST, unchecked, LCG sampling, 256 threads: unionized
    # (staged rows and not), nuclide, hash
    (r"k_plainILi0ELi0ELb0ELb0ELb1ELi256E", 64, 0),
    (r"k_plainILi0ELi0ELb0ELb0ELb0ELi256E", 64, 0),
    (r"k_plainILi1ELi0ELb0ELb0ELb0ELi256E", 64, 64),
    (r"k_plainILi2ELi0ELb0ELb0ELb0ELi256E", 64, 160),
    # persistent list kernel, FAST, unchecked, 256 threads
    (r"k_list_lookupILi0ELi0ELb0ELi256E", 64, 0),
    (r"k_list_lookupILi1ELi0ELb0ELi256E", 64, 0),
    (r"k_list_lookupILi2ELi0ELb0ELi256E", 80, 0),
    # the union-table list kernel (two blocks per SM by design)
    (r"k_list_lookup_tableILi0ELi256E", 128, 0),
]


@pytest.mark.parametrize("pattern,regs,spill", BUDGETS)
def test_hot_kernel_budgets(reports, pattern, regs, spill):
    e = entry(reports, pattern)
    assert e["regs"] <= regs, (pattern, e)
    assert e["spill"] <= spill, (pattern, e)
