"""The C-ABI boundary: the library loads, exports every entry point that
include/xsgb.h declares, and its structs are laid out like the reference's
(openmp-threading/XSbench_header.h:54-102).  No compute call needs a GPU here."""
import ctypes as C
import os
import re
import subprocess

import pytest

import oracle
import xsbench_gb300 as X
from conftest import ROOT, golden_json, product_inputs

HEADER = os.path.join(ROOT, "include", "xsgb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xs_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 20
    L = X.lib()
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", X.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (xs_\w+)", out))
    assert set(names) <= exported
    # and the Python binding covers all of them
    assert set(names) == set(X._SIGNATURES)


def test_struct_layout_matches_reference():
    g = golden_json("layout")
    for st, ct in (("NuclideGridPoint", X.GridPoint), ("Inputs", X.Inputs),
                   ("SimulationData", X.SimData)):
        assert C.sizeof(ct) == g[st]["sizeof"], st
        for f, off in g[st].items():
            if f != "sizeof":
                assert getattr(ct, f).offset == off, (st, f)
    # the oracle's mirror too
    for st, ct in (("NuclideGridPoint", oracle.GridPoint), ("Inputs", oracle.Inputs),
                   ("SimulationData", oracle.SimData)):
        assert C.sizeof(ct) == g[st]["sizeof"], st


def test_c_header_compiles_as_c99_and_layout_asserts(tmp_path):
    g = golden_json("layout")
    src = tmp_path / "t.c"
    src.write_text(
        '#include <stddef.h>\n#include "xsgb.h"\n'
        f'_Static_assert(sizeof(xs_gridpoint) == {g["NuclideGridPoint"]["sizeof"]}, "gp");\n'
        f'_Static_assert(sizeof(xs_inputs) == {g["Inputs"]["sizeof"]}, "in");\n'
        f'_Static_assert(sizeof(xs_simdata) == {g["SimulationData"]["sizeof"]}, "sd");\n'
        f'_Static_assert(offsetof(xs_simdata, length_index_grid) == {g["SimulationData"]["length_index_grid"]}, "lig");\n'
        'int main(void){ return 0; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(tmp_path / "t")], check=True)


def test_status_strings_and_errors_without_gpu():
    L = X.lib()
    for s in range(9):
        assert L.xs_status_str(s)
    h = C.c_void_p()
    with X.grid_init(product_inputs("tiny_hash")) as p:
        st = L.xs_ctx_create(C.byref(p.inputs), C.byref(p.sd), 0, C.byref(h))
        assert st in (0, 4)          # ok on a GB300, "no device" elsewhere
        if st == 0:
            L.xs_ctx_destroy(h)
        else:
            assert b"device" in L.xs_last_error()
        # argument checks come before any device work
        st = L.xs_ctx_create(C.byref(p.inputs), None, 0, C.byref(h))
        assert st == 1


def test_run_calls_reject_null_context():
    L = X.lib()
    r = X.RunResult()
    assert L.xs_run_event(None, None, None, None, C.byref(r)) == 1
    assert L.xs_run_history(None, None, C.byref(r)) == 1
    assert L.xs_lookup_samples(None, None, None, None, 0, None, None, C.byref(r)) == 1
    assert L.xs_ctx_sync(None, C.byref(r)) == 1


def test_driver_binary_built():
    from xsbench_gb300 import build as B
    assert os.access(B.EXE_PATH, os.X_OK)
    p = subprocess.run([B.EXE_PATH, "-q"], capture_output=True, text=True)
    assert p.returncode == 2 and "invalid argument" in p.stderr


def test_gather_ceiling_probe_is_built_and_checks_its_argument():
    """build() leaves the gather-ceiling probe beside the library; it is an
    sm_103a binary, and it refuses a buffer size outside [2^28, 2^37] before
    touching any device."""
    from xsbench_gb300 import build as B
    assert os.path.exists(B.PROBE_PATH) and os.access(B.PROBE_PATH, os.X_OK)
    p = subprocess.run([B.PROBE_PATH, "40"], capture_output=True, text=True, timeout=60)
    assert p.returncode == 2 and "buffer_log2" in p.stdout


DROP_IN = r"""
#include "XSbench_header.h"
#include "xsgb.h"
/* the binding of the reference's Main.c:82-83 (event-based, kernel 0) */
unsigned long long drop_in(Inputs in, SimulationData SD, int mype, int *status)
{
    unsigned long long verification = 0;
    xs_status st = xs_run_event_based_simulation(*(xs_inputs *)&in, *(xs_simdata *)&SD, mype,
                                                 &verification);
    *status = (int)st;
    return verification;
}
int main(void)
{
    Inputs in;
    SimulationData SD;
    memset(&in, 0, sizeof in);
    memset(&SD, 0, sizeof SD);
    int st = 0;
    drop_in(in, SD, 0, &st);
    printf("%d %s\n", st, xs_status_str((xs_status)st));
    return 0;
}
"""


def test_drop_in_binding_compiles_with_the_reference_header(tmp_path):
    """The call a maintainer adds to the reference's Main.c compiles in one
    translation unit with the reference's own XSbench_header.h (no clashing
    names, struct casts as the integration notes show) and links against the
    library; an empty problem is refused before any device work."""
    ref = os.path.join(oracle.REFERENCE_DIR, "openmp-threading")
    if not os.path.exists(os.path.join(ref, "XSbench_header.h")):
        pytest.skip("reference checkout not present")
    from xsbench_gb300 import build as B
    src = tmp_path / "drop_in.c"
    src.write_text(DROP_IN)
    exe = tmp_path / "drop_in"
    subprocess.run(["gcc", "-std=gnu99", "-Wall", "-Werror", "-I", ref, "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", B.LIB_DIR,
                    "-lxsgb", f"-Wl,-rpath,{B.LIB_DIR}"], check=True)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.split()[0] == "1"          # XS_ERR_INVALID_ARGUMENT


def test_e2e_breakdown_module_parses_its_arguments():
    """The end-to-end breakdown diagnostic (python -m xsbench_gb300.e2e_breakdown)
    answers --help without a GPU."""
    import sys
    p = subprocess.run([sys.executable, "-m", "xsbench_gb300.e2e_breakdown", "--help"],
                       capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert p.returncode == 0 and "--kernel" in p.stdout
