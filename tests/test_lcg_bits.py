"""The integer form of the reference's LCG draw (xsbench_gb300/csrc/lcg_bits.h)
against the floating-point one it replaces on the device: (double)s / 2^63
(openmp-threading/Simulation.c:462-470), the material roll against the
running sums (Simulation.c:426-460) and the energy bucket floor(E * 2^k), for
random states and for the rounding edges (ties, carries into the next binade,
states next to powers of two).  CPU only: the header is compiled with the
system C compiler."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(os.path.dirname(HERE), "xsbench_gb300", "csrc")

WRAP = r"""
#include "lcg_bits.h"
void values(const uint64_t *s, double *out, long n)
{ for (long i = 0; i < n; i++) out[i] = xsgb_lcg_value(s[i]); }
void buckets(const uint64_t *s, int *out, long n, int k)
{ for (long i = 0; i < n; i++) out[i] = xsgb_lcg_bucket(s[i], k); }
uint64_t threshold(double x) { return xsgb_lcg_threshold(x); }
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("lcg")
    src, so = d / "wrap.c", d / "libwrap.so"
    src.write_text(WRAP)
    subprocess.run([cc, "-O2", "-shared", "-fPIC", "-I", HDR, "-o", str(so), str(src)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.values.argtypes = [P, P, C.c_long]
    lib.buckets.argtypes = [P, P, C.c_long, C.c_int]
    lib.threshold.argtypes = [C.c_double]
    lib.threshold.restype = C.c_uint64
    return lib


def states():
    rng = np.random.default_rng(3)
    s = [rng.integers(0, 2**63, 2_000_000, dtype=np.uint64)]
    edges = []
    for e in range(50, 63):                       # every binade that rounds
        base = np.uint64(1) << np.uint64(e)
        sh = e - 52                               # bits dropped below the 53 kept
        for q in (0, 1, 2, 3, (1 << 52) - 1, (1 << 52) - 2):
            top = base + (np.uint64(q) << np.uint64(sh)) if sh > 0 else base + np.uint64(q)
            for d in range(-3, 4):
                edges.append(int(top) + d)
            if sh > 0:
                half = 1 << (sh - 1)
                for d in (-1, 0, 1):
                    edges.append(int(top) + half + d)
    edges += [0, 1, 2, 2**53 - 1, 2**53, 2**53 + 1, 2**63 - 1, 2**63 - 2, 2**63 - 512, 2**63 - 513]
    e = np.array([x for x in edges if 0 <= x < 2**63], dtype=np.uint64)
    return np.concatenate(s + [e])


def test_value_bit_identical(lib):
    s = states()
    got = np.empty(s.size)
    lib.values(s.ctypes.data, got.ctypes.data, s.size)
    want = s.astype(np.float64) * 2.0**-63       # the C conversion, to nearest
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.parametrize("k", [0, 1, 8, 12, 15, 16])
def test_bucket_is_floor_of_scaled_draw(lib, k):
    s = states()
    got = np.empty(s.size, np.int32)
    lib.buckets(s.ctypes.data, got.ctypes.data, s.size, k)
    E = s.astype(np.float64) * 2.0**-63
    want = np.minimum((E * 2.0**k).astype(np.int64), 2**k - 1)
    assert np.array_equal(got, want)


def test_material_roll_by_state(lib):
    """s < T(x) exactly when draw(s) < x, for the reference's running sums and
    for random thresholds."""
    dist = [0.140, 0.052, 0.275, 0.134, 0.154, 0.064, 0.066, 0.055, 0.008, 0.015, 0.025, 0.013]
    sums = []
    for i in range(1, 12):          # Simulation.c:450-457, summed in its order
        run = 0.0
        for j in range(i, 0, -1):
            run += dist[j]
        sums.append(run)
    rng = np.random.default_rng(4)
    xs = sums + list(rng.random(20)) + [0.0, 1.0, 2.0**-60, 0.5, 1 - 2.0**-53]
    s = states()
    draw = s.astype(np.float64) * 2.0**-63
    for x in xs:
        T = lib.threshold(float(x))
        assert np.array_equal(s < np.uint64(T), draw < x), x
        # T itself is the first state that reaches x
        if 0 < T < 2**63:
            assert float(np.uint64(T)) * 2.0**-63 >= x > float(np.uint64(T - 1)) * 2.0**-63
