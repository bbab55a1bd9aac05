"""Integer energy bins (xsbench_gb300/csrc/bin_bits.h) against the FP64
arithmetic they replace: floor(E * 2^k) of the unionized grid's bins, and the
hash grid's (long)(E / (1.0 / bins)) (openmp-threading/Simulation.c:350-351)
wherever the integer path answers; random energies and energies within a few
ulps of every bin edge.  CPU only: the header is compiled with the system C
compiler."""
import ctypes as C
import shutil
import subprocess
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(os.path.dirname(HERE), "xsbench_gb300", "csrc")

WRAP = r"""
#include "bin_bits.h"
void floors(const double *E, int *out, long n, int k)
{ for (long i = 0; i < n; i++) out[i] = xsgb_floor_scaled_pow2(E[i], k); }
void hash_bins(const double *E, long *out, int *ok, long n, unsigned bins)
{
    const int mb = xsgb_hash_margin_bits(bins);
    for (long i = 0; i < n; i++) ok[i] = xsgb_hash_bin(E[i], bins, mb, &out[i]);
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("bins")
    src, so = d / "wrap.c", d / "libwrap.so"
    src.write_text(WRAP)
    subprocess.run([cc, "-O2", "-shared", "-fPIC", "-I", HDR, "-o", str(so), str(src)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.floors.argtypes = [P, P, C.c_long, C.c_int]
    lib.hash_bins.argtypes = [P, P, P, C.c_long, C.c_uint]
    return lib


def energies(edges):
    rng = np.random.default_rng(5)
    E = [rng.random(1_000_000), rng.random(10000) * 1e-6, rng.random(1000) * 1e-300,
         np.array([0.0, -0.0, 5e-324, 2.0**-1074 * 7, 1 - 2.0**-53, 0.5, 2.0**-30])]
    # a few ulps either side of every edge
    ed = np.asarray(edges, dtype=np.float64)
    for s in range(1, 4):
        up, dn = ed.copy(), ed.copy()
        for _ in range(s):
            up = np.nextafter(up, 2.0)
            dn = np.nextafter(dn, -1.0)
        E += [up, dn]
    E.append(ed)
    E = np.concatenate(E)
    return E[(E >= 0) & (E < 1) | (E == 0)]


@pytest.mark.parametrize("k", [1, 10, 22, 31])
def test_floor_scaled_pow2(lib, k):
    E = energies(np.arange(1, 2**min(k, 16)) / 2.0**min(k, 16))
    got = np.empty(E.size, np.int32)
    lib.floors(E.ctypes.data, got.ctypes.data, E.size, k)
    want = np.floor(E * 2.0**k).astype(np.int64)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("bins", [10000, 500, 3, 7919, 65536, 1_000_000])
def test_hash_bin_matches_division(lib, bins):
    du = 1.0 / bins
    b = np.arange(1, bins)
    # edge candidates: b*du as the reference's own products, b/bins, and the
    # midpoints of the products' neighbourhoods
    E = energies(np.concatenate([b * du, b / bins]))
    got = np.empty(E.size, np.int64)
    ok = np.empty(E.size, np.int32)
    lib.hash_bins(E.ctypes.data, got.ctypes.data, ok.ctypes.data, E.size, bins)
    want = (E / du).astype(np.int64)             # (long)(E / du): truncation
    sel = ok == 1
    assert np.array_equal(got[sel], want[sel])
    # the integer path answers for all but the energies near an edge
    rng_part = slice(0, 1_000_000)
    assert ok[rng_part].mean() > 0.999
