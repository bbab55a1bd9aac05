"""The host-sample pipeline's chunk schedule (xsbench_gb300/csrc/pipeline_chunks.h),
compiled with the system C compiler: every batch is cut into chunks that add
up to it, none empty or longer than a whole chunk; batches longer than 2.75
chunks ramp up and down by chunk/8, chunk/4, chunk/2 with whole-tile middle
chunks; the whole-chunk size follows the batch length.  CPU only."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HDR = os.path.join(os.path.dirname(HERE), "xsbench_gb300", "csrc")

WRAP = r"""
#include "pipeline_chunks.h"
long chunks(long n, long chunk, long tile, long *sizes, long max)
{ return xsgb_pipeline_chunks(n, chunk, tile, sizes, max); }
long whole(long n, int batched, long tile) { return xsgb_pipeline_whole(n, batched, tile); }
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("chunks")
    src, so = d / "wrap.c", d / "libwrap.so"
    src.write_text(WRAP)
    subprocess.run([cc, "-O2", "-std=c99", "-Wall", "-Werror", "-shared", "-fPIC", "-I", HDR,
                    "-o", str(so), str(src)], check=True)
    lib = C.CDLL(str(so))
    lib.chunks.argtypes = [C.c_long, C.c_long, C.c_long, C.c_void_p, C.c_long]
    lib.chunks.restype = C.c_long
    lib.whole.argtypes = [C.c_long, C.c_int, C.c_long]
    lib.whole.restype = C.c_long
    return lib


def schedule(lib, n, chunk, tile):
    k = lib.chunks(n, chunk, tile, None, 0)
    out = np.zeros(k, np.int64)
    assert lib.chunks(n, chunk, tile, out.ctypes.data, k) == k
    return out


SIZES = [1, 2, 31, 1023, 1024, 1025, 262144, 262145, 2097151, 2097152, 2097153, 5767168,
         5767169, 11534336, 11534337, 17000000, 100000000, 123456789]


@pytest.mark.parametrize("chunk,tile", [(1 << 21, 1024), (1 << 21, 2048), (1 << 22, 1024),
                                        (1 << 23, 2048), (8192, 8192), (1 << 20, 512)])
def test_chunks_cover_the_batch(lib, chunk, tile):
    for n in SIZES:
        s = schedule(lib, n, chunk, tile)
        assert s.sum() == n, (n, chunk, tile)
        assert (s > 0).all() and (s <= chunk).all(), (n, chunk, tile, s)
        r = [chunk // 8, chunk // 4, chunk // 2]
        ramped = n > 2 * sum(r) + chunk and r[0] >= tile
        if ramped:
            assert list(s[:3]) == r and list(s[-3:]) == r[::-1], (n, s)
            mid = s[3:-3]
            assert len(mid) >= 1
            assert (mid[:-1] % tile == 0).all(), (n, mid)   # whole tiles but the last
            assert (mid[:-1] == mid[0]).all()               # equal
        else:
            assert (s[:-1] == chunk).all(), (n, s)


def test_large_problem_schedule(lib):
    # the bench's end-to-end configuration: 17M lookups, 2^21-lookup chunks,
    # 1,024-lookup tiles -> 13 chunks
    s = schedule(lib, 17_000_000, lib.whole(17_000_000, 0, 1024), 1024)
    assert len(s) == 13 and s.sum() == 17_000_000
    assert list(s[:3]) == [262144, 524288, 1048576]


def test_whole_chunk_follows_the_batch(lib):
    assert lib.whole(17_000_000, 0, 1024) == 1 << 21
    assert lib.whole(17_000_000, 1, 1024) == 1 << 22
    assert lib.whole(100_000_000, 0, 2048) == 1 << 23
    assert lib.whole(100_000_000, 1, 2048) == 1 << 23
    assert lib.whole(10**10, 0, 1024) == 1 << 24      # at most 2^24
    assert lib.whole(1, 0, 1024) == 1 << 21
    assert lib.whole(1, 0, 1 << 22) == 1 << 22        # never below a tile
