"""ctypes front end of the CPU oracle (oracle/xs_oracle.c).

TEST INFRASTRUCTURE ONLY.  This is the checker for the GB300 lookup kernels;
only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm import it, and never as the thing measured or shipped.

Parity of the oracle itself is pinned by tests/test_oracle_golden.py against
fixtures dumped from the reference's own openmp-threading build
(tests/golden/make_golden.py) and against the published verification hashes
(openmp-threading/io.c:89-90).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libxsref.so")
REF_EXE_PATH = os.path.join(HERE, "_ref", "XSBench")
# The reference checkout whose sources oracle/Makefile compiles into oracle/_ref
# (the one setting for its location; XSBENCH_REFERENCE_DIR overrides it).
REFERENCE_DIR = os.environ.get("XSBENCH_REFERENCE_DIR", "/root/reference")

UNIONIZED, NUCLIDE, HASH = 0, 1, 2          # XSbench_header.h:37-39
HISTORY_BASED, EVENT_BASED = 1, 2           # XSbench_header.h:42-43
GRID_NAMES = {"unionized": UNIONIZED, "nuclide": NUCLIDE, "hash": HASH}
HASH_SMALL_EVENT, HASH_LARGE_EVENT = 945990, 952131      # io.c:89-90
HASH_SMALL_HISTORY, HASH_LARGE_HISTORY = 941535, 954318  # io.c:94-95
HASH_MODULUS = 999983                                     # Main.c:109


class GridPoint(C.Structure):  # XSbench_header.h:54-61
    _fields_ = [(n, C.c_double) for n in
                ("energy", "total_xs", "elastic_xs", "absorbtion_xs", "fission_xs", "nu_fission_xs")]


class Inputs(C.Structure):  # XSbench_header.h:63-75
    _fields_ = [("nthreads", C.c_int), ("n_isotopes", C.c_long), ("n_gridpoints", C.c_long),
                ("lookups", C.c_int), ("HM", C.c_char_p), ("grid_type", C.c_int),
                ("hash_bins", C.c_int), ("particles", C.c_int), ("simulation_method", C.c_int),
                ("binary_mode", C.c_int), ("kernel_id", C.c_int)]


class SimData(C.Structure):  # XSbench_header.h:77-102 (no AML members)
    _fields_ = [("num_nucs", C.POINTER(C.c_int)), ("concs", C.POINTER(C.c_double)),
                ("mats", C.POINTER(C.c_int)), ("unionized_energy_array", C.POINTER(C.c_double)),
                ("index_grid", C.POINTER(C.c_int)), ("nuclide_grid", C.POINTER(GridPoint)),
                ("length_num_nucs", C.c_int), ("length_concs", C.c_int), ("length_mats", C.c_int),
                ("length_unionized_energy_array", C.c_int), ("length_index_grid", C.c_long),
                ("length_nuclide_grid", C.c_int), ("max_num_nucs", C.c_int),
                ("p_energy_samples", C.POINTER(C.c_double)), ("length_p_energy_samples", C.c_int),
                ("mat_samples", C.POINTER(C.c_int)), ("length_mat_samples", C.c_int)]


@dataclass
class Config:
    """The reference's run configuration, resolved the way read_CLI does it
    (openmp-threading/io.c:227-454)."""
    size: str = "large"
    grid: str = "unionized"
    method: str = "event"
    lookups: int | None = None
    particles: int = 500000
    n_gridpoints: int | None = None
    hash_bins: int = 10000

    def inputs(self) -> Inputs:
        size = self.size.lower()
        if size not in ("small", "large", "xl", "xxl"):
            raise ValueError(f"unknown problem size {self.size!r}")
        n_iso = 68 if size == "small" else 355
        if self.n_gridpoints is not None:
            n_gp = int(self.n_gridpoints)
        elif size == "xl":
            n_gp = 238847
        elif size == "xxl":
            n_gp = int(238847 * 2.1)
        else:
            n_gp = 11303
        method = EVENT_BASED if self.method == "event" else HISTORY_BASED
        if self.lookups is not None:
            lookups, particles = int(self.lookups), int(self.particles)
        elif method == EVENT_BASED:
            lookups, particles = 34 * 500000, 0
        else:
            lookups, particles = 34, int(self.particles)
        self._hm = self.size.encode()
        return Inputs(nthreads=os.cpu_count() or 1, n_isotopes=n_iso, n_gridpoints=n_gp,
                      lookups=lookups, HM=self._hm, grid_type=GRID_NAMES[self.grid],
                      hash_bins=int(self.hash_bins), particles=particles,
                      simulation_method=method, binary_mode=0, kernel_id=0)


def datafile_digest(path: str) -> tuple:
    """(length, sha256) of a dataset file in the format of binary_write
    (openmp-threading/io.c:456-474: the raw SimulationData struct, then
    num_nucs, concs, mats, nuclide_grid, index_grid, unionized_energy_array)
    with the bytes the reference leaves undefined zeroed: the struct's pointer
    fields (stale addresses) and its unused sample fields and padding (bytes
    0-48 and 80-112), and the row padding of the 12 x max_num_nucs concs and
    mats tables past each material's num_nucs entries (Materials.c mallocs the
    tables and fills only those)."""
    import hashlib
    import struct
    b = bytearray(open(path, "rb").read())
    n_nn, n_concs, n_mats = struct.unpack_from("<3i", b, 48)
    max_nucs = struct.unpack_from("<i", b, 76)[0]
    b[0:48] = bytes(48)
    b[80:112] = bytes(32)
    nn = struct.unpack_from(f"<{n_nn}i", b, 112)
    concs_at = 112 + 4 * n_nn
    mats_at = concs_at + 8 * n_concs
    for m, k in enumerate(nn):
        row_end = (m + 1) * max_nucs
        for j in range(m * max_nucs + k, min(row_end, n_concs)):
            b[concs_at + 8 * j:concs_at + 8 * j + 8] = bytes(8)
        for j in range(m * max_nucs + k, min(row_end, n_mats)):
            b[mats_at + 4 * j:mats_at + 4 * j + 4] = bytes(4)
    return len(b), hashlib.sha256(bytes(b)).hexdigest()


def build() -> None:
    """Compile liboracle.so."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def build_reference(cuda: bool = True) -> bool:
    """Compile the reference's own sources where they lie under REFERENCE_DIR
    into oracle/_ref (its openmp-threading build and, with `cuda`, its
    cuda/Simulation.cu as an sm_103a cubin).  Returns False, building
    nothing, where the reference is absent."""
    if not os.path.isdir(os.path.join(REFERENCE_DIR, "openmp-threading")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_DIR}"], check=True)
    if cuda and os.path.isdir(os.path.join(REFERENCE_DIR, "cuda")):
        subprocess.run(["make", "-s", "-C", HERE, "refcuda", f"REF={REFERENCE_DIR}"], check=True)
    return True


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.or_grid_init.argtypes = [P(Inputs), P(SimData)]
        L.or_grid_init.restype = C.c_int
        L.or_simdata_free.argtypes = [P(SimData)]
        L.or_sample_event.argtypes = [C.c_long, P(C.c_double), P(C.c_int)]
        L.or_macro_xs.argtypes = [P(Inputs), P(SimData), C.c_double, C.c_int, P(C.c_double)]
        L.or_run_event.argtypes = [P(Inputs), P(SimData), C.c_long, C.c_long, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_run_event.restype = C.c_ulonglong
        L.or_run_event_k1.argtypes = [P(Inputs), P(SimData), C.c_long, C.c_long, C.c_int,
                                      C.c_void_p]
        L.or_run_event_k1.restype = C.c_ulonglong
        L.or_run_event_samples.argtypes = [P(Inputs), P(SimData), C.c_long, C.c_void_p,
                                           C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.or_run_event_samples.restype = C.c_ulonglong
        L.or_run_history.argtypes = [P(Inputs), P(SimData), C.c_long, C.c_long, C.c_int]
        L.or_run_history.restype = C.c_ulonglong
        L.or_lcg_skip.argtypes = [C.c_uint64, C.c_uint64]
        L.or_lcg_skip.restype = C.c_uint64
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def simdata_arrays(sd: SimData, inp: Inputs) -> dict:
    """numpy views (no copy) of the setup arrays; mats/concs restricted to the
    valid prefix of each material row."""
    out = {}
    n_gp_total = sd.length_nuclide_grid
    out["nuclide_grid"] = np.ctypeslib.as_array(
        C.cast(sd.nuclide_grid, C.POINTER(C.c_double)), shape=(n_gp_total * 6,)).reshape(-1, 6)
    out["num_nucs"] = np.ctypeslib.as_array(sd.num_nucs, shape=(sd.length_num_nucs,))
    mats = np.ctypeslib.as_array(sd.mats, shape=(sd.length_mats,)).reshape(12, sd.max_num_nucs)
    concs = np.ctypeslib.as_array(sd.concs, shape=(sd.length_concs,)).reshape(12, sd.max_num_nucs)
    nn = out["num_nucs"]
    out["mats"] = np.concatenate([mats[m, :nn[m]] for m in range(12)])
    out["concs"] = np.concatenate([concs[m, :nn[m]] for m in range(12)])
    if sd.length_unionized_energy_array > 0:
        out["unionized_energy_array"] = np.ctypeslib.as_array(
            sd.unionized_energy_array, shape=(sd.length_unionized_energy_array,))
    if sd.length_index_grid > 0:
        out["index_grid"] = np.ctypeslib.as_array(sd.index_grid, shape=(sd.length_index_grid,))
    return out


class Problem:
    """Oracle-side problem: the reference setup plus its lookup loops."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        self.inp = cfg.inputs()
        self.sd = SimData()
        if lib().or_grid_init(C.byref(self.inp), C.byref(self.sd)) != 0:
            raise MemoryError("oracle grid init failed")

    def close(self):
        if self.sd is not None:
            lib().or_simdata_free(C.byref(self.sd))
            self.sd = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def arrays(self) -> dict:
        return simdata_arrays(self.sd, self.inp)

    def run_event(self, first=0, n=None, nthreads=0, want_macro=False, want_samples=False):
        n = self.inp.lookups if n is None else int(n)
        macro = np.empty((n, 5), np.float64) if want_macro else None
        maxidx = np.empty(n, np.uint8)
        e = np.empty(n, np.float64) if want_samples else None
        m = np.empty(n, np.int32) if want_samples else None
        v = lib().or_run_event(C.byref(self.inp), C.byref(self.sd), int(first), n, int(nthreads),
                               _ptr(macro), _ptr(maxidx), _ptr(e), _ptr(m))
        return dict(verification=int(v), macro=macro, max_idx=maxidx, energy=e, mat=m)

    def run_samples(self, energy, mat, nthreads=0):
        energy = np.ascontiguousarray(energy, np.float64)
        mat = np.ascontiguousarray(mat, np.int32)
        n = energy.shape[0]
        macro = np.empty((n, 5), np.float64)
        maxidx = np.empty(n, np.uint8)
        v = lib().or_run_event_samples(C.byref(self.inp), C.byref(self.sd), n, _ptr(energy),
                                       _ptr(mat), int(nthreads), _ptr(macro), _ptr(maxidx))
        return dict(verification=int(v), macro=macro, max_idx=maxidx)

    def run_history(self, first=0, n=None, nthreads=0):
        n = self.inp.particles if n is None else int(n)
        return int(lib().or_run_history(C.byref(self.inp), C.byref(self.sd), int(first), n,
                                        int(nthreads)))


def sample_event(i: int):
    e = C.c_double()
    m = C.c_int()
    lib().or_sample_event(int(i), C.byref(e), C.byref(m))
    return e.value, m.value
