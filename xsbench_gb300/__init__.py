"""xsbench_gb300 -- GB300 (sm_103a) event-based macroscopic cross-section
lookup, a drop-in for the lookup loop of XSBench.

This module is the Python host side over the C ABI of include/xsgb.h
(libxsgb.so, built in-tree by ``python -m xsbench_gb300.build``).  It mirrors
the reference's interface for the path: ``read_cli`` (openmp-threading/io.c:227),
``grid_init`` (GridInit.c:3), ``Context.run_event`` (the
run_event_based_simulation seam, Simulation.c:15) and the verification hash
(Main.c:109).  There is no CPU fallback: without the built library every call
raises.

Array arguments may be numpy arrays (host) or torch CUDA tensors (device);
device outputs are written in place by the kernels.
"""
from __future__ import annotations

import ctypes as C
import os
import shlex

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libxsgb.so")

UNIONIZED, NUCLIDE, HASH = 0, 1, 2
HISTORY_BASED, EVENT_BASED = 1, 2
KERNEL_PLAIN, KERNEL_BATCHED = 0, 1
ARITH_FAST, ARITH_EXACT = 0, 1
GRID_NAMES = {"unionized": UNIONIZED, "nuclide": NUCLIDE, "hash": HASH}
HASH_MODULUS = 999983                                      # Main.c:109
EXPECTED_HASH = {("event", "small"): 945990, ("event", "large"): 952131,     # io.c:89-90
                 ("history", "small"): 941535, ("history", "large"): 954318}  # io.c:94-95

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "no device",
          5: "timeout", 6: "data out of range", 7: "unsupported", 8: "I/O error"}


class XSError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {message}")
        self.status = status


class GridPoint(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("energy", "total_xs", "elastic_xs", "absorbtion_xs", "fission_xs", "nu_fission_xs")]


class Inputs(C.Structure):
    _fields_ = [("nthreads", C.c_int), ("n_isotopes", C.c_long), ("n_gridpoints", C.c_long),
                ("lookups", C.c_int), ("HM", C.c_char_p), ("grid_type", C.c_int),
                ("hash_bins", C.c_int), ("particles", C.c_int), ("simulation_method", C.c_int),
                ("binary_mode", C.c_int), ("kernel_id", C.c_int)]


class SimData(C.Structure):
    _fields_ = [("num_nucs", C.POINTER(C.c_int)), ("concs", C.POINTER(C.c_double)),
                ("mats", C.POINTER(C.c_int)), ("unionized_energy_array", C.POINTER(C.c_double)),
                ("index_grid", C.POINTER(C.c_int)), ("nuclide_grid", C.POINTER(GridPoint)),
                ("length_num_nucs", C.c_int), ("length_concs", C.c_int), ("length_mats", C.c_int),
                ("length_unionized_energy_array", C.c_int), ("length_index_grid", C.c_long),
                ("length_nuclide_grid", C.c_int), ("max_num_nucs", C.c_int),
                ("p_energy_samples", C.POINTER(C.c_double)), ("length_p_energy_samples", C.c_int),
                ("mat_samples", C.POINTER(C.c_int)), ("length_mat_samples", C.c_int)]


class RunOpts(C.Structure):
    _fields_ = [("kernel", C.c_int), ("arith", C.c_int), ("first", C.c_long), ("count", C.c_long),
                ("block_threads", C.c_int), ("tile_lookups", C.c_int),
                ("energy_buckets", C.c_int), ("checked", C.c_int), ("async_", C.c_int),
                ("stream", C.c_void_p)]


class RunResult(C.Structure):
    _fields_ = [("verification", C.c_ulonglong), ("device_ms", C.c_float),
                ("kernel_launches", C.c_int)]


# exported symbols of include/xsgb.h, with their ctypes signatures
_P = C.POINTER
_SIGNATURES = {
    "xs_status_str": ([C.c_int], C.c_char_p),
    "xs_last_error": ([], C.c_char_p),
    "xs_read_cli": ([C.c_int, _P(C.c_char_p), _P(Inputs)], C.c_int),
    "xs_grid_init": ([_P(Inputs), _P(SimData)], C.c_int),
    "xs_simdata_free": ([_P(SimData)], None),
    "xs_binary_write": ([C.c_char_p, _P(SimData)], C.c_int),
    "xs_binary_read": ([C.c_char_p, _P(SimData)], C.c_int),
    "xs_ctx_create": ([_P(Inputs), _P(SimData), C.c_int, _P(C.c_void_p)], C.c_int),
    "xs_ctx_create_on_device": ([_P(Inputs), C.c_int, _P(C.c_void_p)], C.c_int),
    "xs_ctx_download": ([C.c_void_p, _P(SimData)], C.c_int),
    "xs_ctx_destroy": ([C.c_void_p], None),
    "xs_ctx_device_bytes": ([C.c_void_p], C.c_size_t),
    "xs_ctx_union_table_bytes": ([C.c_void_p], C.c_size_t),
    "xs_ctx_sync": ([C.c_void_p, _P(RunResult)], C.c_int),
    "xs_run_opts_init": ([_P(RunOpts)], None),
    "xs_run_event": ([C.c_void_p, _P(RunOpts), C.c_void_p, C.c_void_p, _P(RunResult)], C.c_int),
    "xs_lookup_samples": ([C.c_void_p, _P(RunOpts), C.c_void_p, C.c_void_p, C.c_long, C.c_void_p,
                           C.c_void_p, _P(RunResult)], C.c_int),
    "xs_run_history": ([C.c_void_p, _P(RunOpts), _P(RunResult)], C.c_int),
    "xs_sample_event": ([C.c_void_p, C.c_long, C.c_long, C.c_void_p, C.c_void_p], C.c_int),
    "xs_run_adjoint": ([C.c_void_p, _P(RunOpts), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                        C.c_void_p, _P(RunResult)], C.c_int),
    "xs_adjoint_samples": ([C.c_void_p, _P(RunOpts), C.c_void_p, C.c_void_p, C.c_long, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _P(RunResult)], C.c_int),
    "xs_autotune": ([C.c_void_p, C.c_char_p, _P(RunOpts)], C.c_int),
    "xs_ctx_grid_type": ([C.c_void_p], C.c_int),
    "xs_run_event_based_simulation": ([Inputs, SimData, C.c_int, _P(C.c_ulonglong)], C.c_int),
    "xs_run_event_batched_static": ([C.c_void_p, C.c_long, C.c_long, C.c_int, C.c_int, C.c_void_p,
                                     C.c_void_p, C.c_void_p, _P(C.c_ulonglong)], C.c_int),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded libxsgb.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m xsbench_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (argt, rest) in _SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = rest
        _lib = L
    return _lib


def _check(status: int, where: str):
    if status != 0:
        raise XSError(status, where, lib().xs_last_error().decode(errors="replace"))


def _addr(x):
    """(address, is_device) of a numpy array, torch tensor or None."""
    if x is None:
        return None, False
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data, False
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return x.data_ptr(), bool(getattr(x, "is_cuda", False))
    raise TypeError(f"unsupported array type {type(x)}")


_DTYPES = {"f64": (np.float64, "float64"), "i32": (np.int32, "int32"), "u8": (np.uint8, "uint8")}


def _check_array(x, n_elems: int, kind: str, name: str, device: bool | None = None):
    """Raises ValueError unless x is None or a contiguous array of n_elems
    elements of type `kind` ("f64", "i32", "u8"); device=True / False also
    requires a CUDA tensor / host array.  The C side receives bare pointers
    and cannot check sizes, so this is where a short or mistyped buffer is
    caught before a kernel writes past its end."""
    if x is None:
        return
    np_t, torch_name = _DTYPES[kind]
    if isinstance(x, np.ndarray):
        ok_type, numel, is_dev = x.dtype == np_t, int(x.size), False
    elif hasattr(x, "data_ptr"):
        ok_type = str(x.dtype).replace("torch.", "") == torch_name
        numel, is_dev = int(x.numel()), bool(getattr(x, "is_cuda", False))
    else:
        raise TypeError(f"{name}: unsupported array type {type(x)}")
    if not ok_type:
        raise ValueError(f"{name} must hold {torch_name} elements, not {x.dtype}")
    if numel != int(n_elems):
        raise ValueError(f"{name} must hold {int(n_elems)} elements, not {numel}")
    if device is True and not is_dev:
        raise ValueError(f"{name} must be a CUDA tensor")
    if device is False and is_dev:
        raise ValueError(f"{name} must be a host array")


# ------------------------------------------------------------------ inputs
def read_cli(args) -> Inputs:
    """Inputs from a reference-style command line (io.c:227-454)."""
    if isinstance(args, str):
        args = shlex.split(args)
    argv = ["xsgb", *[str(a) for a in args]]
    keep = [a.encode() for a in argv]
    arr = (C.c_char_p * len(keep))(*keep)
    inp = Inputs()
    _check(lib().xs_read_cli(len(keep), arr, C.byref(inp)), "xs_read_cli")
    # HM points into argv: keep a private copy alive with the struct
    hm = inp.HM
    inp._hm = C.create_string_buffer(hm)
    inp.HM = C.cast(inp._hm, C.c_char_p)
    return inp


def make_inputs(size="large", grid="unionized", method="event", lookups=None, particles=None,
                gridpoints=None, hash_bins=None, kernel_id=0) -> Inputs:
    args = ["-s", size, "-G", grid, "-m", method, "-k", str(kernel_id)]
    if lookups is not None:
        args += ["-l", str(int(lookups))]
    if particles is not None:
        args += ["-p", str(int(particles))]
    if gridpoints is not None:
        args += ["-g", str(int(gridpoints))]
    if hash_bins is not None:
        args += ["-h", str(int(hash_bins))]
    return read_cli(args)


# ------------------------------------------------------------- host setup
class HostProblem:
    """The reference's SimulationData, built by xs_grid_init (GridInit.c:3)."""

    def __init__(self, inputs: Inputs, sd: SimData | None = None):
        self.inputs = inputs
        self.sd = SimData()
        if sd is None:
            _check(lib().xs_grid_init(C.byref(inputs), C.byref(self.sd)), "xs_grid_init")
        else:
            self.sd = sd

    @classmethod
    def from_file(cls, inputs: Inputs, path: str) -> "HostProblem":
        sd = SimData()
        _check(lib().xs_binary_read(path.encode(), C.byref(sd)), "xs_binary_read")
        return cls(inputs, sd)

    def write(self, path: str):
        _check(lib().xs_binary_write(path.encode(), C.byref(self.sd)), "xs_binary_write")

    def arrays(self, copy: bool = False) -> dict:
        """The setup arrays by reference name.  Without `copy` the arrays are
        views of the C arrays and are valid only until close()."""
        if copy:
            return {k: np.array(v) for k, v in self.arrays().items()}
        sd = self.sd
        out = {"nuclide_grid": np.ctypeslib.as_array(
            C.cast(sd.nuclide_grid, C.POINTER(C.c_double)),
            shape=(sd.length_nuclide_grid * 6,)).reshape(-1, 6)}
        out["num_nucs"] = np.ctypeslib.as_array(sd.num_nucs, shape=(12,))
        mats = np.ctypeslib.as_array(sd.mats, shape=(sd.length_mats,)).reshape(12, -1)
        concs = np.ctypeslib.as_array(sd.concs, shape=(sd.length_concs,)).reshape(12, -1)
        nn = out["num_nucs"]
        out["mats"] = np.concatenate([mats[m, :nn[m]] for m in range(12)])
        out["concs"] = np.concatenate([concs[m, :nn[m]] for m in range(12)])
        if sd.length_unionized_energy_array > 0:
            out["unionized_energy_array"] = np.ctypeslib.as_array(
                sd.unionized_energy_array, shape=(sd.length_unionized_energy_array,))
        if sd.length_index_grid > 0:
            out["index_grid"] = np.ctypeslib.as_array(sd.index_grid, shape=(sd.length_index_grid,))
        return out

    def close(self):
        if self.sd is not None:
            lib().xs_simdata_free(C.byref(self.sd))
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


def grid_init(inputs: Inputs) -> HostProblem:
    return HostProblem(inputs)


# ----------------------------------------------------------------- device
class Result:
    def __init__(self, r: RunResult):
        self.verification = int(r.verification)
        self.device_ms = float(r.device_ms)
        self.kernel_launches = int(r.kernel_launches)

    @property
    def hash(self) -> int:
        return self.verification % HASH_MODULUS

    def __repr__(self):
        return (f"Result(verification={self.verification}, hash={self.hash}, "
                f"device_ms={self.device_ms:.3f}, launches={self.kernel_launches})")


def _opts(kernel=KERNEL_PLAIN, arith=ARITH_FAST, first=0, count=0, tile=0, buckets=0,
          checked=False, async_=False, stream=None, block=0) -> RunOpts:
    o = RunOpts()
    lib().xs_run_opts_init(C.byref(o))
    o.kernel = {"plain": KERNEL_PLAIN, "batched": KERNEL_BATCHED}.get(kernel, kernel)
    o.arith = {"fast": ARITH_FAST, "exact": ARITH_EXACT}.get(arith, arith)
    o.first, o.count = int(first), int(count)
    o.tile_lookups, o.energy_buckets = int(tile), int(buckets)
    o.block_threads = int(block)
    o.checked, o.async_ = int(bool(checked)), int(bool(async_))
    if stream is not None:
        o.stream = C.c_void_p(stream if isinstance(stream, int) else stream.cuda_stream)
    return o


class Context:
    """A problem resident on one GPU (xs_ctx)."""

    def __init__(self, inputs: Inputs, problem: HostProblem | None = None, device: int = 0):
        self.inputs = inputs
        self._h = C.c_void_p()
        # row length of the 12-row material tables (d_concs is 12 x this):
        # the fuel's nuclide count, Materials.c:7-30
        self.max_num_nucs = (int(problem.sd.max_num_nucs) if problem is not None
                             else (34 if int(inputs.n_isotopes) == 68 else 321))
        if problem is None:
            _check(lib().xs_ctx_create_on_device(C.byref(inputs), int(device), C.byref(self._h)),
                   "xs_ctx_create_on_device")
        else:
            _check(lib().xs_ctx_create(C.byref(inputs), C.byref(problem.sd), int(device),
                                       C.byref(self._h)), "xs_ctx_create")

    @property
    def device_bytes(self) -> int:
        return int(lib().xs_ctx_device_bytes(self._h))

    @property
    def union_table_bytes(self) -> int:
        """Bytes of the union table (0: the lookups read index entries and
        interval records)."""
        return int(lib().xs_ctx_union_table_bytes(self._h))

    def _count(self, first=0, count=0, **_):
        return int(count) if int(count) > 0 else int(self.inputs.lookups) - int(first)

    def run_event(self, macro_out=None, max_idx_out=None, **kw) -> Result:
        n = self._count(**kw)
        _check_array(macro_out, n * 5, "f64", "macro_out")
        _check_array(max_idx_out, n, "u8", "max_idx_out")
        o = _opts(**kw)
        r = RunResult()
        pm, _ = _addr(macro_out)
        pi, _ = _addr(max_idx_out)
        _check(lib().xs_run_event(self._h, C.byref(o), pm, pi, C.byref(r)), "xs_run_event")
        return Result(r)

    def lookup_samples(self, energy, mat, macro_out=None, max_idx_out=None, **kw) -> Result:
        n = int(energy.shape[0])
        if int(mat.shape[0]) != n:
            raise ValueError("energy and mat lengths differ")
        if macro_out is not None and tuple(macro_out.shape) != (n, 5):
            raise ValueError("macro_out must be (n, 5)")
        _check_array(energy, n, "f64", "energy")
        _check_array(mat, n, "i32", "mat")
        _check_array(macro_out, n * 5, "f64", "macro_out")
        _check_array(max_idx_out, n, "u8", "max_idx_out")
        o = _opts(**kw)
        r = RunResult()
        pe, _ = _addr(energy)
        pmat, _ = _addr(mat)
        pm, _ = _addr(macro_out)
        pi, _ = _addr(max_idx_out)
        _check(lib().xs_lookup_samples(self._h, C.byref(o), pe, pmat, n, pm, pi, C.byref(r)),
               "xs_lookup_samples")
        return Result(r)

    def sample_event(self, first: int, count: int, energy_out=None, mat_out=None):
        """(energy, material) of lookups [first, first+count) (Simulation.c:735-750)."""
        if energy_out is None:
            energy_out = np.empty(int(count), np.float64)
        if mat_out is None:
            mat_out = np.empty(int(count), np.int32)
        _check_array(energy_out, int(count), "f64", "energy_out")
        _check_array(mat_out, int(count), "i32", "mat_out")
        pe, _ = _addr(energy_out)
        pm, _ = _addr(mat_out)
        _check(lib().xs_sample_event(self._h, int(first), int(count), pe, pm), "xs_sample_event")
        return energy_out, mat_out

    def run_history(self, **kw) -> Result:
        o = _opts(**kw)
        r = RunResult()
        _check(lib().xs_run_history(self._h, C.byref(o), C.byref(r)), "xs_run_history")
        return Result(r)

    def run_event_batched_static(self, first: int, count: int, arith="fast", buckets=0,
                                 macro_out=None, max_idx_out=None, stream=None) -> int:
        """Batched lookups with no device allocation (at most 524,288 per call;
        outputs on the device or None); returns the un-modded verification sum."""
        v = C.c_ulonglong()
        _check_array(macro_out, int(count) * 5, "f64", "macro_out", device=True)
        _check_array(max_idx_out, int(count), "u8", "max_idx_out", device=True)
        pm, _ = _addr(macro_out)
        pi, _ = _addr(max_idx_out)
        a = {"fast": ARITH_FAST, "exact": ARITH_EXACT}.get(arith, arith)
        s = None if stream is None else C.c_void_p(stream if isinstance(stream, int) else stream.cuda_stream)
        _check(lib().xs_run_event_batched_static(self._h, int(first), int(count), int(a),
                                                 int(buckets), pm, pi, s, C.byref(v)),
               "xs_run_event_batched_static")
        return int(v.value)

    def adjoint(self, gbar, energy=None, mat=None, macro_out=None, d_concs=None, d_xs=None,
                d_energy=None, **kw) -> Result:
        """Gradients of L = sum(gbar * macro_xs): d_energy is written, d_concs
        (12 x max_num_nucs) and d_xs (n_isotopes x n_gridpoints x 5) are added
        to.  Lookups are [first, first+count) of the event batch, or the
        caller's (energy, mat) samples."""
        n = int(energy.shape[0]) if energy is not None else self._count(**kw)
        if energy is not None:
            _check_array(energy, n, "f64", "energy")
            _check_array(mat, n, "i32", "mat")
        _check_array(gbar, n * 5, "f64", "gbar")
        _check_array(macro_out, n * 5, "f64", "macro_out")
        _check_array(d_concs, 12 * int(self.max_num_nucs), "f64", "d_concs")
        _check_array(d_xs, int(self.inputs.n_isotopes) * int(self.inputs.n_gridpoints) * 5, "f64",
                     "d_xs")
        _check_array(d_energy, n, "f64", "d_energy")
        o = _opts(**kw)
        r = RunResult()
        a = [_addr(x)[0] for x in (gbar, macro_out, d_concs, d_xs, d_energy)]
        if energy is None:
            _check(lib().xs_run_adjoint(self._h, C.byref(o), *a, C.byref(r)), "xs_run_adjoint")
        else:
            n = int(energy.shape[0])
            pe, _ = _addr(energy)
            pm, _ = _addr(mat)
            _check(lib().xs_adjoint_samples(self._h, C.byref(o), pe, pm, n, *a, C.byref(r)),
                   "xs_adjoint_samples")
        return Result(r)

    def autotune(self, cache_path: str | None = None) -> dict:
        """Time the kernel shapes and grid types and keep the fastest (xs_autotune)."""
        o = RunOpts()
        _check(lib().xs_autotune(self._h, cache_path.encode() if cache_path else None,
                                 C.byref(o)), "xs_autotune")
        return {"kernel": ("plain", "batched")[o.kernel], "tile": o.tile_lookups,
                "buckets": o.energy_buckets, "block": o.block_threads, "grid": self.grid_type}

    @property
    def grid_type(self) -> str:
        return {0: "unionized", 1: "nuclide", 2: "hash"}[lib().xs_ctx_grid_type(self._h)]

    def sync(self) -> Result:
        r = RunResult()
        _check(lib().xs_ctx_sync(self._h, C.byref(r)), "xs_ctx_sync")
        return Result(r)

    def download(self) -> HostProblem:
        sd = SimData()
        _check(lib().xs_ctx_download(self._h, C.byref(sd)), "xs_ctx_download")
        return HostProblem(self.inputs, sd)

    def close(self):
        if self._h:
            lib().xs_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_event_based_simulation(inputs: Inputs, problem: HostProblem, mype: int = 0) -> int:
    """The reference seam (XSbench_header.h:117): un-modded verification sum."""
    v = C.c_ulonglong()
    _check(lib().xs_run_event_based_simulation(inputs, problem.sd, int(mype), C.byref(v)),
           "xs_run_event_based_simulation")
    return int(v.value)
