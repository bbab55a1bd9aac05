"""The product's host problem setup (xs_grid_init) and command line
(xs_read_cli) against the reference: every setup array is compared by sha256
with the arrays the reference's grid_init_do_not_profile built
(openmp-threading/GridInit.c:3), and the CLI resolution with read_CLI
(openmp-threading/io.c:227-454)."""
import os

import numpy as np
import pytest

import oracle
import xsbench_gb300 as X
from conftest import golden_json, oracle_config, product_inputs, sha


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "tiny_nuclide",
                                  "small_unionized", "small_hash", "small_nuclide",
                                  "large_hash", "large_nuclide", "large_unionized", "xl_hash"])
def test_grid_init_matches_reference(name):
    g = golden_json("setup_" + name)
    with X.grid_init(product_inputs(name)) as p:
        a = p.arrays()
        assert set(a) == set(g["sha256"])
        for k, v in a.items():
            assert sha(v) == g["sha256"][k], k
        assert p.sd.max_num_nucs == g["max_num_nucs"]
        assert p.sd.length_index_grid == g["length_index_grid"]


def test_grid_init_matches_oracle_memcmp():
    name = "tiny_unionized"
    with X.grid_init(product_inputs(name)) as p, oracle.Problem(oracle_config(name)) as o:
        a, b = p.arrays(), o.arrays()
        for k in a:
            assert np.array_equal(a[k], b[k]), k


def test_grid_init_thread_count_invariant(monkeypatch):
    name = "tiny_unionized"
    digests = []
    for t in ("1", "3", "8"):
        monkeypatch.setenv("XSGB_HOST_THREADS", t)
        with X.grid_init(product_inputs(name)) as p:
            digests.append({k: sha(v) for k, v in p.arrays().items()})
    assert digests[0] == digests[1] == digests[2]


def test_binary_file_round_trip(tmp_path):
    name = "tiny_hash"
    path = str(tmp_path / "XS_data.dat")
    inp = product_inputs(name)
    with X.grid_init(inp) as p:
        p.write(path)
        a = p.arrays(copy=True)
    with X.HostProblem.from_file(inp, path) as q:
        b = q.arrays(copy=True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # the file layout is the reference's: struct, then six arrays (io.c:456-474)
    sz = os.path.getsize(path)
    g = golden_json("layout")
    n_pts = 68 * 1000
    expect = (g["SimulationData"]["sizeof"] + 12 * 4 + 12 * 34 * 8 + 12 * 34 * 4 + n_pts * 48
              + 500 * 68 * 4)
    assert sz == expect


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash", "small_unionized"])
def test_binary_write_matches_reference_writer(tmp_path, name):
    """xs_binary_write writes, byte for byte, the file the reference's own
    binary_write writes for the same problem (openmp-threading/io.c:456-474;
    digest from the reference build, tests/golden/make_golden.py), apart from
    the struct's pointer fields and unused sample fields, which the reference
    dumps as stale addresses and uninitialised memory, and the unfilled row
    padding of its concs and mats tables (oracle.datafile_digest)."""
    g = golden_json("datafile")
    rec = g[name]
    path = str(tmp_path / "XS_data.dat")
    inp = X.read_cli(rec["args"] + ["-m", "event"])
    with X.grid_init(inp) as p:
        p.write(path)
    assert oracle.datafile_digest(path) == (rec["bytes"], rec["sha256_masked"])


def reference_exe():
    if not os.path.exists(oracle.REF_EXE_PATH):
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    return oracle.REF_EXE_PATH


@pytest.mark.parametrize("name", ["tiny_unionized", "tiny_hash"])
def test_binary_read_of_reference_written_file(tmp_path, name):
    """A file written by the reference build itself is read by xs_binary_read
    into arrays identical to the reference's setup (sha256 of every array),
    and its masked digest is the committed one."""
    import subprocess
    g = golden_json("datafile")
    rec = g[name]
    subprocess.run([reference_exe(), *rec["args"], "-m", "event", "-l", "1000", "-t", "2",
                    "-b", "write"], cwd=str(tmp_path), capture_output=True, timeout=600)
    path = str(tmp_path / "XS_data.dat")
    assert oracle.datafile_digest(path) == (rec["bytes"], rec["sha256_masked"])
    setup = golden_json("setup_" + name)
    with X.HostProblem.from_file(product_inputs(name), path) as q:
        for k, v in q.arrays().items():
            assert sha(v) == setup["sha256"][k], k


def test_reference_reads_file_written_here(tmp_path):
    """The reference build reads a file written by xs_binary_write
    (binary_read, io.c:476-508) and its lookups give the reference's
    verification value for that problem."""
    import re
    import subprocess
    exe = reference_exe()
    name = "tiny_unionized"
    full = golden_json("full_" + name)
    with X.grid_init(product_inputs(name)) as p:
        p.write(str(tmp_path / "XS_data.dat"))
    out = subprocess.run([exe, "-s", "small", "-g", "1000", "-G", "unionized", "-m", "event",
                          "-l", str(full["lookups"]), "-t", "4", "-b", "read"],
                         cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert "Reading all data structures" in out.stdout
    m = re.search(r"Verification checksum: (\d+)", out.stdout)
    assert m and int(m.group(1)) == full["hash"], out.stdout[-500:]


def test_binary_read_rejects_garbage(tmp_path):
    path = tmp_path / "bad.dat"
    path.write_bytes(b"\x01" * 64)
    with pytest.raises(X.XSError) as e:
        X.HostProblem.from_file(product_inputs("tiny_hash"), str(path))
    assert e.value.status == 8
    with pytest.raises(X.XSError) as e:
        X.HostProblem.from_file(product_inputs("tiny_hash"), str(tmp_path / "missing.dat"))
    assert e.value.status == 8


def test_read_cli_defaults_and_event_rule():
    # io.c:231-272 defaults; -m event multiplies lookups by particles (io.c:319-323)
    d = X.read_cli([])
    assert (d.simulation_method, d.n_isotopes, d.n_gridpoints, d.lookups, d.particles,
            d.grid_type, d.hash_bins, d.kernel_id) == (1, 355, 11303, 34, 500000, 0, 10000, 0)
    e = X.read_cli("-m event")
    assert e.lookups == 17000000 and e.particles == 0
    e2 = X.read_cli("-l 100 -m event")      # user lookups: no multiplication
    assert e2.lookups == 100
    s = X.read_cli("-s small -G hash -h 500")
    assert s.n_isotopes == 68 and s.grid_type == 2 and s.hash_bins == 500
    xl = X.read_cli("-s XL")
    assert xl.n_gridpoints == 238847
    xxl = X.read_cli("-s XXL")
    assert xxl.n_gridpoints == int(238847 * 2.1)
    g = X.read_cli("-s XL -g 5000")
    assert g.n_gridpoints == 5000


@pytest.mark.parametrize("args", ["-t 0", "-l 0", "-s medium", "-G foo", "-m foo", "-b x",
                                  "-q", "-t"])
def test_read_cli_errors(args):
    with pytest.raises(X.XSError) as e:
        X.read_cli(args)
    assert e.value.status == 1


def test_grid_init_rejects_bad_inputs():
    inp = product_inputs("tiny_unionized")
    inp.n_isotopes = 100   # the material lists need 68 or >= 355 nuclides
    with pytest.raises(X.XSError):
        X.grid_init(inp)
    inp = product_inputs("tiny_unionized")
    inp.n_gridpoints = 1
    with pytest.raises(X.XSError):
        X.grid_init(inp)
