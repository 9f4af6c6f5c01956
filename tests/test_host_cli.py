"""The lbmcl host program (C++ over the C ABI): the reference's command line,
its output files byte for byte, and make test8 / make test32 against the
reference's golden data."""
import os
import subprocess

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lbmcl_bin():
    from lbmcl_gb300 import build
    build.build_library()
    return build.build_host()


def run(binary, *args, cwd=None):
    return subprocess.run([binary, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=600)


# ---------------------------------------------------------------- CPU ------
def test_help_and_exit_code(lbmcl_bin):
    r = run(lbmcl_bin, "-h")
    assert r.returncode == 1  # lbm_options.hpp:103-122 exits 1
    for flag in ("-d  --dim", "-n  --viscosity", "-u  --velocity", "-i  --iterations", "-e  --every",
                 "-F  --use_double", "-s  --stride", "--precision"):
        assert flag in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["-d", "-3"], "Please enter a valid lattice dimension"),
    (["-i", "-1"], "Please enter a valid number of iterations"),
    (["-n", "-0.1"], "Please enter a valid viscosity value"),
    (["-e", "-2"], "Please enter a valid number for save simulation results every N iterations"),
    (["-s", "-4"], "Please enter a valid number for stride value"),
    (["--precision", "fp8"], "Please enter a valid precision"),
])
def test_rejects_bad_values(lbmcl_bin, args, msg):
    r = run(lbmcl_bin, *args)
    assert r.returncode == 1 and msg in r.stderr


def test_rounds_dim_and_stride_like_the_reference(lbmcl_bin, tmp_path):
    # the messages come from the constructor, before any device work
    r = run(lbmcl_bin, "-d", "12", "-s", "24", "-i", "0", "-e", "0", "-v", tmp_path)
    assert "dim is rounded to the previous power of 2: 8" in r.stdout
    assert "stride is rounded to the previous power of 2: 16" in r.stdout


def test_rejects_oversized_work_group(lbmcl_bin):
    r = run(lbmcl_bin, "-d", "4", "-w", "8,8,8")
    assert r.returncode == 255 and "Please enter a good work_group_size" in r.stderr


# ------------------------------------------- the reference's own writers ------
def _digest_runs():
    import json
    with open(os.path.join(GOLD, "host_digests.json")) as fh:
        return json.load(fh)["runs"]


def test_digests_come_from_the_reference_writers(tmp_path):
    """Where the reference tree was present at build time (oracle/_ref), the
    committed digests are re-derived from the reference's own writers fed
    with the oracle's data (tests/golden/make_host_golden.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_host_golden", os.path.join(GOLD, "make_host_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    if not os.path.exists(mg.LIB):
        pytest.skip("the reference writers are built only where the reference tree is present")
    assert mg.generate()["runs"] == _digest_runs()


# ---------------------------------------------------------------- GPU ------
@pytest.mark.gpu
@pytest.mark.parametrize("k", range(3))
def test_output_files_equal_the_reference_writers(lbmcl_bin, tmp_path, capi, k):
    """For each run (make testall at 8^3 with f and map dumps, an FP64 run
    with f dumps, a 32^3 test32-like run) every file the lbmcl program
    writes has the SHA-256 of the file the reference's own writers
    (lbmcl.hpp:159-334, compiled against an OpenCL stand-in) write for the
    same run, and no file is missing or extra."""
    import hashlib
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_host_golden", os.path.join(GOLD, "make_host_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    entry = _digest_runs()[k]
    r = run(lbmcl_bin, *mg.cli_args(entry["run"], tmp_path, tmp_path))
    assert r.returncode == 0, r.stderr
    got = {f.name: hashlib.sha256(f.read_bytes()).hexdigest() for f in sorted(tmp_path.iterdir())}
    assert sorted(got) == sorted(entry["files"])
    bad = [f for f in got if got[f] != entry["files"][f]]
    assert not bad, bad


@pytest.mark.gpu
def test_make_test8_against_golden(lbmcl_bin, tmp_path, capi):
    """make test8 (Makefile:73-78): the VTI files against the reference's
    golden Sailfish data, with verify.py's metrics."""
    from lbmcl_gb300 import vti
    r = run(lbmcl_bin, "-d", 8, "-n", 0.0089, "-u", 0.05, "-i", 10, "-e", 1, "-w", "8,8,8", "-s", 8,
            "-v", tmp_path)
    assert r.returncode == 0, r.stderr
    g8 = np.load(os.path.join(GOLD, "sailfish_ldc8.npz"))
    for it in range(0, 11):
        got = vti.read_vti(str(tmp_path / f"lbmcl.{it:02d}.vti"))
        c = vti.compare({"rho": g8[f"rho_{it}"], "v": g8[f"v_{it}"]}, got)
        assert c["mae_rho"] < 2e-6 and c["mae_v"] < 1e-6, (it, c)
    assert "Kernels MLUPS:" in r.stdout and r.stderr.count(";") == 11


@pytest.mark.gpu
def test_make_test32_against_golden(lbmcl_bin, tmp_path, capi):
    """make test32 (Makefile:81-86): 500 iterations, every 20, -w 32,32,1 -s 32."""
    from lbmcl_gb300 import vti
    r = run(lbmcl_bin, "-d", 32, "-n", 0.0089, "-u", 0.05, "-i", 500, "-e", 20, "-w", "32,32,1", "-s", 32,
            "-v", tmp_path)
    assert r.returncode == 0, r.stderr
    assert len(list(tmp_path.glob("lbmcl.*.vti"))) == 26
    g = np.load(os.path.join(GOLD, "sailfish_ldc32.npz"))
    for it in (20, 500):
        got = vti.read_vti(str(tmp_path / f"lbmcl.{it:03d}.vti"))
        c = vti.compare({"rho": g[f"rho_{it}"], "v": g[f"v_{it}"]}, got)
        assert c["mae_rho"] < 5e-6 and c["mae_v"] < 2e-6, (it, c)


@pytest.mark.gpu
def test_sixteen_bit_runs(lbmcl_bin, tmp_path, capi):
    from lbmcl_gb300 import vti
    for p in ("fp16", "bf16"):
        d = tmp_path / p
        d.mkdir()
        r = run(lbmcl_bin, "-d", 32, "-i", 40, "-e", 40, "--precision", p, "--seed", 5, "--noise", 1e-4, "-v", d)
        assert r.returncode == 0, r.stderr
        got = vti.read_vti(str(d / "lbmcl.40.vti"))
        assert np.isfinite(np.nan_to_num(got["rho"], nan=1.0)).all()


# --------------------------------------------------------- binary output ------
def test_binary_vti_round_trip_cpu(tmp_path):
    """write_vti_binary (raw and zlib) reads back to the same arrays as the
    ASCII file of the same fields."""
    from lbmcl_gb300 import vti
    rng = np.random.default_rng(3)
    dim = 10
    for dt in (np.float32, np.float64):
        rho = rng.standard_normal(dim ** 3).astype(dt)
        u = rng.standard_normal(3 * dim ** 3).astype(dt)
        rho[0] = np.nan  # a wall site: outside the interior, never written
        want = vti.interior_fields(dim, rho, u)
        vti.write_vti_ascii(str(tmp_path / "a.vti"), dim, rho, u)
        a = vti.read_vti(str(tmp_path / "a.vti"))
        for comp in (False, True):
            p = tmp_path / f"b{int(comp)}.vti"
            vti.write_vti_binary(str(p), dim, rho, u, compress=comp, block=1000)
            b = vti.read_vti(str(p))
            assert b["extent"] == a["extent"] == (0, dim - 3, 0, dim - 3, 0, dim - 3)
            for name in ("rho", "v"):
                assert b[name].dtype == dt
                np.testing.assert_array_equal(b[name], want[name])
                np.testing.assert_array_equal(b[name], a[name])


def test_read_f_raw_de_indexes_csoa_cpu(tmp_path, oracle):
    from lbmcl_gb300 import vti
    dim, n = 8, 512
    f = np.arange(19 * n, dtype=np.float32).reshape(19, n)
    for stride in (1, 8, 64, n):
        buf = oracle.soa_to_csoa(f.reshape(19, dim, dim, dim), dim, stride)
        buf.astype(np.float32).tofile(tmp_path / "f.raw")
        np.testing.assert_array_equal(vti.read_f_raw(str(tmp_path / "f.raw"), dim, stride), f)


def test_rejects_bad_format(lbmcl_bin):
    r = run(lbmcl_bin, "--format", "hdf5")
    assert r.returncode == 1 and "Please enter a valid format" in r.stderr


@pytest.mark.gpu
def test_binary_format_matches_oracle(lbmcl_bin, oracle, tmp_path, capi):
    """--format binary at 8^3 (-f, every iteration): the raw appended VTI holds
    the oracle's rho, u bit for bit, f_<it>.raw the oracle's f buffer in the
    CSoA layout of the run's stride."""
    from lbmcl_gb300 import vti
    for prec, dt, flag in (("f32", np.float32, []), ("f64", np.float64, ["-F"])):
        d = tmp_path / prec
        d.mkdir()
        r = run(lbmcl_bin, "-d", 8, "-i", 4, "-e", 1, "-s", 8, "-v", d, "-p", d, "-f", "--format", "binary", *flag)
        assert r.returncode == 0, r.stderr
        assert "FORMAT           = binary" in r.stdout
        o = oracle.OracleLattice(8, 0.0089, 0.05, prec, 8)
        for it in range(0, 5):
            if it:
                o.step(1, every=1)
            got = vti.read_vti(str(d / f"lbmcl.{it}.vti"))
            want = vti.interior_fields(8, o.rho, o.u)
            for name in ("rho", "v"):
                assert got[name].dtype == dt
                np.testing.assert_array_equal(got[name], want[name])
        o = oracle.OracleLattice(8, 0.0089, 0.05, prec, 8)
        for it in range(0, 5):
            if it >= 2:  # f_<it> is the buffer iteration it reads: f_0 and f_1 both hold the init state
                o.step(1)
            raw = np.fromfile(d / f"f_{it}.raw", dt)
            np.testing.assert_array_equal(np.nan_to_num(raw, nan=-7.0), np.nan_to_num(o.state, nan=-7.0))
