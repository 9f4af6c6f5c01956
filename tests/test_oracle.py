"""The CPU oracle pinned against the reference (CPU only).

* bit-exact against the digests of the reference's own kernels.cl run
  (tests/golden/ref_runs.json, made by tests/golden/make_golden.py);
* against the reference's golden Sailfish VTI data (verify.py metrics);
* live against oracle/_ref when it is built here;
* its noise generator: Philox4x32-10 known answers, the logarithm, moments.
"""
import ctypes
import hashlib
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _runs():
    with open(os.path.join(GOLD, "ref_runs.json")) as fh:
        return json.load(fh)


def _lids():
    return dict(np.load(os.path.join(GOLD, "lid_profiles.npz")))


@pytest.mark.parametrize("name", sorted(_runs().keys()))
def test_oracle_bit_exact_vs_reference_kernel(oracle, name):
    run = _runs()[name]
    dim, prec, stride, visc, vel, lidkey, iters, every, dig_every = run["spec"]
    lid = _lids()[lidkey] if lidkey else None
    L = oracle.OracleLattice(dim, visc, vel, prec, stride, lid=lid, threads=2)
    assert sha(L.map) == run["map"]
    d = run["digests"]
    assert [sha(L.state), sha(L.rho), sha(L.u)] == d["0"]
    for it in range(1, iters + 1):
        L.step(1, every=every)
        if str(it) in d:
            got = [sha(L.state), sha(L.rho), sha(L.u)]
            assert got == d[str(it)], f"{name}: iteration {it} differs from the reference kernel"


def test_oracle_full_f_ldc8(oracle):
    g = np.load(os.path.join(GOLD, "ref_f8_f32.npz"))
    L = oracle.OracleLattice(8, 0.0089, 0.05, "f32", 8, threads=1)
    np.testing.assert_array_equal(L.state.view(np.uint32), g["f_0"].view(np.uint32))
    for it in range(1, 11):
        L.step(1, every=1)
        if f"f_{it}" in g:
            np.testing.assert_array_equal(L.state.view(np.uint32), g[f"f_{it}"].view(np.uint32))


def _verify(dim, oracle_lat, gold, steps, every):
    from lbmcl_gb300 import vti
    worst = {}
    it = 0
    for target in steps:
        oracle_lat.step(target - it, every=every)
        it = target
        pred = vti.interior_fields(dim, oracle_lat.rho, oracle_lat.u)
        c = vti.compare({"rho": gold[f"rho_{target}"], "v": gold[f"v_{target}"]}, pred)
        for k, v in c.items():
            worst[k] = max(worst.get(k, 0.0), v)
    return worst


def test_oracle_vs_sailfish_8(oracle):
    """make test8 (Makefile:73-78): 8^3, 10 iterations, every 1."""
    gold = np.load(os.path.join(GOLD, "sailfish_ldc8.npz"))
    L = oracle.OracleLattice(8, 0.0089, 0.05, "f32", 8)
    w = _verify(8, L, gold, list(range(0, 11)), 1)
    assert w["mae_rho"] < 2e-6 and w["mae_v"] < 1e-6, w
    assert w["mse_rho"] < 1e-12 and w["mse_v"] < 1e-12, w


def test_oracle_vs_sailfish_32(oracle):
    """make test32 (Makefile:81-86): 32^3, 500 iterations, every 20."""
    gold = np.load(os.path.join(GOLD, "sailfish_ldc32.npz"))
    L = oracle.OracleLattice(32, 0.0089, 0.05, "f32", 32)
    w = _verify(32, L, gold, [20, 500], 20)
    assert w["mae_rho"] < 5e-6 and w["mae_v"] < 2e-6, w
    assert w["mse_rho"] < 1e-11 and w["mse_v"] < 1e-12, w


def test_sailfish_order_is_closer_to_the_sailfish_data(oracle):
    """The compiled-out Sailfish summation order (kernels.cl:352-354,
    368-375) against the golden Sailfish runs: closer than the reference's
    active order at both sizes (not bit-equal: Sailfish's collision is
    evaluated in its own order too)."""
    for dim, steps, every, name, lim in [(8, list(range(0, 11)), 1, "sailfish_ldc8.npz", (4e-7, 2e-7)),
                                         (32, [20, 500], 20, "sailfish_ldc32.npz", (2e-6, 5e-7))]:
        gold = np.load(os.path.join(GOLD, name))
        ws = _verify(dim, oracle.OracleLattice(dim, 0.0089, 0.05, "f32", dim, order="sailfish"), gold, steps, every)
        wr = _verify(dim, oracle.OracleLattice(dim, 0.0089, 0.05, "f32", dim), gold, steps, every)
        assert ws["mae_rho"] < lim[0] and ws["mae_v"] < lim[1], (dim, ws)
        assert ws["mae_rho"] <= wr["mae_rho"] and ws["mae_v"] <= wr["mae_v"], (dim, ws, wr)
        assert ws["mse_rho"] < wr["mse_rho"], (dim, ws, wr)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_vs_ref_live(oracle, prec):
    if not oracle.ref_available(prec):
        pytest.skip("oracle/_ref not built (needs the reference tree)")
    rng = np.random.default_rng(5)
    lid = 0.04 + 0.02 * rng.random(16 * 16)
    a = oracle.OracleLattice(16, 0.02, 0.07, prec, 32, lid=lid, threads=3)
    b = oracle.RefLattice(16, 0.02, 0.07, prec, 32, lid=lid)
    for it in range(6):
        a.step(1, every=2)
        b.step(1, every=2)
        w = np.uint32 if prec == "f32" else np.uint64
        np.testing.assert_array_equal(a.state.view(w), b.state.view(w))
        np.testing.assert_array_equal(a.rho.view(w), b.rho.view(w))
        np.testing.assert_array_equal(a.u.view(w), b.u.view(w))


def test_cell_types_match_reference_rules(oracle):
    dim = 8
    ct = oracle.cell_types(dim).reshape(dim, dim, dim)
    assert (ct[0] == oracle.WALL).all() and (ct[:, :, -1] == oracle.WALL).all()
    assert ct[1, 1, 1] == oracle.CORNER and ct[1, dim - 2, dim - 2] == oracle.CORNER
    # the FRONT corners are not CORNER (kernels.cl:254-260 lists BACK corners only)
    assert ct[dim - 2, 1, 1] == (oracle.LEFT | oracle.BOTTOM | oracle.FRONT)
    assert ct[dim - 2, 3, 3] == (oracle.FRONT | oracle.MOVING)
    assert ct[3, 3, 3] == oracle.FLUID
    assert ct[dim - 2, 1, 3] == (oracle.FRONT | oracle.BOTTOM)


def test_philox_known_answers(oracle):
    """Philox4x32-10 known-answer vectors of the Random123 distribution."""
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_series_log_accuracy(oracle):
    """The single-precision logarithm of the noise generator (IEEE + - * /
    only) against the library logarithm, over the float range."""
    L = oracle.lib()
    L.lbmo_logf.argtypes = [ctypes.c_float]
    L.lbmo_logf.restype = ctypes.c_float
    xs = np.concatenate([np.geomspace(1e-38, 1.0, 3000), np.linspace(0.01, 0.9999, 3000),
                         [1.5e-45, 1e-40, 1.0, 2.0, 3.0e38]]).astype(np.float32)
    for x in xs:
        got = L.lbmo_logf(float(x))
        ref = math.log(float(x))
        assert abs(got - ref) <= 2.5e-7 * max(1.0, abs(ref)), (x, got, ref)


def test_gauss_moments(oracle):
    z = np.array([oracle.gauss(1234, s, q) for s in range(4000) for q in range(5)])
    assert abs(z.mean()) < 0.03
    assert abs(z.var() - 1.0) < 0.04
    assert abs((z ** 4).mean() - 3.0) < 0.25
    stats = pytest.importorskip("scipy.stats")
    assert stats.kstest(z, "norm").pvalue > 1e-3
    # deterministic and keyed by all of (seed, site, q)
    assert oracle.gauss(1, 2, 3) == oracle.gauss(1, 2, 3)
    assert len({oracle.gauss(1, 2, 3), oracle.gauss(2, 2, 3), oracle.gauss(1, 3, 3), oracle.gauss(1, 2, 4)}) == 4


def test_noise_only_on_fluid(oracle):
    a = oracle.OracleLattice(12, 0.0089, 0.05, "f64", 8, seed=99, noise_sigma=1e-4)
    b = oracle.OracleLattice(12, 0.0089, 0.05, "f64", 8)
    fa = a.f_soa()
    fb = b.f_soa()
    fluid = (a.map == oracle.FLUID).reshape(12, 12, 12)
    d = np.nan_to_num(fa - fb)
    assert np.all(d[:, ~fluid] == 0)
    assert 0.5e-4 < d[:, fluid].std() < 1.5e-4
