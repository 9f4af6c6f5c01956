"""Full-size checks (minutes; opt in with LBM_FULLSIZE=1).

* 256^3 FP32 and FP64, nu = 0.0089, lid 0.05, N(0, 1e-4) seeded noise, 1000
  iterations: the whole F buffer against the CPU oracle (OpenMP), bit for bit
  and within 1e-5 / 1e-12.
* 512^3: size-independent properties -- kernel variants agree bit for bit
  (FP64 sums of the state), runs are deterministic, the state stays finite.
"""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("LBM_FULLSIZE") != "1", reason="set LBM_FULLSIZE=1")]

TOL = {"f32": 1e-5, "f64": 1e-12}


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_256_cube_1000_iterations_against_oracle(capi, oracle, prec):
    dim, steps = 256, 1000
    o = oracle.OracleLattice(dim, 0.0089, 0.05, prec, None, seed=1234, noise_sigma=1e-4)
    with capi.Lattice(dim, 0.0089, 0.05, precision="fp32" if prec == "f32" else "fp64", stride=0, seed=1234,
                      noise_sigma=1e-4) as L:
        L.step(steps, every=steps)
        g = L.f()
        rho, u = L.rho(), L.u()
    o.step(steps, every=steps)
    ref = o.state
    gn, rn = np.isnan(g), np.isnan(ref)
    assert np.array_equal(gn, rn)
    d = np.abs(g[~gn].astype(np.float64) - ref[~rn].astype(np.float64)).max()
    assert d <= TOL[prec], d
    w = np.uint32 if prec == "f32" else np.uint64
    assert np.array_equal(g.view(w), ref.view(w)), "not bit-identical"
    assert np.array_equal(rho.view(w), o.rho.view(w)) and np.array_equal(u.view(w), o.u.view(w))


@pytest.mark.parametrize("prec,variants", [("fp32", ("narrow", "direct", "staged")),
                                           ("fp16", ("direct", "narrow", "staged")),
                                           ("bf16", ("direct", "narrow"))])
def test_512_cube_variants_agree(capi, prec, variants):
    sums = []
    for k in variants:
        with capi.Lattice(512, 0.005, 0.08, precision=prec, seed=1234, noise_sigma=1e-4, kernel=k) as L:
            L.step(30)
            L.sync()
            sums.append(L.reduce())
    for s in sums[1:]:
        assert s == sums[0]
    assert np.isfinite(sums[0][0]) and abs(sums[0][0] / sums[0][2] - 1.0) < 1e-3


def test_512_cube_deterministic(capi):
    out = []
    for _ in range(2):
        with capi.Lattice(512, 0.005, 0.08, precision="fp16", seed=9, noise_sigma=1e-4) as L:
            L.step(50)
            out.append(L.reduce())
    assert out[0] == out[1]
