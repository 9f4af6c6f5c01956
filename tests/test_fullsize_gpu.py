"""Largest-size checks (minutes and ~100 GB of host memory; opt in with
LBM_FULLSIZE=1).  The 256^3 x 1000 parity runs are always on
(tests/test_config_gpu.py).

* 512^3: size-independent properties -- kernel variants agree bit for bit
  (FP64 sums of the state), runs are deterministic, the state stays finite.
* 640^3 FP32 (19 dim^3 > 2^32 population offsets): two iterations bit for
  bit against the oracle.
"""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("LBM_FULLSIZE") != "1", reason="set LBM_FULLSIZE=1")]

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


def _host_mem_available() -> float:
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return float(line.split()[1]) * 1024
    except OSError:
        pass
    return 0.0


def test_offsets_beyond_32_bits_against_oracle(capi, oracle):
    """dim 640: 19 dim^3 = 4.98e9 population offsets exceed 2^32 (the largest
    sizes).  Two FP32 iterations with seeded noise, the whole F buffer and the
    moments bit for bit against the oracle; compared in chunks to bound host
    memory (two 20 GB buffers)."""
    if _host_mem_available() < 100e9:
        pytest.skip("needs ~100 GB of host memory")
    dim, steps = 640, 2
    stride = 1 << 21  # the largest power of two dividing 640^3 = 2^21 * 125: CSoA blocks of 2^21 sites
    assert 19 * dim ** 3 > 2 ** 32
    o = oracle.OracleLattice(dim, 0.0089, 0.05, "f32", stride, seed=77, noise_sigma=1e-4)
    o.step(steps, every=steps)
    with capi.Lattice(dim, 0.0089, 0.05, precision="fp32", stride=stride, seed=77, noise_sigma=1e-4) as L:
        L.step(steps, every=steps)
        g = L.f()
        rho, u = L.rho(), L.u()
    ref = o.state
    chunk = 1 << 28
    for s0 in range(0, g.size, chunk):
        a, b = g[s0:s0 + chunk], ref[s0:s0 + chunk]
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"F differs in [{s0}, {s0 + chunk})"
    assert np.array_equal(rho.view(np.uint32), o.rho.view(np.uint32))
    assert np.array_equal(u.view(np.uint32), o.u.view(np.uint32))
