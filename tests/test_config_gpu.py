"""The specified cavities at full size, through the C ABI.

* 256^3 FP32 and FP64, nu = 0.0089, lid 0.05, N(0, 1e-4) seeded noise, 1000
  iterations (the plain-precision cavity the throughput is quoted on): the
  whole F buffer, rho and u against the CPU oracle (OpenMP), within the
  specified 1e-5 (FP32) / 1e-12 (FP64) and bit for bit.  The reference path:
  kernels.cl:321-425 driven by lbmcl.hpp:505-520.
* the 512^3 cavity's physics (nu = 0.005, lid u = 0.08, seeded N(0, 1e-4)
  noise) at 128^3 x 1000 iterations: FP16 and BF16 deviation storage against
  the FP64 run of the same seed; FP16 keeps the mid-plane u_x within 1e-3
  relative L2 (BF16, 8-bit mantissa, within 2e-2).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f64": 1e-12}


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_256_cube_1000_iterations_against_oracle(capi, oracle, prec):
    dim, steps = 256, 1000
    with capi.Lattice(dim, 0.0089, 0.05, precision="fp32" if prec == "f32" else "fp64", stride=0, seed=1234,
                      noise_sigma=1e-4) as L:
        L.step(steps, every=steps)
        g = L.f()
        rho, u = L.rho(), L.u()
    o = oracle.OracleLattice(dim, 0.0089, 0.05, prec, None, seed=1234, noise_sigma=1e-4)
    o.step(steps, every=steps)
    ref = o.state
    gn, rn = np.isnan(g), np.isnan(ref)
    assert np.array_equal(gn, rn)
    d = np.abs(g[~gn].astype(np.float64) - ref[~rn].astype(np.float64)).max()
    assert d <= TOL[prec], d
    w = np.uint32 if prec == "f32" else np.uint64
    assert np.array_equal(g.view(w), ref.view(w)), "not bit-identical"
    assert np.array_equal(rho.view(w), o.rho.view(w)) and np.array_equal(u.view(w), o.u.view(w))


def _moments_after(capi, prec, dim, steps):
    """rho, u (FP64 copies) that iteration `steps` stores, i.e. of the state
    after steps - 1 iterations, for the 512^3 cavity's physics."""
    with capi.Lattice(dim, 0.005, 0.08, precision=prec, stride=0, seed=1234, noise_sigma=1e-4) as L:
        L.step(steps - 1)
        L.step(1, every=steps)
        L.sync()
        return L.rho().astype(np.float64), L.u().astype(np.float64).reshape(3, dim, dim, dim)


def test_sixteen_bit_storage_accuracy_at_the_512_cube_physics(capi):
    dim, steps = 128, 1000
    rho64, u64 = _moments_after(capi, "fp64", dim, steps)
    ok = np.isfinite(rho64)
    mid = dim // 2
    ref_mid = u64[0, :, mid, :]
    m = np.isfinite(ref_mid)
    assert np.linalg.norm(ref_mid[m]) > 0
    limits = {"fp16": 1e-3, "bf16": 2e-2}
    errs = {}
    for prec, lim in limits.items():
        rho, u = _moments_after(capi, prec, dim, steps)
        assert np.isfinite(rho[ok]).all() and np.isfinite(u.reshape(3, -1)[:, ok]).all()
        um = u[0, :, mid, :]
        errs[prec] = float(np.linalg.norm(um[m] - ref_mid[m]) / np.linalg.norm(ref_mid[m]))
        assert np.abs(rho[ok] - rho64[ok]).max() < 1e-2
    for prec, lim in limits.items():
        assert errs[prec] <= lim, errs
    # FP16 (11-bit mantissa of s (f - w)) is closer than BF16
    assert errs["fp16"] < errs["bf16"], errs
