"""Parity of the sm_103a library (through the C ABI) with the CPU oracle.

Bars: max |df| <= 1e-5 in FP32 and <= 1e-12 in FP64 against the
oracle on identical inputs, lattice map bit-exact.  The FP32 / FP64 kernels
evaluate every expression in the reference's operand order without FMA
contraction, so they are also checked for bit-for-bit equality.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {"f32": 1e-5, "f64": 1e-12}
GPU_PREC = {"f32": "fp32", "f64": "fp64"}


def assert_f_close(gpu, ref, tol, what=""):
    assert gpu.shape == ref.shape
    gn, rn = np.isnan(gpu), np.isnan(ref)
    assert np.array_equal(gn, rn), f"{what}: NaN positions differ ({(gn != rn).sum()} slots)"
    d = np.abs(gpu[~gn].astype(np.float64) - ref[~rn].astype(np.float64))
    assert d.size == 0 or d.max() <= tol, f"{what}: max |df| = {d.max():.3e} > {tol}"


def bits(a):
    return a.view(np.uint32 if a.dtype == np.float32 else np.uint64)


@pytest.mark.parametrize("dim", [4, 8, 12, 16, 32])
def test_map_bit_exact(capi, oracle, dim):
    with capi.Lattice(dim, precision="fp32", stride=0) as L:
        np.testing.assert_array_equal(L.cell_map(), oracle.cell_types(dim))


@pytest.mark.parametrize("kernel", ["direct", "staged", "aa"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim,stride", [(8, 8), (32, 8), (16, 1), (16, 4096), (4, 4), (12, 16)])
def test_f_after_each_step(capi, oracle, prec, dim, stride, kernel):
    """Config 1 shape (32^3, stride 8, 10 steps) and layout / size variations:
    the full post-stream buffer, wall slots included, after every iteration,
    for the iteration-kernel variants (the in-place AA one in both of its
    layouts)."""
    o = oracle.OracleLattice(dim, 0.0089, 0.05, prec, stride)
    with capi.Lattice(dim, 0.0089, 0.05, precision=GPU_PREC[prec], stride=stride, kernel=kernel) as L:
        assert_f_close(L.f(), o.state, TOL[prec], "initial")
        for it in range(1, 11):
            o.step(1, every=1)
            L.step(1, every=1)
            g = L.f()
            assert_f_close(g, o.state, TOL[prec], f"iteration {it}")
            assert np.array_equal(bits(g), bits(o.state)), f"iteration {it}: not bit-identical"
            np.testing.assert_array_equal(bits(L.rho()), bits(o.rho))
            np.testing.assert_array_equal(bits(L.u()), bits(o.u))


@pytest.mark.parametrize("kernel", ["direct", "narrow", "staged", "aa"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_sailfish_order(capi, oracle, prec, kernel):
    """The Sailfish summation order of rho and u (kernels.cl:352-354,
    368-375; compiled out in the reference) against the oracle's, bit for
    bit, with a lid profile, noise and macro output; it differs from the
    reference order's run, and its reductions follow it too."""
    if prec == "f64" and kernel == "narrow":
        pytest.skip("no narrow FP64 variant")
    rng = np.random.default_rng(5)
    dim = 24
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    kw = dict(lid=lid, seed=99, noise_sigma=1e-4)
    o = oracle.OracleLattice(dim, 0.01, 0.05, prec, 8, order="sailfish", **kw)
    r = oracle.OracleLattice(dim, 0.01, 0.05, prec, 8, **kw)
    with capi.Lattice(dim, 0.01, 0.05, precision=GPU_PREC[prec], stride=8, kernel=kernel, order="sailfish",
                      **kw) as L:
        for chunk in (1, 5, 34):
            o.step(chunk, every=chunk)
            r.step(chunk, every=chunk)
            L.step(chunk, every=chunk)
            g = L.f()
            assert np.array_equal(bits(g), bits(o.state)), f"after {o.it}: not bit-identical"
            np.testing.assert_array_equal(bits(L.rho()), bits(o.rho))
            np.testing.assert_array_equal(bits(L.u()), bits(o.u))
        assert not np.array_equal(bits(o.state), bits(r.state))
        # the reduction forms the moments of the current state, which the
        # next iteration stores
        m = L.reduce()[0]
    o.step(1, every=1)
    rho = o.rho[~np.isnan(o.rho)].astype(np.float64)
    assert abs(m - rho.sum()) <= 1e-12 * rho.sum()


def test_sailfish_order_refuses_the_adjoint(capi):
    with capi.Lattice(16, precision="fp32", order="sailfish") as L:
        L.adjoint_set_loss(8, np.zeros(16 * 16))
        with pytest.raises(capi.LbmError, match="summation order"):
            L.adjoint_forward(4, 2)


@pytest.mark.parametrize("kernel", ["direct", "staged", "aa"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_lid_profile_noise_and_macro_every(capi, oracle, prec, kernel):
    """Per-column lid, seeded noise on FLUID populations, macros every 3rd
    iteration; 60 iterations at 24^3 with block-size and stride changes."""
    rng = np.random.default_rng(11)
    dim = 24
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    o = oracle.OracleLattice(dim, 0.01, 0.05, prec, 64, lid=lid, seed=1234, noise_sigma=1e-4)
    with capi.Lattice(dim, 0.01, 0.05, precision=GPU_PREC[prec], stride=64, lid=lid, seed=1234,
                      noise_sigma=1e-4, block_threads=96, kernel=kernel) as L:
        assert np.array_equal(bits(L.f()), bits(o.state)), "initial state (noise) differs"
        for chunk in (1, 2, 7, 20, 30):
            o.step(chunk, every=3)
            L.step(chunk, every=3)
            g = L.f()
            assert_f_close(g, o.state, TOL[prec], f"after {o.it}")
            assert np.array_equal(bits(g), bits(o.state))
            np.testing.assert_array_equal(bits(L.rho()), bits(o.rho))
            np.testing.assert_array_equal(bits(L.u()), bits(o.u))
        assert L.iteration == o.it == 60


def test_golden_sailfish_8_and_32(capi):
    """make test8 / make test32 through the library against the reference's
    golden data (verify.py metrics)."""
    from lbmcl_gb300 import vti
    g8 = np.load(os.path.join(GOLD, "sailfish_ldc8.npz"))
    with capi.Lattice(8, precision="fp32", stride=8) as L:
        for it in range(0, 11):
            if it:
                L.step(1, every=1)
            c = vti.compare({"rho": g8[f"rho_{it}"], "v": g8[f"v_{it}"]}, vti.interior_fields(8, L.rho(), L.u()))
            assert c["mae_rho"] < 2e-6 and c["mae_v"] < 1e-6, (it, c)
    g32 = np.load(os.path.join(GOLD, "sailfish_ldc32.npz"))
    with capi.Lattice(32, precision="fp32", stride=32) as L:
        done = 0
        for it in (20, 500):
            L.step(it - done, every=20)
            done = it
            c = vti.compare({"rho": g32[f"rho_{it}"], "v": g32[f"v_{it}"]}, vti.interior_fields(32, L.rho(), L.u()))
            assert c["mae_rho"] < 5e-6 and c["mae_v"] < 2e-6, (it, c)


@pytest.mark.parametrize("kernel", ["direct", "staged", "aa"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_64cube_200_steps(capi, oracle, prec, kernel):
    o = oracle.OracleLattice(64, 0.0089, 0.05, prec, 64, seed=7, noise_sigma=1e-4)
    with capi.Lattice(64, 0.0089, 0.05, precision=GPU_PREC[prec], stride=64, seed=7, noise_sigma=1e-4,
                      kernel=kernel) as L:
        o.step(200, every=100)
        L.step(200, every=100)
        g = L.f()
        assert_f_close(g, o.state, TOL[prec], "64^3 x 200")
        assert np.array_equal(bits(g), bits(o.state))


@pytest.mark.parametrize("kernel,steps", [("auto", 5), ("aa", 5), ("aa", 6)])
@pytest.mark.parametrize("prec", ["fp32", "fp64", "fp16", "bf16"])
def test_load_dump_round_trip(capi, prec, kernel, steps):
    """F dump / load and raw dump / load round trips (the in-place AA lattice
    in both of its layouts)."""
    with capi.Lattice(16, precision=prec, stride=16, seed=3, noise_sigma=1e-4, kernel=kernel) as L:
        L.step(steps)
        f0 = L.f()
        raw = L.raw()
        L.load_f(f0)
        f1 = L.f()
        np.testing.assert_array_equal(np.isnan(f0), np.isnan(f1))
        if prec in ("fp32", "fp64"):
            np.testing.assert_array_equal(bits(f0), bits(f1))
        else:
            assert np.nanmax(np.abs(f1 - f0)) < 1e-6
        L.load_raw(raw)
        np.testing.assert_array_equal(L.raw(), raw)


@pytest.mark.parametrize("kernel,pre", [("auto", 0), ("aa", 0), ("aa", 1)])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_load_then_continue(capi, oracle, prec, kernel, pre):
    """A state loaded from the host continues exactly like the oracle (into
    an AA lattice in either layout)."""
    o = oracle.OracleLattice(16, 0.0089, 0.05, prec, 8, seed=5, noise_sigma=1e-4)
    o.step(7, every=0)
    with capi.Lattice(16, 0.0089, 0.05, precision=GPU_PREC[prec], stride=8, kernel=kernel) as L:
        L.step(pre)
        L.load_f(o.state)
        assert np.array_equal(bits(L.f()), bits(o.state))
        o.step(5, every=5)
        L.step(5, every=5)
        assert np.array_equal(bits(L.f()), bits(o.state))


@pytest.mark.parametrize("kernel,steps", [("auto", 25), ("aa", 25), ("aa", 24)])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reduce_matches_oracle_moments(capi, oracle, prec, kernel, steps):
    dim = 32
    o = oracle.OracleLattice(dim, 0.0089, 0.05, prec, 32, seed=1, noise_sigma=1e-4)
    with capi.Lattice(dim, 0.0089, 0.05, precision=GPU_PREC[prec], stride=32, seed=1, noise_sigma=1e-4,
                      kernel=kernel) as L:
        o.step(steps, every=0)
        L.step(steps, every=0)
        mass, energy, count = L.reduce()
    # the moments of the current state are what the next iteration stores
    o.step(1, every=1)
    sm = (o.map == oracle.FLUID) | ((o.map & oracle.MOVING) != 0)
    r = o.rho[sm].astype(np.float64)
    u = o.u.reshape(3, -1)[:, sm].astype(np.float64)
    m_ref = r.sum()
    e_ref = (0.5 * r * (u ** 2).sum(0)).sum()
    assert count == sm.sum()
    assert abs(mass - m_ref) <= 1e-12 * m_ref
    assert abs(energy - e_ref) <= 1e-9 * e_ref


def test_sixteen_bit_storage_close_to_fp64(capi):
    """FP16 / BF16 deviation storage against the FP64 run, same seed."""
    dim, steps = 32, 300
    kw = dict(viscosity=0.005, velocity=0.08, stride=32, seed=9, noise_sigma=1e-4)
    with capi.Lattice(dim, precision="fp64", **kw) as R:
        R.step(steps, every=steps)
        u64 = R.u().reshape(3, dim, dim, dim)
        r64 = R.rho()
    errs = {}
    for prec in ("fp16", "bf16", "fp32"):
        with capi.Lattice(dim, precision=prec, **kw) as L:
            L.step(steps, every=steps)
            u = L.u().reshape(3, dim, dim, dim).astype(np.float64)
            r = L.rho().astype(np.float64)
        fluid = ~np.isnan(u64[0])
        mid = u64[0, :, dim // 2, :]
        e_mid = np.linalg.norm(np.nan_to_num(u[0, :, dim // 2, :] - mid)) / np.linalg.norm(np.nan_to_num(mid))
        e_rho = np.nanmax(np.abs(r - r64))
        errs[prec] = (e_mid, e_rho)
        assert np.isfinite(u[:, fluid]).all()
    assert errs["fp32"][0] < 1e-5
    assert errs["fp16"][0] < 1e-3, errs
    assert errs["bf16"][0] < 2e-2, errs


def test_divergence_is_reported(capi):
    """An unstable run (tau near 0.5, lid near the lattice sound speed) makes
    densities non-finite; lbm_sync reports it as EDIVERGED."""
    with capi.Lattice(16, viscosity=0.0, velocity=0.6, precision="fp32") as L:
        L.step(400)
        with pytest.raises(capi.LbmError) as e:
            L.sync()
        assert e.value.code == capi.EDIVERGED


def test_timing_and_iteration_counters(capi):
    with capi.Lattice(32, precision="fp32", profile_steps=True) as L:
        L.step(10)
        L.step(5, every=5)
        tot, ker = L.timing()
        assert L.iteration == 15
        assert tot > 0 and 0 < ker <= tot


def test_deterministic_repeat(capi):
    outs = []
    for _ in range(2):
        with capi.Lattice(48, precision="fp16", seed=4, noise_sigma=1e-4) as L:
            L.step(40)
            outs.append(L.raw())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("prec", ["fp32", "fp64", "fp16", "bf16"])
@pytest.mark.parametrize("dim,stages", [(8, 2), (24, 3), (64, 0), (136, 5), (256, 0)])
def test_kernel_variants_agree(capi, prec, dim, stages):
    """The iteration kernels move data differently but run the same site
    update: their populations and macros agree bit for bit."""
    outs = []
    for kernel in ("direct", "staged", "narrow", "aa"):
        with capi.Lattice(dim, 0.005, 0.08, precision=prec, seed=21, noise_sigma=1e-4, kernel=kernel,
                          stages=stages) as L:
            L.step(7)
            L.step(6, every=6)
            L.sync()
            outs.append((L.f(), L.rho(), L.u()))
    # the F view; the raw buffers may differ at wall sites, whose slots no
    # iteration or dump ever reads
    for other in outs[1:]:
        np.testing.assert_array_equal(bits(outs[0][0]), bits(other[0]))
        np.testing.assert_array_equal(bits(outs[0][1]), bits(other[1]))
        np.testing.assert_array_equal(bits(outs[0][2]), bits(other[2]))


@pytest.mark.parametrize("prec", ["fp32", "fp16", "fp64"])
@pytest.mark.parametrize("nsteps,every", [(50, 0), (37, 20), (40, 7), (70, 33)])
def test_graph_replay_matches_direct_launches(capi, prec, nsteps, every):
    """lbm_step replays captured CUDA graphs of 16 plain iterations (one per
    starting buffer parity); runs split by macro iterations fall back to
    direct launches.  The state, rho and u equal those of direct launches
    bit for bit, from both parities."""
    res = []
    for g in (0, 1, 4):  # default 16 per graph, no graphs, 4 per graph
        with capi.Lattice(32, 0.0089, 0.05, precision=prec, stride=8, seed=3, noise_sigma=1e-4,
                          graph_iterations=g) as L:
            L.step(5, every=every)          # odd parity first
            L.step(nsteps, every=every)
            L.step(16)                      # an exact graph run at the end
            res.append((L.f(), L.rho(), L.u()))
    for r in res[1:]:
        for a, b in zip(res[0], r):
            np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("prec,kernel", [("fp32", "direct"), ("fp32", "staged"), ("fp16", "narrow"),
                                         ("fp16", "staged"), ("bf16", "direct"), ("fp32", "aa"), ("fp16", "aa"),
                                         ("fp64", "aa")])
def test_graph_replay_every_kernel_variant(capi, prec, kernel):
    """Graph replay of each iteration-kernel variant (the staged one with its
    mbarrier ring and dynamic shared memory) equals its direct launches."""
    res = []
    for g in (0, 1):
        with capi.Lattice(48, 0.0089, 0.05, precision=prec, stride=0, seed=4, noise_sigma=1e-4, kernel=kernel,
                          graph_iterations=g) as L:
            L.step(3)
            L.step(40, every=40)
            res.append((L.f(), L.rho(), L.u()))
    for a, b in zip(*res):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16", "fp64"])
@pytest.mark.parametrize("dim", [8, 40, 136])
def test_in_place_variant_matches_two_lattices_every_step(capi, prec, dim):
    """The AA lattice (one buffer, alternating local and neighbour steps)
    against the default two-lattice kernels after every iteration of both
    kinds, macro iterations included: bit for bit.  dim 136 gives rows that
    start inside a warp (17 vectors of 8 sites)."""
    outs = {}
    for kernel in ("auto", "aa"):
        res = []
        with capi.Lattice(dim, 0.005, 0.08, precision=prec, seed=13, noise_sigma=1e-4, kernel=kernel,
                          graph_iterations=1) as L:
            res.append(L.f())
            for it in range(1, 8):
                L.step(1, every=3)
                res.append((L.f(), L.rho(), L.u()))
        outs[kernel] = res
    np.testing.assert_array_equal(bits(outs["auto"][0]), bits(outs["aa"][0]))
    for a, b in zip(outs["auto"][1:], outs["aa"][1:]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(bits(x), bits(y))


def test_in_place_variant_memory_and_adjoint_refusal(capi):
    """The AA handle holds one population lattice (its budget check counts
    one), and the gradient calls refuse it with a status and a message."""
    import ctypes as C
    dim = 32
    fbytes = 19 * dim ** 3 * 4
    with capi.Lattice(dim, precision="fp32", kernel="aa") as L:
        L.adjoint_set_loss(16, None)
        J = C.c_double()
        assert capi.lib().lbm_adjoint_forward(L.h, 4, 4, C.byref(J)) == capi.ESTATE
        assert "two-lattice" in capi.lib().lbm_last_error().decode()
        L.step(3)
        L.sync()
    # a budget between the one-lattice and the two-lattice needs: only AA fits
    n = dim ** 3
    nvec = (dim // 4) * (dim - 2) ** 2
    two = (2 * fbytes + n + 16 * n + dim * dim * 4 + min(1 << 25, 19 * n) * 4 + (-(-nvec // 128) + 2) * 16 +
           4 * 8 + 4)  # lbm_init's need of a two-lattice FP32 handle
    with pytest.raises(capi.LbmError):
        capi.Lattice(dim, precision="fp32", max_device_bytes=two - fbytes // 2)
    with capi.Lattice(dim, precision="fp32", kernel="aa", max_device_bytes=two - fbytes // 2) as L:
        L.step(2)
        L.sync()
