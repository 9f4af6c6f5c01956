"""The backward sweep without a tau gradient, which recomputes each segment
storing only the adjoint's linearisation point of every iteration (u of the
FLUID sites, rho of the lid sites) instead of full states: the same lid and
initial-population gradients as the full-state sweep, one and two adjoint
steps per launch, graph replay, the fallback when its buffers do not fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(dim, seed):
    rng = np.random.default_rng(seed)
    return 0.05 + 0.01 * rng.standard_normal(dim * dim), 0.02 * rng.standard_normal(dim * dim)


def grads(capi, prec, dim, iters, every, want_tau, **kw):
    # the recompute paths unless a test asks for recorded tail points
    kw.setdefault("adjoint_tail_segments", -1)
    lid, target = case(dim, dim + iters)
    with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=0.53, seed=3, noise_sigma=1e-4, **kw) as L:
        L.adjoint_set_loss(dim // 2, target)
        J = L.adjoint_forward(iters, every)
        return (J,) + tuple(L.adjoint_backward(1.0, want_tau=want_tau))


@pytest.mark.parametrize("prec,steps", [("fp32", 1), ("fp32", 2), ("fp16", 1), ("fp16", 2), ("bf16", 2),
                                        ("fp64", 1)])
@pytest.mark.parametrize("dim,iters,every", [(16, 23, 6), (40, 17, 17)])
def test_point_sweep_matches_full_state_sweep(capi, prec, steps, dim, iters, every):
    """The adjoint linearised at the forward's own moments (the values its
    collision used) against the adjoint that re-forms the moments from the
    stored populations: equal up to the rounding of those moments."""
    J0, t0, l0, f0 = grads(capi, prec, dim, iters, every, True, adjoint_steps=steps)
    J1, t1, l1, f1 = grads(capi, prec, dim, iters, every, False, adjoint_steps=steps)
    assert J0 == J1 and t1 is None
    tol = 1e-10 if prec == "fp64" else 1e-5
    assert np.abs(l1 - l0).max() <= tol * np.abs(l0).max()
    assert np.abs(f1 - f0).max() <= tol * np.abs(f0).max()
    assert np.isfinite(f1).all()


@pytest.mark.parametrize("prec,steps", [("fp32", 2), ("fp16", 2), ("fp64", 1)])
def test_point_sweep_graph_replay_is_exact(capi, prec, steps):
    """Full segments replayed as captured graphs against direct launches, bit
    for bit, and a second sweep reusing the graphs."""
    dim, iters, every = 24, 43, 10
    lid, target = case(dim, 17)
    res = []
    for g in (0, 1):
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=0.53, seed=6, noise_sigma=1e-4,
                          adjoint_steps=steps, graph_iterations=g, adjoint_tail_segments=-1) as L:
            L.adjoint_set_loss(12, target)
            f0 = L.f()
            out = []
            for _ in range(2):
                L.load_f(f0)
                J = L.adjoint_forward(iters, every)
                out.append((J,) + tuple(L.adjoint_backward(1.0, want_tau=False)))
            res.append(out)
    for a, b in zip(res[0], res[1]):
        assert a[0] == b[0]
        np.testing.assert_array_equal(a[2], b[2])
        np.testing.assert_array_equal(a[3], b[3])
    np.testing.assert_array_equal(res[0][0][2], res[0][1][2])


def test_full_states_on_request_and_switching_paths(capi):
    """adjoint_full_states = 1 takes the full-state sweep without a tau
    gradient too (bit for bit the tau-gradient sweep's lid and initial
    gradients); one handle alternating between both sweeps keeps its results."""
    dim, iters, every = 24, 30, 10
    ref = grads(capi, "fp32", dim, iters, every, True, adjoint_steps=1)
    full = grads(capi, "fp32", dim, iters, every, False, adjoint_steps=1, adjoint_full_states=True)
    np.testing.assert_array_equal(full[2], ref[2])
    np.testing.assert_array_equal(full[3], ref[3])
    lid, target = case(dim, dim + iters)
    out = []
    with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53, seed=3, noise_sigma=1e-4,
                      adjoint_steps=1) as L:
        L.adjoint_set_loss(dim // 2, target)
        f0 = L.f()
        # R_0 loaded explicitly each time: no lid dependence through the init
        for want_tau in (False, True, False, True):
            L.load_f(f0)
            L.adjoint_forward(iters, every)
            out.append(L.adjoint_backward(1.0, want_tau=want_tau))
    with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53, adjoint_steps=1) as L:
        L.adjoint_set_loss(dim // 2, target)
        L.load_f(f0)
        L.adjoint_forward(iters, every)
        fresh = L.adjoint_backward(1.0, want_tau=True)
    np.testing.assert_array_equal(out[0][1], out[2][1])
    np.testing.assert_array_equal(out[1][1], out[3][1])
    np.testing.assert_array_equal(out[1][1], fresh[1])
    np.testing.assert_array_equal(out[1][2], fresh[2])


def _init_bytes_fp32(dim, block=128):
    """Device bytes lbm_init takes for an FP32 handle (its budget rule)."""
    n = dim ** 3
    fbytes = 19 * n * 4
    nvec = (dim // 4) * (dim - 2) ** 2
    grid = -(-nvec // block)
    stage = min(1 << 25, 19 * n) * 4
    return 2 * fbytes + n + 4 * n * 4 + dim * dim * 4 + stage + (grid + 2) * 2 * 8 + 4 * 8 + 4


def test_point_sweep_falls_back_when_short_of_memory(capi):
    """With a device budget too small for the stored points (one segment of
    40 iterations: 40 planes sets + 2 state scratch buffers) but enough for
    two state buffers, the sweep takes the full-state path, recursive here
    (every state recomputed from the checkpoint), and gives its gradients."""
    dim, iters, every = 16, 40, 40
    lid, target = case(dim, 31)
    n, nc = dim ** 3, dim * dim
    fbytes = 19 * n * 4
    gi = -(-((dim - 4) ** 2 * (dim // 2)) // 128)
    gf = -(-(4 * (dim - 3) * (dim // 2)) // 128)
    used = (_init_bytes_fp32(dim) + nc * 4 + fbytes + (-(-n // 256) + 1) * 16 + 2 * 19 * n * 4 + nc * 8 +
            (gi + gf) * 8)
    cap = used + int(2.5 * fbytes)
    assert 40 * 3 * n * 4 + 2 * fbytes > cap - used  # the points do not fit
    res = {}
    for budget in (0, cap):
        with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53, adjoint_steps=1,
                          max_device_bytes=budget) as L:
            L.adjoint_set_loss(8, target)
            L.adjoint_forward(iters, every)
            res[budget] = L.adjoint_backward(1.0, want_tau=False)
    assert np.abs(res[cap][1] - res[0][1]).max() <= 1e-5 * np.abs(res[0][1]).max()
    assert np.abs(res[cap][2] - res[0][2]).max() <= 1e-5 * np.abs(res[0][2]).max()


def test_autograd_without_tau_gradient(capi):
    """The autograd harness asks for no tau gradient when tau does not need
    one (the stored-point sweep); lid gradient as the C ABI's."""
    torch = pytest.importorskip("torch")
    from lbmcl_gb300.adjoint import cavity_loss
    dim, iters, plane = 16, 30, 8
    lid0, target = case(dim, 9)
    lid = torch.tensor(lid0.reshape(dim, dim), dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(0.54, dtype=torch.float64)
    J = cavity_loss(lid, tau, None, dim=dim, iterations=iters, plane_y=plane, target=target, checkpoint_every=6,
                    precision="fp64")
    J.backward()
    with capi.Lattice(dim, velocity=0.0, precision="fp64", lid=lid0, tau=0.54) as L:
        L.adjoint_set_loss(plane, target)
        L.adjoint_forward(iters, 6)
        _, g_lid, _ = L.adjoint_backward(1.0, want_f0=False, want_tau=False)
    np.testing.assert_array_equal(lid.grad.numpy(), g_lid)


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("want_tau", [True, False])
def test_fp32_adjoint_equals_fp64_adjoint_of_the_same_trajectory(capi, prec, want_tau):
    """The FP32 adjoint against the FP64-arithmetic adjoint of the same
    trajectory (same storage, same forward, same linearisation points): what
    remains is the FP32 adjoint's own rounding, within 1e-5."""
    dim, iters, every = 32, 300, 30
    lid, target = case(dim, 41)
    res = {}
    for a64 in (False, True):
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=0.53, seed=8, noise_sigma=1e-4,
                          adjoint_fp64=a64) as L:
            L.adjoint_set_loss(dim // 2, target)
            J = L.adjoint_forward(iters, every)
            res[a64] = (J,) + tuple(L.adjoint_backward(1.0, want_tau=want_tau))
    (J32, t32, l32, f32), (J64, t64, l64, f64) = res[False], res[True]
    assert abs(J32 - J64) <= 1e-6 * J64
    assert np.linalg.norm(l32 - l64) <= 1e-5 * np.linalg.norm(l64)
    assert np.linalg.norm(f32 - f64) <= 1e-5 * np.linalg.norm(f64)
    if want_tau:
        assert abs(t32 - t64) <= 1e-5 * abs(t64)


@pytest.mark.parametrize("prec,dim,iters,every", [("fp32", 16, 23, 6), ("fp16", 40, 17, 17), ("bf16", 64, 12, 4),
                                                  ("fp32", 100, 9, 9), ("fp16", 136, 7, 7), ("fp32", 68, 30, 10)])
def test_staged_two_step_adjoint(capi, prec, dim, iters, every):
    """The two-step stored-point adjoint with its planes staged by TMA, across
    tile columns whose boxes start left of the lattice (x = -4) or run past
    its end, several z-chunks and odd segments: bit for bit the initial
    population gradient of one adjoint step per launch (the same arithmetic
    per site; the lid gradient sums a column's terms in another order) and
    within rounding of the two-step kernel that loads from HBM per thread."""
    one = grads(capi, prec, dim, iters, every, False, adjoint_steps=1)
    direct = grads(capi, prec, dim, iters, every, False, adjoint_steps=2, adjoint_kernel="direct")
    staged = grads(capi, prec, dim, iters, every, False, adjoint_steps=2, adjoint_kernel="staged")
    again = grads(capi, prec, dim, iters, every, False, adjoint_steps=2, adjoint_kernel="staged")
    for r in (direct, staged, again):
        assert r[0] == one[0] and r[1] is None
    np.testing.assert_array_equal(staged[3], one[3])
    np.testing.assert_array_equal(staged[2], again[2])
    np.testing.assert_array_equal(staged[3], again[3])
    for ref in (one, direct):
        assert np.abs(staged[2] - ref[2]).max() <= 1e-6 * np.abs(ref[2]).max()
        assert np.abs(staged[3] - ref[3]).max() <= 1e-6 * np.abs(ref[3]).max()
    assert np.abs(staged[2]).max() > 0 and np.isfinite(staged[3]).all()


@pytest.mark.parametrize("prec,steps", [("fp32", 2), ("fp16", 2), ("bf16", 1), ("fp64", 1)])
@pytest.mark.parametrize("dim,iters,every", [(24, 37, 8), (40, 20, 10)])
def test_recorded_tail_points_are_exact(capi, prec, steps, dim, iters, every):
    """Segments whose linearisation points the adjoint forward recorded (all
    of them, two, or one) skip the recompute in the backward sweep: the
    same loss and gradients bit for bit as recomputing every segment; with a
    tau gradient (full-state sweep) the recorded points are not used."""
    ref = grads(capi, prec, dim, iters, every, False, adjoint_steps=steps, adjoint_tail_segments=-1)
    for tail in (0, 2, 1):
        got = grads(capi, prec, dim, iters, every, False, adjoint_steps=steps, adjoint_tail_segments=tail)
        assert got[0] == ref[0] and got[1] is None
        np.testing.assert_array_equal(got[2], ref[2])
        np.testing.assert_array_equal(got[3], ref[3])
    full = grads(capi, prec, dim, iters, every, True, adjoint_steps=steps, adjoint_tail_segments=-1)
    tail = grads(capi, prec, dim, iters, every, True, adjoint_steps=steps, adjoint_tail_segments=0)
    assert full[1] == tail[1]
    np.testing.assert_array_equal(full[2], tail[2])
    np.testing.assert_array_equal(full[3], tail[3])
