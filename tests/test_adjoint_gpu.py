"""The hand-written adjoint against FP64 central finite differences, the
stored-trajectory adjoint against the checkpointed one, and the autograd
harness.  Small grids; FP64 handles unless stated."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def loss_of(capi, dim, iters, lid, tau, plane, target, prec="fp64", f0=None, seed=0, noise=0.0, stride=None):
    with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=tau, seed=seed, noise_sigma=noise,
                      stride=stride) as L:
        if f0 is not None:
            L.load_f(f0)
        L.adjoint_set_loss(plane, target)
        return L.adjoint_forward(iters, iters)


def setup_case(dim=16, seed=2):
    rng = np.random.default_rng(seed)
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    target = 0.02 * rng.standard_normal(dim * dim)
    return lid, target


@pytest.mark.parametrize("every", [1, 7])
def test_gradients_match_central_differences(capi, every):
    dim, iters, tau, plane = 16, 60, 0.53, 8
    lid, target = setup_case(dim)
    with capi.Lattice(dim, velocity=0.0, precision="fp64", lid=lid, tau=tau, seed=4, noise_sigma=1e-4) as L:
        L.adjoint_set_loss(plane, target)
        J = L.adjoint_forward(iters, every)
        g_tau, g_lid, _ = L.adjoint_backward(1.0, want_f0=False)
    assert J > 0
    h = 1e-6
    # lid: a MOVING column, a column on a FRONT edge (init contribution only), one in the middle
    for (x, y) in [(5, 7), (1, 6), (9, 9)]:
        lp, lm = lid.copy(), lid.copy()
        lp[x + y * dim] += h
        lm[x + y * dim] -= h
        fd = (loss_of(capi, dim, iters, lp, tau, plane, target, seed=4, noise=1e-4) -
              loss_of(capi, dim, iters, lm, tau, plane, target, seed=4, noise=1e-4)) / (2 * h)
        floor = 20 * 2.2e-16 * J / h
        assert abs(g_lid[y, x] - fd) <= 1e-6 * abs(fd) + floor, (x, y, g_lid[y, x], fd)
    fd = (loss_of(capi, dim, iters, lid, tau + h, plane, target, seed=4, noise=1e-4) -
          loss_of(capi, dim, iters, lid, tau - h, plane, target, seed=4, noise=1e-4)) / (2 * h)
    assert abs(g_tau - fd) <= 1e-6 * abs(fd), (g_tau, fd)


def test_initial_population_gradient(capi):
    dim, iters, tau, plane = 16, 40, 0.56, 7
    lid, target = setup_case(dim, 3)
    with capi.Lattice(dim, velocity=0.0, precision="fp64", lid=lid, tau=tau, stride=16) as L:
        f0 = L.f()
        L.adjoint_set_loss(plane, target)
        L.load_f(f0)  # R_0 given explicitly: no lid dependence through the init
        J0 = L.adjoint_forward(iters, 5)
        _, _, g0 = L.adjoint_backward(1.0)
    n = dim ** 3
    h = 1e-6
    rng = np.random.default_rng(8)
    for _ in range(6):
        x, y, z = rng.integers(2, dim - 2, size=3)
        q = int(rng.integers(0, 19))
        idx = x + y * dim + z * dim * dim
        k = ((idx // 16) * 19 + q) * 16 + (idx & 15)
        fp, fm = f0.copy(), f0.copy()
        fp[k] += h
        fm[k] -= h
        fd = (loss_of(capi, dim, iters, lid, tau, plane, target, f0=fp, stride=16) -
              loss_of(capi, dim, iters, lid, tau, plane, target, f0=fm, stride=16)) / (2 * h)
        # FD round-off floor: a few eps * J / h
        floor = 20 * 2.2e-16 * J0 / h
        assert abs(g0[k] - fd) <= 1e-6 * abs(fd) + floor, (x, y, z, q, g0[k], fd)
    assert np.isnan(g0).sum() == 0 and g0.shape == (19 * n,)


def test_checkpointing_is_exact(capi):
    """Recomputed segments reproduce the stored trajectory bit for bit (one
    adjoint step per launch, so that every schedule sums in the same order)."""
    dim, iters = 24, 50
    lid, target = setup_case(dim, 5)
    out = []
    for every in (1, 8, 50):
        with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.52, seed=1, noise_sigma=1e-4,
                          adjoint_steps=1) as L:
            L.adjoint_set_loss(12, target)
            L.adjoint_forward(iters, every)
            out.append(L.adjoint_backward(1.0))
    for o in out[1:]:
        assert o[0] == out[0][0]
        np.testing.assert_array_equal(o[1], out[0][1])
        np.testing.assert_array_equal(o[2], out[0][2])


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
def test_fp32_adjoint_close_to_fp64(capi, prec):
    dim, iters, plane = 24, 80, 12
    lid, target = setup_case(dim, 6)
    res = {}
    for p in ("fp64", prec):
        with capi.Lattice(dim, velocity=0.0, precision=p, lid=lid, tau=0.55, seed=2, noise_sigma=1e-4) as L:
            L.adjoint_set_loss(plane, target)
            L.adjoint_forward(iters, 10)
            res[p] = L.adjoint_backward(1.0, want_f0=False)
    g64, g = res["fp64"], res[prec]
    tol = {"fp32": 1e-4, "fp16": 5e-2, "bf16": 2e-1}[prec]
    assert abs(g[0] - g64[0]) <= tol * abs(g64[0])
    assert np.linalg.norm(g[1] - g64[1]) <= tol * np.linalg.norm(g64[1])


@pytest.mark.parametrize("states,steps", [(2, 1), (3, 1), (5, 1), (9, 1), (3, 2), (6, 2)])
def test_recursive_checkpointing(capi, states, steps):
    """With fewer state buffers than a segment needs, the backward sweep
    checkpoints the segment recursively (2-3 buffers: every state recomputed
    from the checkpoint).  One step per launch: the same launches on the same
    states as the stored trajectory, so the gradients are bit for bit equal;
    two steps per launch pair the steps differently (sums in another order)."""
    dim, iters, every = 16, 45, 45
    lid, target = setup_case(dim, 11)
    res = {}
    for cap in (0, states):
        with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53, seed=5, noise_sigma=1e-4,
                          adjoint_steps=steps, adjoint_max_states=cap) as L:
            L.adjoint_set_loss(8, target)
            J = L.adjoint_forward(iters, every if cap else 1)
            res[cap] = (J,) + tuple(L.adjoint_backward(1.0))
    (J0, t0, l0, f0), (J1, t1, l1, f1) = res[0], res[states]
    assert J0 == J1
    if steps == 1:
        assert t0 == t1
        np.testing.assert_array_equal(l0, l1)
        np.testing.assert_array_equal(f0, f1)
    else:
        assert abs(t1 - t0) <= 1e-5 * abs(t0)
        assert np.abs(l1 - l0).max() <= 1e-5 * np.abs(l0).max()
        assert np.abs(f1 - f0).max() <= 1e-5 * np.abs(f0).max()


def test_recursive_checkpointing_refuses_one_buffer(capi):
    dim = 16
    lid, target = setup_case(dim, 12)
    with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53, adjoint_max_states=1) as L:
        L.adjoint_set_loss(8, target)
        L.adjoint_forward(10, 10)
        with pytest.raises(capi.LbmError, match="too few"):
            L.adjoint_backward(1.0)


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("dim,iters,every", [(16, 23, 6), (40, 17, 17), (64, 12, 4)])
def test_two_step_adjoint_matches_one_step(capi, prec, dim, iters, every):
    """The two-steps-per-launch adjoint (shared-memory a_k) against the
    one-step kernels: same per-site arithmetic, sums in another order.  dim
    40 and 64 cross tile and z-chunk borders; odd segment lengths end with a
    single step."""
    lid, target = setup_case(dim, dim + iters)
    res = {}
    for steps in (1, 2):
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=0.53, seed=3, noise_sigma=1e-4,
                          adjoint_steps=steps) as L:
            L.adjoint_set_loss(dim // 2, target)
            J = L.adjoint_forward(iters, every)
            res[steps] = (J,) + tuple(L.adjoint_backward(1.0))
    (J1, t1, l1, f1), (J2, t2, l2, f2) = res[1], res[2]
    assert J1 == J2
    assert abs(t2 - t1) <= 1e-5 * abs(t1)
    assert np.abs(l2 - l1).max() <= 1e-5 * np.abs(l1).max()
    assert np.abs(f2 - f1).max() <= 1e-5 * np.abs(f1).max()
    assert np.isfinite(f2).all()


def test_autograd_harness(capi):
    torch = pytest.importorskip("torch")
    from lbmcl_gb300.adjoint import cavity_loss
    dim, iters, plane = 16, 30, 8
    lid0, target = setup_case(dim, 9)
    lid = torch.tensor(lid0.reshape(dim, dim), dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(0.54, dtype=torch.float64, requires_grad=True)
    J = cavity_loss(lid, tau, None, dim=dim, iterations=iters, plane_y=plane, target=target, checkpoint_every=6,
                    precision="fp64")
    (3.0 * J).backward()
    with capi.Lattice(dim, velocity=0.0, precision="fp64", lid=lid0, tau=0.54) as L:
        L.adjoint_set_loss(plane, target)
        J2 = L.adjoint_forward(iters, iters)
        g_tau, g_lid, _ = L.adjoint_backward(3.0, want_f0=False)
    assert abs(float(J.detach()) - J2) <= 1e-15 * abs(J2)
    np.testing.assert_allclose(lid.grad.numpy(), g_lid, rtol=1e-12, atol=0)
    assert abs(float(tau.grad) - g_tau) <= 1e-12 * abs(g_tau)


@pytest.mark.parametrize("prec,dim,iters", [("fp64", 12, 15), ("fp64", 16, 20), ("fp32", 16, 20)])
def test_adjoint_matches_reference_adjoint(capi, prec, dim, iters):
    """Field by field against the independent numpy FP64 adjoint of the
    reference algorithm (oracle/adjoint_ref.py)."""
    from oracle import adjoint_ref
    rng = np.random.default_rng(dim + iters)
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    target = 0.02 * rng.standard_normal(dim * dim)
    tau, plane = 0.55, dim // 2
    J_ref, gt_ref, gl_ref, a0_ref = adjoint_ref.run(dim, None, lid, tau, iters, plane, target)
    with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=tau, stride=0) as L:
        L.adjoint_set_loss(plane, target)
        J = L.adjoint_forward(iters, 4)
        gt, gl, g0 = L.adjoint_backward(1.0)
    g0 = g0.reshape(19, dim, dim, dim).astype(np.float64)
    tol = 1e-10 if prec == "fp64" else 2e-4
    assert abs(J - J_ref) <= tol * J_ref
    scale = np.abs(a0_ref).max()
    bad = np.argwhere(np.abs(g0 - a0_ref) > tol * scale)
    assert bad.size == 0, f"{len(bad)} slots differ, first (q, z, y, x) = {bad[:5].tolist()}"
    assert np.abs(gl - gl_ref).max() <= tol * np.abs(gl_ref).max()
    assert abs(gt - gt_ref) <= tol * abs(gt_ref)


def test_adjoint_api_errors(capi):
    """Misuse of the gradient entry points returns a status and a message
    (no exit, no CUDA error), and leaves the handle usable."""
    import ctypes as C
    dim = 16
    lid, target = setup_case(dim, 21)
    L = capi.lib()
    with capi.Lattice(dim, velocity=0.0, precision="fp32", lid=lid, tau=0.53) as lat:
        h = lat.h
        # the loss plane must hold FLUID sites
        for bad in (0, 1, dim - 2, dim):
            assert L.lbm_adjoint_set_loss(h, bad, None) == capi.EINVAL
        # a forward needs a loss; a backward needs the forward of the current state
        J = C.c_double()
        assert L.lbm_adjoint_forward(h, 5, 5, C.byref(J)) == capi.ESTATE
        gt = C.c_double()
        assert L.lbm_adjoint_backward(h, 1.0, C.byref(gt), None, None, 0) == capi.ESTATE
        lat.adjoint_set_loss(8, target)
        assert L.lbm_adjoint_forward(h, 0, 5, C.byref(J)) == capi.EINVAL
        assert L.lbm_adjoint_forward(h, 5, 0, C.byref(J)) == capi.EINVAL
        lat.adjoint_forward(6, 3)
        # a gradient buffer of the wrong size
        buf = np.zeros(10, np.float32)
        assert L.lbm_adjoint_backward(h, 1.0, C.byref(gt), None, buf.ctypes.data_as(C.c_void_p), buf.nbytes) \
            == capi.EINVAL
        assert "grad_f0" in L.lbm_last_error().decode()
        # stepping after the forward invalidates it
        lat.step(1)
        assert L.lbm_adjoint_backward(h, 1.0, C.byref(gt), None, None, 0) == capi.ESTATE
        # and the handle still works
        J2 = lat.adjoint_forward(6, 3)
        g = lat.adjoint_backward(1.0, want_f0=False)
        assert np.isfinite(J2) and np.isfinite(g[0]) and np.isfinite(g[1]).all()


@pytest.mark.parametrize("prec,steps,every", [("fp32", 1, 8), ("fp32", 2, 10), ("fp16", 2, 6), ("fp64", 1, 5)])
def test_segment_graph_replay_is_exact(capi, prec, steps, every):
    """Full segments of the backward sweep replayed as one captured graph
    (from a staged copy of the checkpoint) against direct launches: the
    same launches on the same states, bit for bit; a second sweep reuses the
    graphs."""
    dim, iters = 24, 43
    lid, target = setup_case(dim, 17)
    res = []
    for g in (0, 1):
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=0.53, seed=6, noise_sigma=1e-4,
                          adjoint_steps=steps, graph_iterations=g) as L:
            L.adjoint_set_loss(12, target)
            f0 = L.f()
            out = []
            for _ in range(2):  # the same start each time (the forward advances the state)
                L.load_f(f0)
                J = L.adjoint_forward(iters, every)
                out.append((J,) + tuple(L.adjoint_backward(1.0)))
            res.append(out)
    for a, b in zip(res[0], res[1]):
        assert a[0] == b[0] and a[1] == b[1]
        np.testing.assert_array_equal(a[2], b[2])
        np.testing.assert_array_equal(a[3], b[3])
    assert res[0][0][1] == res[0][1][1]   # the replayed second sweep repeats the first
