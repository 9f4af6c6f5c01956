"""The numpy FP64 reference adjoint (oracle/adjoint_ref.py) against central
finite differences of the oracle itself (CPU only)."""
import numpy as np
import pytest

from oracle import adjoint_ref


def loss(oracle, dim, lid, tau, iters, plane, target):
    return adjoint_ref.run(dim, None, lid, tau, iters, plane, target)[0]


@pytest.mark.parametrize("dim,iters", [(10, 12), (12, 25)])
def test_reference_adjoint_matches_finite_differences(oracle, dim, iters):
    rng = np.random.default_rng(dim)
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    target = 0.02 * rng.standard_normal(dim * dim)
    tau, plane = 0.55, dim // 2
    J, g_tau, g_lid, _ = adjoint_ref.run(dim, None, lid, tau, iters, plane, target)
    h = 1e-6
    for (x, y) in [(3, 4), (1, 5), (dim - 3, dim - 4)]:
        lp, lm = lid.copy(), lid.copy()
        lp[x + y * dim] += h
        lm[x + y * dim] -= h
        fd = (loss(oracle, dim, lp, tau, iters, plane, target) - loss(oracle, dim, lm, tau, iters, plane, target)) / (2 * h)
        assert abs(g_lid[y, x] - fd) <= 1e-6 * abs(fd) + 20 * 2.2e-16 * J / h, (x, y, g_lid[y, x], fd)
    fd = (loss(oracle, dim, lid, tau + h, iters, plane, target) -
          loss(oracle, dim, lid, tau - h, iters, plane, target)) / (2 * h)
    assert abs(g_tau - fd) <= 1e-6 * abs(fd) + 20 * 2.2e-16 * J / h, (g_tau, fd)
