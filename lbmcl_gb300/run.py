"""Run one cavity through the C ABI and report MLUPS (also the small case
the ncu captures profile).

    python -m lbmcl_gb300.run --dim 256 --precision fp16 --steps 4 [--every 0]
"""
from __future__ import annotations

import argparse
import time

from . import capi


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--dim", type=int, default=256)
    ap.add_argument("--precision", default="fp32", choices=sorted(capi.PRECISIONS))
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--every", type=int, default=0)
    ap.add_argument("--viscosity", type=float, default=0.0089)
    ap.add_argument("--velocity", type=float, default=0.05)
    ap.add_argument("--noise", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--kernel", default="auto", choices=sorted(capi.KERNELS))
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--adjoint-steps", type=int, default=0, help="adjoint steps per launch (0 = default)")
    ap.add_argument("--adjoint-max-states", type=int, default=0, help="cap on the backward sweep's state buffers")
    ap.add_argument("--adjoint", default="", help="T,c: also run an adjoint forward/backward of T iterations, "
                                                  "checkpoint every c")
    ap.add_argument("--tau", action="store_true", help="the adjoint also forms dJ/dtau (full-state segments)")
    ap.add_argument("--adjoint-kernel", default="auto", choices=["auto", "direct", "staged"],
                    help="two-step adjoint of the stored-point sweep: per-thread loads or TMA-staged planes")
    ap.add_argument("--adjoint-tail", type=int, default=0,
                    help="trailing segments whose points the adjoint forward records (0 = as many as fit, -1 = none)")
    a = ap.parse_args(argv)
    with capi.Lattice(a.dim, a.viscosity, a.velocity, precision=a.precision, stride=0, seed=a.seed,
                      noise_sigma=a.noise, block_threads=a.block, profile_steps=True, kernel=a.kernel,
                      stages=a.stages, adjoint_steps=a.adjoint_steps,
                      adjoint_max_states=a.adjoint_max_states, adjoint_kernel=a.adjoint_kernel,
                      adjoint_tail_segments=a.adjoint_tail) as L:
        t0 = time.perf_counter()
        L.step(a.steps, every=a.every)
        L.sync()
        wall = time.perf_counter() - t0
        total_ms, kernels_ms = L.timing()
        mass, energy, count = L.reduce()
        if a.adjoint:
            T, c = (int(v) for v in a.adjoint.split(","))
            L.adjoint_set_loss(a.dim // 2, None)
            t0 = time.perf_counter()
            J = L.adjoint_forward(T, c)
            t1 = time.perf_counter()
            g_tau, g_lid, _ = L.adjoint_backward(1.0, want_f0=False, want_tau=a.tau)
            t2 = time.perf_counter()
            print(f"adjoint T={T} c={c} loss={J:.6e} forward={1e3 * (t1 - t0) / T:.4f} ms/iter "
                  f"backward={1e3 * (t2 - t1) / T:.4f} ms/iter |dJ/dlid|={float((g_lid ** 2).sum()) ** 0.5:.6e}"
                  + (f" dJ/dtau={g_tau:.6e}" if a.tau else ""))
    wet = (a.dim - 2) ** 3
    print(f"dim={a.dim} precision={a.precision} steps={a.steps} kernels={kernels_ms:.3f} ms "
          f"kernel MLUPS={wet * a.steps / (kernels_ms * 1e3):.1f} wall={wall * 1e3:.1f} ms "
          f"mass={mass:.9e} energy={energy:.6e} sites={count:.0f}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
