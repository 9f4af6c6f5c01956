"""Accuracy and gradient checks of the workloads the library is specified on.

    python -m lbmcl_gb300.validate storage  [--dim 512 --steps 5000]
    python -m lbmcl_gb300.validate adjoint  [--dim 64 --steps 2000 --every 100 ...]
    python -m lbmcl_gb300.validate lidfield [--dim 256 --steps 10000 --every 100 --columns 8]

storage   16-bit deviation storage (FP16, BF16) and FP32 against the FP64 run
          of the same seeded cavity (nu = 0.005, lid u = 0.08, N(0, 1e-4)
          noise): max / RMS error of rho and u over the FLUID and MOVING
          sites, relative L2 error of u_x on the mid-plane y = dim/2, MLUPS.
adjoint   64^3, nu = 0.01: loss = mid-plane u_x MSE against the field of a
          seeded forward run with lid 0.06; controls lid (0.05), tau, initial
          populations (seeded N(0, 1e-4) perturbation).  The FP32 adjoint with
          checkpoints against FP64 central finite differences (h = 1e-6) and
          against the FP64 stored-trajectory adjoint.
lidfield  256^3, nu = 0.0089: per-column lid field 0.05 + N(0, 0.005); target
          made by a forward run with a smooth lid (4 random 2-D sinusoids of
          total amplitude 0.02 around 0.05); 16-bit forward, FP32 adjoint,
          sqrt checkpointing.  Adjoint/forward time, device memory, gradient
          error against FP64 finite differences on random active columns and
          against the FP64 adjoint.
Each prints one JSON object.  Every run uses the GPU library only.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi


def _u_at(L, dim, steps):
    """rho, u of the state after `steps` iterations (the moments iteration
    `steps` stored, i.e. of R_{steps-1})."""
    L.step(steps - 1)
    L.step(1, every=steps)
    L.sync()
    return L.rho().astype(np.float64), L.u().astype(np.float64).reshape(3, dim, dim, dim)


def storage(args):
    dim, steps = args.dim, args.steps
    kw = dict(viscosity=0.005, velocity=0.08, seed=args.seed, noise_sigma=1e-4, stride=0)
    import torch
    out = {"check": "storage", "dim": dim, "steps": steps, "nu": 0.005, "lid": 0.08, "seed": args.seed}
    ref = None
    for prec in ("fp64", "fp32", "fp16", "bf16"):
        with capi.Lattice(dim, precision=prec, **kw) as L:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rho, u = _u_at(L, dim, steps)
            secs = time.perf_counter() - t0
        mlups = (dim - 2) ** 3 * steps / secs / 1e6
        if ref is None:
            ref = (rho, u)
            out["fp64_mlups"] = round(mlups, 1)
            ok = np.isfinite(rho)
            out["sites"] = int(ok.sum())
            continue
        rr, ur = ref
        ok = np.isfinite(rr)
        drho = np.abs(rho[ok] - rr.reshape(-1)[ok]) if rho.ndim == 1 else None
        du = np.abs(u.reshape(3, -1)[:, ok] - ur.reshape(3, -1)[:, ok])
        mid = dim // 2
        um, urm = u[0, :, mid, :], ur[0, :, mid, :]
        m = np.isfinite(urm)
        out[prec] = {
            "mlups": round(mlups, 1),
            "rho_max_err": float(drho.max()), "rho_rms_err": float(np.sqrt((drho ** 2).mean())),
            "u_max_err": float(du.max()), "u_rms_err": float(np.sqrt((du ** 2).mean())),
            "u_max_ref": float(np.abs(ur.reshape(3, -1)[:, ok]).max()),
            "midplane_ux_rel_l2": float(np.linalg.norm(um[m] - urm[m]) / np.linalg.norm(urm[m])),
            "finite": bool(np.isfinite(u.reshape(3, -1)[:, ok]).all()),
        }
    print(json.dumps(out), flush=True)


def _loss(dim, steps, lid, tau, plane, target, prec, f0=None, stride=None, seed=0, noise=0.0, every=None):
    with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=tau, stride=stride, seed=seed,
                      noise_sigma=noise) as L:
        if f0 is not None:
            L.load_f(f0)
        L.adjoint_set_loss(plane, target)
        return L.adjoint_forward(steps, every or steps)


def adjoint(args):
    import torch
    dim, steps, c = args.dim, args.steps, args.every
    nu = 0.01
    tau = 3 * nu + 0.5
    plane = dim // 2
    rng = np.random.default_rng(args.seed)
    # target: forward run with lid 0.06 (same seeded noise), u_x of plane y
    with capi.Lattice(dim, nu, 0.06, precision="fp64", seed=args.seed, noise_sigma=1e-4, stride=0) as L:
        L.step(steps)
        L.step(1, every=steps + 1)
        ut = L.u().reshape(3, dim, dim, dim)[0, :, plane, :]
    target = np.nan_to_num(ut).reshape(-1)  # [z, x]
    lid = np.full(dim * dim, 0.05)
    out = {"check": "adjoint", "dim": dim, "steps": steps, "checkpoint_every": c, "nu": nu, "plane_y": plane}
    grads = {}
    for prec, every in (("fp32", c), ("fp64", 1)):
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=tau, seed=args.seed, noise_sigma=1e-4,
                          stride=0) as L:
            f0 = L.f()
            L.adjoint_set_loss(plane, target)
            L.load_f(f0)   # the initial populations are a control
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J = L.adjoint_forward(steps, every)
            t1 = time.perf_counter()
            g = L.adjoint_backward(1.0)
            t2 = time.perf_counter()
        grads[prec] = (J, g, f0, t1 - t0, t2 - t1)
    J32, (gt32, gl32, g032), f0_32, tf, tb = grads["fp32"]
    J64, (gt64, gl64, g064), f0_64, _, _ = grads["fp64"]
    out["loss_fp32"], out["loss_fp64"] = J32, J64
    out["fp32_forward_s"], out["fp32_backward_s"] = round(tf, 3), round(tb, 3)
    # FP64 stored-trajectory adjoint vs the checkpointed FP32 adjoint, whole fields
    out["vs_fp64_stored_trajectory"] = {
        "tau_rel": abs(gt32 - gt64) / abs(gt64),
        "lid_rel_l2": float(np.linalg.norm(gl32 - gl64) / np.linalg.norm(gl64)),
        "f0_rel_l2": float(np.linalg.norm(g032 - g064) / np.linalg.norm(g064)),
    }
    # FP64 central finite differences
    h = 1e-6
    fd = {}
    cols = [(int(x), int(y)) for x, y in rng.integers(2, dim - 2, size=(args.columns, 2))]
    rows = []
    for (x, y) in cols:
        lp, lm = lid.copy(), lid.copy()
        lp[x + y * dim] += h
        lm[x + y * dim] -= h
        d = (_loss(dim, steps, lp, tau, plane, target, "fp64", f0=f0_64, stride=0) -
             _loss(dim, steps, lm, tau, plane, target, "fp64", f0=f0_64, stride=0)) / (2 * h)
        rows.append({"x": x, "y": y, "fd": d, "adj_fp32": float(gl32[y, x]), "adj_fp64": float(gl64[y, x]),
                     "rel_fp32": abs(gl32[y, x] - d) / abs(d), "rel_fp64": abs(gl64[y, x] - d) / abs(d)})
    fd["lid"] = rows
    d = (_loss(dim, steps, lid, tau + h, plane, target, "fp64", f0=f0_64, stride=0) -
         _loss(dim, steps, lid, tau - h, plane, target, "fp64", f0=f0_64, stride=0)) / (2 * h)
    fd["tau"] = {"fd": d, "adj_fp32": gt32, "adj_fp64": gt64, "rel_fp32": abs(gt32 - d) / abs(d),
                 "rel_fp64": abs(gt64 - d) / abs(d)}
    rows = []
    n = dim ** 3
    for _ in range(args.columns):
        x, y, z = (int(v) for v in rng.integers(2, dim - 2, size=3))
        q = int(rng.integers(0, 19))
        k = q * n + x + y * dim + z * dim * dim
        fp, fm = f0_64.copy(), f0_64.copy()
        fp[k] += h
        fm[k] -= h
        d = (_loss(dim, steps, lid, tau, plane, target, "fp64", f0=fp, stride=0) -
             _loss(dim, steps, lid, tau, plane, target, "fp64", f0=fm, stride=0)) / (2 * h)
        rows.append({"site": [x, y, z], "q": q, "fd": d, "adj_fp32": float(g032[k]), "adj_fp64": float(g064[k]),
                     "fd_roundoff": 2.2e-16 * J64 / h})
    fd["f0"] = rows
    out["finite_differences_fp64_h1e-6"] = fd
    print(json.dumps(out), flush=True)


def smooth_lid(dim, rng, amplitude=0.02, base=0.05):
    """A smooth lid field [y, x]: base + the sum of four seeded 2-D sinusoids
    (wave numbers 1..3, random phases) scaled to a peak deviation of
    `amplitude`."""
    x = np.arange(dim) / dim
    X, Y = np.meshgrid(x, x)  # [y, x]
    f = np.zeros((dim, dim))
    for _ in range(4):
        kx, ky = rng.integers(1, 4, size=2)
        ph = rng.uniform(0, 2 * np.pi, size=2)
        f += np.sin(2 * np.pi * kx * X + ph[0]) * np.sin(2 * np.pi * ky * Y + ph[1])
    f *= amplitude / np.abs(f).max()
    return base + f


def lidfield(args):
    import torch
    dim, steps, c = args.dim, args.steps, args.every
    nu = 0.0089
    tau = 3 * nu + 0.5
    plane = dim // 2
    rng = np.random.default_rng(args.seed)
    target_lid = smooth_lid(dim, rng).reshape(-1)
    with capi.Lattice(dim, nu, 0.05, precision="fp32", lid=target_lid, stride=0) as L:
        L.step(steps)
        L.step(1, every=steps + 1)
        target = np.nan_to_num(L.u().reshape(3, dim, dim, dim)[0, :, plane, :]).reshape(-1)
    lid = 0.05 + 0.005 * rng.standard_normal(dim * dim)
    out = {"check": "lidfield", "dim": dim, "steps": steps, "checkpoint_every": c, "nu": nu, "plane_y": plane,
           "storage": args.precision, "adjoint": "fp32"}
    with capi.Lattice(dim, velocity=0.0, precision=args.precision, lid=lid, tau=tau, stride=0) as L:
        stream = torch.cuda.ExternalStream(L.stream)
        L.step(3)
        L.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.step(100)
        e1.record(stream)
        e1.synchronize()
        fwd_ms = e0.elapsed_time(e1) / 100
    free0, total = torch.cuda.mem_get_info()
    with capi.Lattice(dim, velocity=0.0, precision=args.precision, lid=lid, tau=tau, stride=0) as L:
        L.adjoint_set_loss(plane, target)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J = L.adjoint_forward(steps, c)
        t1 = time.perf_counter()
        free1, _ = torch.cuda.mem_get_info()
        gt, gl, _ = L.adjoint_backward(1.0, want_f0=False)
        t2 = time.perf_counter()
        free2, _ = torch.cuda.mem_get_info()
    out.update({"loss": J, "forward_ms_per_iter": round(fwd_ms, 4),
                "checkpointed_forward_ms_per_iter": round((t1 - t0) * 1e3 / steps, 4),
                "backward_ms_per_iter": round((t2 - t1) * 1e3 / steps, 4),
                "adjoint_over_forward": round((t2 - t1) * 1e3 / steps / fwd_ms, 3),
                "device_gb_used_peak": round((free0 - min(free1, free2)) / 1e9, 2)})
    if args.fp64_adjoint:
        # FP64 states are 4x the 16-bit ones: wider top-level checkpoints, and
        # the backward sweep checkpoints each segment again as memory requires
        c64 = args.fp64_every
        free_a, _ = torch.cuda.mem_get_info()
        with capi.Lattice(dim, velocity=0.0, precision="fp64", lid=lid, tau=tau, stride=0) as L:
            L.adjoint_set_loss(plane, target)
            t0 = time.perf_counter()
            J64 = L.adjoint_forward(steps, c64)
            t1 = time.perf_counter()
            gt64, gl64, _ = L.adjoint_backward(1.0, want_f0=False)
            t2 = time.perf_counter()
            free_b, _ = torch.cuda.mem_get_info()
        act = (slice(2, dim - 2), slice(2, dim - 2))
        out["fp64_adjoint_run"] = {"checkpoint_every": c64, "forward_s": round(t1 - t0, 1),
                                   "backward_s": round(t2 - t1, 1),
                                   "device_gb_used": round((free_a - free_b) / 1e9, 1)}
        out["vs_fp64_adjoint"] = {"loss_fp64": J64,
                                  "lid_rel_l2": float(np.linalg.norm(gl[act] - gl64[act]) / np.linalg.norm(gl64[act])),
                                  "tau_rel": abs(gt - gt64) / abs(gt64)}
    h = 1e-6
    rows = []
    for (x, y) in [(int(a), int(b)) for a, b in rng.integers(2, dim - 2, size=(args.columns, 2))]:
        lp, lm = lid.copy(), lid.copy()
        lp[x + y * dim] += h
        lm[x + y * dim] -= h
        d = (_loss(dim, steps, lp, tau, plane, target, "fp64", stride=0) -
             _loss(dim, steps, lm, tau, plane, target, "fp64", stride=0)) / (2 * h)
        row = {"x": x, "y": y, "fd_fp64": d, "adjoint": float(gl[y, x]), "rel": abs(gl[y, x] - d) / abs(d)}
        if args.fp64_adjoint:
            row["adjoint_fp64"] = float(gl64[y, x])
            row["rel_fp64"] = abs(gl64[y, x] - d) / abs(d)
        rows.append(row)
    out["finite_differences_fp64_h1e-6"] = rows
    print(json.dumps(out), flush=True)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("storage")
    p.add_argument("--dim", type=int, default=512)
    p.add_argument("--steps", type=int, default=5000)
    p.add_argument("--seed", type=int, default=1234)
    p = sub.add_parser("adjoint")
    p.add_argument("--dim", type=int, default=64)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--every", type=int, default=100)
    p.add_argument("--columns", type=int, default=4)
    p.add_argument("--seed", type=int, default=1234)
    p = sub.add_parser("lidfield")
    p.add_argument("--dim", type=int, default=256)
    p.add_argument("--steps", type=int, default=10000)
    p.add_argument("--every", type=int, default=100)
    p.add_argument("--columns", type=int, default=8)
    p.add_argument("--precision", default="fp16")
    p.add_argument("--fp64-adjoint", action="store_true")
    p.add_argument("--fp64-every", type=int, default=500, help="top-level checkpoint interval of the FP64 adjoint")
    p.add_argument("--seed", type=int, default=1234)
    a = ap.parse_args(argv)
    {"storage": storage, "adjoint": adjoint, "lidfield": lidfield}[a.cmd](a)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
