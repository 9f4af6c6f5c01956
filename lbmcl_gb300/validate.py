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
          sqrt checkpointing.  Adjoint/forward time, device memory, and the
          gradient's error budget on random active columns: the FP32
          adjoint's rounding (against the FP64 adjoint of the same 16-bit
          trajectory), the storage rounding it linearises through (against
          central differences of the 16-bit model), the model difference
          (against the FP64 model's adjoint) and the FP64 adjoint's exactness
          (against FP64 central differences).
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
    """The 256^3 x 10000 lid-field gradient and its error budget.

    g_32   FP32 adjoint of the 16-bit trajectory (the product; lid control,
           stored-point sweep)
    g_a64  FP64-arithmetic adjoint of the same 16-bit trajectory
    fd16   central differences of the 16-bit model itself, h well above the
           FP16 quantum of the stored deviations, three h halving, Richardson
           extrapolated (FD(h) = g + c h^2 + rounding noise / h)
    g_64   FP64 adjoint of the FP64 trajectory (the FP64 model)
    fd64   FP64 central differences (h = 1e-6) of the FP64 model
    Components: (i) adjoint rounding |g_32 - g_a64|; (ii) linearisation of
    the storage rounding |g_a64 - fd16|; (iii) the model difference
    |g_a64 - g_64|; and the exactness |g_64 - fd64| of the FP64 adjoint.
    """
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
    cols = [(int(a), int(b)) for a, b in rng.integers(2, dim - 2, size=(args.columns, 2))]
    act = (slice(2, dim - 2), slice(2, dim - 2))
    out = {"check": "lidfield", "dim": dim, "steps": steps, "checkpoint_every": c, "nu": nu, "plane_y": plane,
           "storage": args.precision, "adjoint": "fp32", "control": "per-column lid field",
           "columns": [{"x": x, "y": y} for x, y in cols]}
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

    def run_adjoint(prec, every, a64=False):
        free0, _ = torch.cuda.mem_get_info()
        with capi.Lattice(dim, velocity=0.0, precision=prec, lid=lid, tau=tau, stride=0, adjoint_fp64=a64) as L:
            L.adjoint_set_loss(plane, target)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J = L.adjoint_forward(steps, every)
            t1 = time.perf_counter()
            free1, _ = torch.cuda.mem_get_info()
            _, gl, _ = L.adjoint_backward(1.0, want_f0=False, want_tau=False)
            t2 = time.perf_counter()
            free2, _ = torch.cuda.mem_get_info()
        return J, gl, t1 - t0, t2 - t1, (free0 - min(free1, free2)) / 1e9

    J, g32, tf, tb, gb = run_adjoint(args.precision, c)
    out.update({"loss": J, "forward_ms_per_iter": round(fwd_ms, 4),
                "checkpointed_forward_ms_per_iter": round(tf * 1e3 / steps, 4),
                "backward_ms_per_iter": round(tb * 1e3 / steps, 4),
                "adjoint_over_forward": round(tb * 1e3 / steps / fwd_ms, 3),
                "device_gb_used_peak": round(gb, 2)})
    rel = lambda a, b: float(np.linalg.norm(a[act] - b[act]) / np.linalg.norm(b[act]))
    col = lambda g: [float(g[y, x]) for x, y in cols]
    _, ga64, tf64, tb64, _ = run_adjoint(args.precision, c, a64=True)
    out["fp64_adjoint_same_trajectory"] = {"backward_s": round(tb64, 1), "lid": col(ga64)}
    out["i_adjoint_rounding"] = {"field_rel_l2": rel(g32, ga64),
                                 "columns_rel": [abs(a - b) / abs(b) for a, b in zip(col(g32), col(ga64))]}

    # central differences of the 16-bit model, h halving, Richardson
    hs = [float(h) for h in args.fd16_h.split(",")]
    fd16 = []
    for (x, y) in cols:
        vals = []
        for h in hs:
            lp, lm = lid.copy(), lid.copy()
            lp[x + y * dim] += h
            lm[x + y * dim] -= h
            vals.append((_loss(dim, steps, lp, tau, plane, target, args.precision, stride=0) -
                         _loss(dim, steps, lm, tau, plane, target, args.precision, stride=0)) / (2 * h))
        rich = [(4 * vals[k + 1] - vals[k]) / 3 for k in range(len(vals) - 1)]
        fd16.append({"x": x, "y": y, "fd": vals, "richardson": rich})
    best16 = [r["richardson"][-1] for r in fd16]
    # the spread of the extrapolations is the FD's own uncertainty
    unc16 = [abs(r["richardson"][-1] - r["richardson"][-2]) / abs(r["richardson"][-1]) if len(r["richardson"]) > 1
             else None for r in fd16]
    out["fd_16bit_model"] = {"h": hs, "columns": fd16}
    out["ii_storage_linearisation"] = {
        "columns_rel": [abs(a - b) / abs(b) for a, b in zip(col(ga64), best16)],
        "fd_uncertainty_rel": unc16}

    if args.fp64_adjoint:
        c64 = args.fp64_every
        J64, g64, tf, tb, gb = run_adjoint("fp64", c64)
        out["fp64_model"] = {"loss": J64, "checkpoint_every": c64, "forward_s": round(tf, 1),
                             "backward_s": round(tb, 1), "device_gb_used": round(gb, 1), "lid": col(g64)}
        out["iii_model_difference"] = {"field_rel_l2": rel(ga64, g64),
                                       "columns_rel": [abs(a - b) / abs(b) for a, b in zip(col(ga64), col(g64))]}
        out["total_fp32_adjoint_vs_fp64_model"] = {
            "field_rel_l2": rel(g32, g64),
            "columns_rel": [abs(a - b) / abs(b) for a, b in zip(col(g32), col(g64))]}
        h = 1e-6
        rows = []
        for (x, y) in cols[:args.fd64_columns]:
            lp, lm = lid.copy(), lid.copy()
            lp[x + y * dim] += h
            lm[x + y * dim] -= h
            d = (_loss(dim, steps, lp, tau, plane, target, "fp64", stride=0) -
                 _loss(dim, steps, lm, tau, plane, target, "fp64", stride=0)) / (2 * h)
            rows.append({"x": x, "y": y, "fd_fp64": d, "adjoint_fp64": float(g64[y, x]),
                         "rel_fp64": abs(g64[y, x] - d) / abs(d), "adjoint_fp32_16bit": float(g32[y, x]),
                         "rel_fp32_16bit": abs(g32[y, x] - d) / abs(d)})
        out["fp64_exactness_fd_h1e-6"] = rows
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
    p.add_argument("--fd16-h", default="1e-3,5e-4,2.5e-4", help="steps of the 16-bit model's central differences")
    p.add_argument("--fd64-columns", type=int, default=4, help="columns checked by FP64 central differences")
    p.add_argument("--seed", type=int, default=1234)
    a = ap.parse_args(argv)
    {"storage": storage, "adjoint": adjoint, "lidfield": lidfield}[a.cmd](a)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
