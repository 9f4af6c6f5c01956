"""Generates the committed golden fixtures of this directory.

Run in a checkout next to the reference tree (it reads the reference's files;
nothing at test time does):

    make -C oracle ref                  # builds oracle/_ref from kernels.cl
    python tests/golden/make_golden.py [--ref /path/to/LBMCL]

Outputs
  sailfish_ldc8.npz    rho / v of the reference's golden VTI files
                       target_results/8/ldc.0.{00..10}.vti (8^3, every step)
  sailfish_ldc32.npz   the same for target_results/32 at steps 20 and 500
  ref_runs.json        SHA-256 digests of the reference kernel's buffers
                       (f, rho, u) after each listed iteration, for the runs
                       in RUNS, executed by the reference's own kernels.cl
                       compiled for the CPU (oracle/_ref)
  ref_f8_f32.npz       full f of run "ldc8" at iterations 0, 1, 2, 10, for
                       diagnostics when a digest differs
  lid_profiles.npz     the per-column lid arrays the runs use
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lbmcl_gb300 import vti  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

# name: (dim, precision, stride, viscosity, velocity, lid key or None, iterations, every, digest every)
RUNS = {
    "ldc8": (8, "f32", 8, 0.0089, 0.05, None, 10, 1, 1),
    "cfg1_32": (32, "f32", 8, 0.0089, 0.05, None, 10, 1, 1),
    "ldc32_f64": (32, "f64", 8, 0.0089, 0.05, None, 10, 1, 1),
    "test32_500": (32, "f32", 32, 0.0089, 0.05, None, 500, 20, 20),
    "lid16_aos": (16, "f32", 1, 0.0089, 0.05, "lid16", 10, 2, 1),
    "lid16_soa_f64": (16, "f64", 4096, 0.01, 0.05, "lid16", 10, 3, 1),
    "dim4_f32": (4, "f32", 4, 0.0089, 0.05, None, 10, 1, 1),
    "dim12_f32": (12, "f32", 16, 0.0089, 0.08, None, 12, 4, 1),
    "dim12_f64": (12, "f64", 64, 0.005, 0.08, None, 12, 4, 1),
}


def lid_profiles() -> dict:
    rng = np.random.default_rng(20240607)
    return {"lid16": 0.05 + 0.005 * rng.standard_normal(16 * 16)}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_digests(name, spec, lids):
    dim, prec, stride, visc, vel, lidkey, iters, every, dig_every = spec
    lid = lids[lidkey] if lidkey else None
    L = po.RefLattice(dim, visc, vel, prec, stride, lid=lid)
    out = {"spec": list(spec), "digests": {"0": [sha(L.state), sha(L.rho), sha(L.u)]},
           "map": sha(L.map)}
    for it in range(1, iters + 1):
        L.step(1, every=every)
        if it % dig_every == 0:
            out["digests"][str(it)] = [sha(L.state), sha(L.rho), sha(L.u)]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("LBMCL_REF", "/root/reference"),
                    help="path of the reference checkout (default: $LBMCL_REF)")
    args = ap.parse_args()
    if not po.ref_available("f32") or not po.ref_available("f64"):
        sys.exit("oracle/_ref is not built: run `make -C oracle ref REF=<path>` first")

    # Sailfish golden files shipped with the reference
    tr = os.path.join(args.ref, "target_results")
    d8 = {}
    for it in range(0, 11):
        v = vti.read_vti(os.path.join(tr, "8", f"ldc.0.{it:02d}.vti"))
        d8[f"rho_{it}"] = v["rho"].astype(np.float32)
        d8[f"v_{it}"] = v["v"].astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "sailfish_ldc8.npz"), **d8)
    d32 = {}
    for it in (20, 500):
        v = vti.read_vti(os.path.join(tr, "32", f"ldc.0.{it:03d}.vti"))
        d32[f"rho_{it}"] = v["rho"].astype(np.float32)
        d32[f"v_{it}"] = v["v"].astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "sailfish_ldc32.npz"), **d32)

    lids = lid_profiles()
    np.savez_compressed(os.path.join(HERE, "lid_profiles.npz"), **lids)

    runs = {name: run_digests(name, spec, lids) for name, spec in RUNS.items()}
    with open(os.path.join(HERE, "ref_runs.json"), "w") as fh:
        json.dump(runs, fh, indent=1, sort_keys=True)

    L = po.RefLattice(8, 0.0089, 0.05, "f32", 8)
    fs = {"f_0": L.state.copy()}
    for it in range(1, 11):
        L.step(1, every=1)
        if it in (1, 2, 10):
            fs[f"f_{it}"] = L.state.copy()
    np.savez_compressed(os.path.join(HERE, "ref_f8_f32.npz"), **fs)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
