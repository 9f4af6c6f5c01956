"""SHA-256 digests of the files the reference's own host writers produce.

The reference host class's writers (lbmcl.hpp:159-334: storeMap, storeF,
storeData) are compiled from the reference tree against an OpenCL stand-in
(`make -C oracle refwriters` -> oracle/_ref/librefwriters.so) and fed with the
oracle's data, which is bit-identical to the reference kernel's.  For each run
below, the files the reference program writes for those command-line flags
are produced and hashed into host_digests.json; tests/test_host_cli.py runs
the lbmcl host program with the same flags on the GPU and compares digests.

    python tests/golden/make_host_golden.py          # needs oracle/_ref
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
LIB = os.path.join(ROOT, "oracle", "_ref", "librefwriters.so")
OUT = os.path.join(HERE, "host_digests.json")

# (flags of the lbmcl program, as the reference CLI takes them)
RUNS = [
    # make testall at 8^3: every iteration, f and map dumps (Makefile:60-78)
    dict(dim=8, prec="f32", iterations=10, every=1, stride=8, lws="8,8,8", dump_f=True, dump_map=True),
    # double precision (-F) with f dumps every iteration, VTI every 2nd
    dict(dim=16, prec="f64", iterations=4, every=2, stride=16, lws="8,8,8", dump_f=True, dump_map=False),
    # test32-like: 32^3, VTI every 20 iterations (Makefile:81-86)
    dict(dim=32, prec="f32", iterations=40, every=20, stride=32, lws="32,32,1", dump_f=False, dump_map=True),
]


def cli_args(r, vdir, pdir):
    a = ["-d", r["dim"], "-n", 0.0089, "-u", 0.05, "-i", r["iterations"], "-e", r["every"], "-w", r["lws"],
         "-s", r["stride"], "-v", vdir, "-p", pdir]
    if r["prec"] == "f64":
        a.append("-F")
    if r["dump_f"]:
        a.append("-f")
    if r["dump_map"]:
        a.append("-m")
    return [str(x) for x in a]


def sha(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def _lib():
    L = C.CDLL(LIB)
    L.refw_store_map.argtypes = [C.c_int, C.c_void_p, C.c_char_p]
    for p in ("f32", "f64"):
        getattr(L, f"refw_store_f_{p}").argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_char_p]
        getattr(L, f"refw_store_data_{p}").argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                                      C.c_char_p]
    return L


def write_run(r, d):
    """The reference program's files of run r into directory d (the order of
    lbmcl.hpp:490-521: map, VTI 0, f 0, then per iteration it the f dump of
    the buffer iteration it reads and, every `every`, the VTI of the moments
    iteration it stored)."""
    from oracle import pyoracle as po
    L = _lib()
    dim, T, every, p = r["dim"], r["iterations"], r["every"], r["prec"]
    o = po.OracleLattice(dim, 0.0089, 0.05, p, r["stride"])
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    db = d.encode()
    if r["dump_map"]:
        L.refw_store_map(dim, ptr(o.map), db)
    store_data = getattr(L, f"refw_store_data_{p}")
    store_f = getattr(L, f"refw_store_f_{p}")
    if every:
        store_data(dim, T, ptr(o.rho), ptr(o.u), 0, db)
    if r["dump_f"]:
        store_f(dim, T, r["stride"], ptr(o.state), 0, db)
    for it in range(1, T + 1):
        if r["dump_f"]:
            store_f(dim, T, r["stride"], ptr(np.ascontiguousarray(o.state)), it, db)
        o.step(1, every=every)
        if every and it % every == 0:
            store_data(dim, T, ptr(o.rho), ptr(o.u), it, db)


def generate() -> dict:
    out = {"what": "SHA-256 of the files the reference's writers (lbmcl.hpp:159-334) produce for each run",
           "runs": []}
    for r in RUNS:
        with tempfile.TemporaryDirectory() as d:
            write_run(r, d)
            files = {f: sha(os.path.join(d, f)) for f in sorted(os.listdir(d))}
        out["runs"].append({"run": r, "files": files})
    return out


if __name__ == "__main__":
    if not os.path.exists(LIB):
        sys.exit(f"{LIB} is missing: build it with `make -C oracle refwriters` where the reference tree is present")
    res = generate()
    with open(OUT, "w") as fh:
        json.dump(res, fh, indent=1)
    print(OUT, sum(len(r["files"]) for r in res["runs"]), "files")
