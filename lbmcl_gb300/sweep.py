"""The reference's benchmark sweep (benchmark.sh:1-176) over the lbmcl program.

For every (dim, work-group shape, stride) of a grid, the program runs
`repeats` times with `-o`; the ';'-separated statistics line each run prints
on stderr (lbmcl.hpp:648-669) is appended to stats.csv, and benchmark.csv gets
one line per configuration: the key device;precision;dim;work-group;stride
followed by the trimmed means of total time, kernels time, total MLUPS and
kernels MLUPS, the run with the smallest and the one with the largest total
time left out (benchmark.sh:111-176).

    python -m lbmcl_gb300.sweep [--precision fp32] [--grid gb300|reference] [--out DIR]

Grids:
  reference  benchmark.sh's own: dim 8..128, work-group x >= y >= z from
             {1, 2, ..., 128} with x*y*z <= 1024 and each <= dim, strides
             1..128, then the same shapes with stride dim^3 (SoA); 10 runs
             each, 50 iterations.
  gb300      the sizes this implementation is run at: dim 128, 256, 512;
             blocks of 32..256 threads; stride dim^3 (the population layout
             on the device does not depend on the stride, which shapes the f
             dumps only); 5 runs each, 50 iterations.
The work-group shape reaches the device as a block of x*y*z threads (rounded
down to a multiple of 32, clamped to 32..256).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

LWS = (1, 2, 4, 8, 16, 32, 64, 128)
STRIDES = (1, 8, 16, 32, 64, 128)


def reference_grid(dims=(8, 16, 32, 64, 128)):
    """(dim, (x, y, z), stride) in benchmark.sh's loop order (:60-100)."""
    def shapes(d):
        for x in LWS:
            for y in LWS:
                if y > x:
                    continue
                for z in LWS:
                    if z <= y and x * y * z <= 1024 and x <= d and y <= d and z <= d:
                        yield (x, y, z)
    out = []
    for d in dims:
        for w in shapes(d):
            for s in STRIDES:
                out.append((d, w, s))
    for d in dims:
        for w in shapes(d):
            out.append((d, w, d ** 3))
    return out


def gb300_grid(dims=(128, 256, 512)):
    return [(d, (b, 1, 1), d ** 3) for d in dims for b in (32, 64, 128, 256)]


def aggregate(lines):
    """benchmark.sh:111-176 over stats lines: per key ($1;$2;$3;$6;$7) the sum
    of columns 9-12 minus the row with the smallest and the row with the
    largest column 9 (first occurrence wins ties), divided by count - 2.
    Keys come out in order of first appearance; numbers as awk prints them
    (%.6g)."""
    groups = {}
    for line in lines:
        f = line.strip().split(";")
        if len(f) < 12:
            continue
        key = ";".join((f[0], f[1], f[2], f[5], f[6]))
        vals = [float(v) for v in f[8:12]]
        g = groups.get(key)
        if g is None:
            groups[key] = g = {"n": 0, "sum": [0.0] * 4, "min": vals, "max": vals}
        g["n"] += 1
        g["sum"] = [a + b for a, b in zip(g["sum"], vals)]
        if g["min"][0] > vals[0]:
            g["min"] = vals
        if g["max"][0] < vals[0]:
            g["max"] = vals
    out = []
    for key, g in groups.items():
        n = g["n"] - 2
        if n <= 0:
            raise ValueError(f"{key}: {g['n']} runs; the trimmed mean needs at least 3")
        means = [(s - lo - hi) / n for s, lo, hi in zip(g["sum"], g["min"], g["max"])]
        out.append(key + ";" + ";".join("%.6g" % m for m in means))
    return out


def run_sweep(binary, grid, precision="fp32", repeats=10, iterations=50, viscosity=0.0089, velocity=0.05,
              out_dir="benchmarks", timeout=600, log=None):
    """Run the grid; returns the benchmark.csv lines.  stats.csv and
    benchmark.csv are (re)written in out_dir, as benchmark.sh does."""
    os.makedirs(out_dir, exist_ok=True)
    stats = os.path.join(out_dir, "stats.csv")
    bench = os.path.join(out_dir, "benchmark.csv")
    for p in (stats, bench):
        if os.path.exists(p):
            os.remove(p)
    prec = ["-F"] if precision == "fp64" else ["--precision", precision]
    with open(stats, "a") as st:
        for d, (x, y, z), s in grid:
            for _ in range(repeats):
                cmd = [binary, "-d", str(d), "-n", str(viscosity), "-u", str(velocity), "-i", str(iterations),
                       "-e", "0", "-w", f"{x},{y},{z}", "-s", str(s), "-o", *prec]
                r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
                if r.returncode != 0:  # benchmark.sh runs under set -e
                    raise RuntimeError(f"{' '.join(cmd)} exited {r.returncode}: {r.stderr.strip()[-400:]}")
                st.write(r.stderr)
                st.flush()
                if log is not None:
                    log.write(r.stderr)
    with open(stats) as st:
        lines = aggregate(st.readlines())
    with open(bench, "w") as fh:
        fh.write("".join(line + "\n" for line in lines))
    return lines


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--precision", default="fp32", choices=("fp32", "fp64", "fp16", "bf16"))
    ap.add_argument("--grid", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--dims", default="", help="comma-separated dims replacing the grid's")
    ap.add_argument("--repeats", type=int, default=0, help="runs per configuration (>= 3)")
    ap.add_argument("--iterations", type=int, default=50)
    ap.add_argument("--out", default="benchmarks")
    ap.add_argument("--binary", default="")
    a = ap.parse_args(argv)
    dims = tuple(int(v) for v in a.dims.split(",")) if a.dims else None
    if a.grid == "reference":
        grid = reference_grid(dims) if dims else reference_grid()
        repeats = a.repeats or 10
    else:
        grid = gb300_grid(dims) if dims else gb300_grid()
        repeats = a.repeats or 5
    binary = a.binary
    if not binary:
        from . import build
        binary = build.build_host()
    lines = run_sweep(binary, grid, a.precision, repeats, a.iterations, out_dir=a.out)
    sys.stdout.write("".join(line + "\n" for line in lines))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
