"""The benchmark sweep (benchmark.sh): grid, trimmed-mean aggregation, and a
run over a stand-in program on CPU; a small real sweep on the GPU."""
import os
import stat

import pytest

from lbmcl_gb300 import sweep


def _bash_grid_count(dims):
    """The loop bounds of benchmark.sh:60-100 counted independently."""
    lws = [1, 2, 4, 8, 16, 32, 64, 128]
    n = 0
    for d in dims:
        shapes = sum(1 for x in lws for y in lws for z in lws
                     if y <= x and z <= y and x * y * z <= 1024 and max(x, y, z) <= d)
        n += shapes * 6 + shapes
    return n


def test_reference_grid_matches_benchmark_sh():
    g = sweep.reference_grid()
    assert len(g) == _bash_grid_count((8, 16, 32, 64, 128))
    assert g[0] == (8, (1, 1, 1), 1)
    assert g[-1][2] == 128 ** 3  # the SoA pass comes last
    assert all(x >= y >= z and x * y * z <= 1024 and x <= d for d, (x, y, z), _ in g)


def test_aggregate_is_the_trimmed_mean():
    rows = [
        "GB300;single;64;50;0;032,001,001;262144;1;10;8;100;120",
        "GB300;single;64;50;0;032,001,001;262144;1;12;9;90;110",
        "GB300;single;64;50;0;032,001,001;262144;1;11;7;95;115",
        "GB300;single;64;50;0;032,001,001;262144;1;10;6;101;121",  # ties the min: first wins
        "GB300;single;64;50;0;064,001,001;262144;1;20;16;50;60",
        "GB300;single;64;50;0;064,001,001;262144;1;21;17;48;58",
        "GB300;single;64;50;0;064,001,001;262144;1;22;18;46;56",
    ]
    out = sweep.aggregate(rows)
    assert out[0] == "GB300;single;64;032,001,001;262144;10.5;6.5;98;118"
    assert out[1] == "GB300;single;64;064,001,001;262144;21;17;48;58"
    with pytest.raises(ValueError):
        sweep.aggregate(rows[:2] + rows[4:6])


def test_run_sweep_over_a_stand_in_program(tmp_path):
    fake = tmp_path / "lbmcl"
    fake.write_text('#!/bin/sh\n'
                    '# prints the statistics line of its -d and -w arguments\n'
                    'while [ $# -gt 0 ]; do case "$1" in -d) d=$2; shift;; -w) w=$2; shift;; esac; shift; done\n'
                    'echo "dev;single;$d;50;0;$w;$((d*d*d));1;5;4;3;2" 1>&2\n')
    fake.chmod(fake.stat().st_mode | stat.S_IEXEC)
    grid = [(16, (32, 1, 1), 16 ** 3), (16, (64, 1, 1), 16 ** 3)]
    lines = sweep.run_sweep(str(fake), grid, repeats=3, out_dir=str(tmp_path / "b"))
    assert lines == ["dev;single;16;32,1,1;4096;5;4;3;2", "dev;single;16;64,1,1;4096;5;4;3;2"]
    assert len((tmp_path / "b" / "stats.csv").read_text().splitlines()) == 6
    assert (tmp_path / "b" / "benchmark.csv").read_text().splitlines() == lines


@pytest.mark.gpu
def test_small_sweep_on_the_gpu(tmp_path, capi):
    from lbmcl_gb300 import build
    binary = build.build_host()
    grid = [(32, (32, 1, 1), 32 ** 3), (32, (8, 8, 2), 32 ** 3)]
    lines = sweep.run_sweep(binary, grid, precision="fp16", repeats=3, iterations=20, out_dir=str(tmp_path))
    assert len(lines) == 2
    for line in lines:
        f = line.split(";")
        assert f[2] == "32" and float(f[-1]) > 0 and float(f[-3]) > 0
