"""The contraction schedule's host tiler (bskit_gb300/csrc/bsk_schedule.cu), no GPU.

The tiler's own source is compiled with ``schedule_harness.cu``, whose wrapped
cudaMalloc / cudaMemcpy / cudaFree keep the schedule in host memory.  Every tile must fit
the tensor-core kernel (at most 64 column shells and 64 shells per pair-factor range,
128 rows), and every triangle must sit in exactly one map entry whose row and column are
its own (i, j, l).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from bskit_gb300 import bins as B

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("sched") / "schedule_harness")
    cmd = [nvcc, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "bskit_gb300", "csrc"),
           "-Xlinker", "--wrap=cudaMalloc", "-Xlinker", "--wrap=cudaMemcpy",
           "-Xlinker", "--wrap=cudaFree",
           os.path.join(HERE, "schedule_harness.cu"),
           os.path.join(ROOT, "bskit_gb300", "csrc", "bsk_schedule.cu"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def schedule(exe, tmp_path, n, tri):
    tri = np.asarray(tri, dtype=int).reshape(-1, 3)
    path = tmp_path / "tri.txt"
    with open(path, "w") as f:
        f.write("%d %d\n" % (n, len(tri)))
        f.writelines("%d %d %d\n" % tuple(t) for t in tri)
    out = subprocess.run([exe, str(path)], check=True, capture_output=True,
                         text=True).stdout.splitlines()
    assert not out[0].startswith("error"), out[0]
    keys = ("i0", "j0", "l0", "ni", "nj", "nc", "nrows", "row_off", "map_off")
    tiles = [dict(zip(keys, map(int, line.split()[1:]))) for line in out
             if line.startswith("tile ")]
    rows = np.array([line.split()[1:] for line in out if line.startswith("r ")], dtype=int)
    cmap = np.array([line.split()[1] for line in out if line.startswith("m ")], dtype=int)
    # every tile fits the kernel, every triangle is in exactly one entry, at its own place
    seen = np.zeros(len(tri), dtype=int)
    for d in tiles:
        assert d["nc"] % 8 == 0 and 8 <= d["nc"] <= 64
        assert d["ni"] <= 64 and d["nj"] <= 64 and 1 <= d["nrows"] <= 128
        for c in range(d["nc"]):
            for r in range(128):
                t = cmap[d["map_off"] + c * 128 + r]
                if t < 0:
                    continue
                assert r < d["nrows"]
                seen[t] += 1
                i, j = rows[d["row_off"] + r]
                assert (i, j, d["l0"] + c) == tuple(tri[t])
                assert d["i0"] <= i < d["i0"] + d["ni"] and d["j0"] <= j < d["j0"] + d["nj"]
    assert np.all(seen == 1)
    return tiles


def test_headline_schedule(harness, tmp_path):
    # 512^3 all-triangle auto binning: 63 shells, 24 305 bins -> 1 086 pair rows in 9 tiles
    kf = 2 * np.pi / 1000.0
    kw = dict(kmin=kf, kmax=128 * kf, dk=2 * kf)
    tiles = schedule(harness, tmp_path, 63, B.generate_triangle_bin_list(return_indices=True,
                                                                          **kw))
    assert len(tiles) == 9
    assert sum(d["nrows"] for d in tiles) == 1086 and sum(d["nc"] for d in tiles) == 352


@pytest.mark.parametrize("num_fields", [2, 3])
def test_cross_lists(harness, tmp_path, num_fields):
    kf = 2 * np.pi / 1000.0
    kw = dict(kmin=kf, kmax=32 * kf, dk=2 * kf)
    schedule(harness, tmp_path, 15, B.generate_triangle_bin_list(
        num_fields=num_fields, return_indices=True, **kw))


def test_more_than_64_shells_cut_rows(harness, tmp_path):
    # 126 shells (dk = k_f to k_Nyq/2 at 512^3): pairs whose third shells span up to 126
    # shells are cut into runs of at most 64
    kf = 2 * np.pi / 1000.0
    kw = dict(kmin=kf, kmax=128 * kf, dk=kf)
    n = len(B.generate_bin_edge_list(**kw))
    assert n == 126
    tri = B.generate_triangle_bin_list(return_indices=True, **kw)
    tiles = schedule(harness, tmp_path, n, tri)
    pairs = {(i, j) for i, j, _ in np.asarray(tri).reshape(-1, 3)}
    assert sum(d["nrows"] for d in tiles) > len(pairs)
    # the GPU test's list: (79, 79) and (70, 5) and (10, 12) two runs each, (0, 0) one
    tri80 = ([(79, 79, l) for l in range(80)] + [(70, 5, l) for l in range(0, 80, 2)] +
             [(10, 12, l) for l in range(0, 80, 7)] + [(0, 0, 0)])
    assert sum(d["nrows"] for d in schedule(harness, tmp_path, 80, tri80)) == 7


def level_choice(exe, tmp_path, shell_r, sides, tri):
    tri = np.asarray(tri, dtype=int).reshape(-1, 3)
    path = tmp_path / "lev.txt"
    with open(path, "w") as f:
        f.write("%d %d %d\n" % (len(shell_r), len(tri), len(sides)))
        f.write(" ".join(map(str, shell_r)) + "\n" + " ".join(map(str, sides)) + "\n")
        f.writelines("%d %d %d\n" % tuple(t) for t in tri)
    out = subprocess.run([exe, "levels", str(path)], check=True, capture_output=True,
                         text=True).stdout.splitlines()
    assert not out[0].startswith("error"), out[0]
    lev = np.array([int(line.split()[2]) for line in out if line.startswith("lev ")])
    cost = {(int(a), int(b)): float(c) for _, a, b, c in
            (line.split() for line in out if line.startswith("cost "))}
    return lev, cost


def _chain_cost(cost, chosen):
    prev, total = -1, 0.0
    for j in sorted(chosen):
        total += cost[(prev, j)]
        prev = j
    return total


@pytest.mark.parametrize("case", ["headline", "mesh256", "cross256"])
def test_grid_level_sides_exact_and_cheapest(harness, tmp_path, case):
    # the level choice of the plan's resident contraction (bsk_triset_create): every bin on a
    # side above max(r_i + r_j + r_l, 2 max r) -- exact -- on the smallest chosen such side,
    # and the chosen chain as cheap as any subset of the candidate sides
    import itertools
    import math
    n, box, kmax, nf, top = {"headline": (512, 1000.0, 128, 1, 384),
                             "mesh256": (256, 500.0, 64, 1, 192),
                             "cross256": (256, 500.0, 64, 2, 192)}[case]
    kf = 2 * math.pi / box
    kw = dict(kmin=kf, kmax=kmax * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = np.unique(B.generate_triangle_bin_list(num_fields=nf, return_indices=True, **kw), axis=0)
    r = [int(np.floor(hi / kf * (1.0 + 1e-9))) for _, hi in edges]
    sides = [s for s in (48, 96, 128, 160, 192, 240, 256, 288, 320, 384, 480) if s < top] + [top]
    lev, cost = level_choice(harness, tmp_path, r, sides, tri)
    v = np.array([max(r[a] + r[b] + r[c], 2 * max(r[a], r[b], r[c])) for a, b, c in tri])
    side = np.array(sides)[lev]
    assert np.all(side > v)
    chosen = sorted(set(lev.tolist()))
    for t in range(len(tri)):  # no smaller chosen side holds the bin
        assert not any(sides[k] > v[t] and sides[k] < side[t] for k in chosen)
    best = min(_chain_cost(cost, list(sub) + [len(sides) - 1])
               for k in range(len(sides)) for sub in itertools.combinations(range(len(sides) - 1), k))
    assert _chain_cost(cost, chosen) <= best * (1 + 1e-12)
