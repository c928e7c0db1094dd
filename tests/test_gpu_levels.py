"""Grid levels: bins of small shells contracted on smaller grids, against the single
reduced grid of the same plan parameters.

A bin (i, j, l) is exact on any grid of side Ng > r_i + r_j + r_l whose Nyquist range holds
its shells (2 r < Ng), r the largest |q_c| of a shell mode: the sum over the grid of three
band-limited fields picks exactly the closed triangles q1 + q2 + q3 = 0, none of which can
wrap around.  So the levelled measurement equals the single-grid one up to rounding.  Each grid's FP32
fields carry their own FFT rounding, so even FP64 contractions agree only to that floor:
the bound is the oracle tests' FP64 bound, 2e-6 of the bin's absolute sum, and for bf16x3
that plus its own bound (tests/test_gpu_parity.py, 4e-6).
"""
import os

import numpy as np
import pytest
import torch

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from bskit_gb300.engine import Plan
from bskit_gb300.serving import bin_lists

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


def _case(n, box, kmax_kf, dk_kf, num_fields=1):
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=kmax_kf * kf, dk=dk_kf * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = B.generate_triangle_bin_list(num_fields=num_fields, return_indices=True, **kw)
    return edges, np.ascontiguousarray(tri, dtype=np.int32)


def _abs_sum(plan, ts, box, slots):
    ng = plan.ngrid
    absf = [torch.stack([plan.field(s, k).abs().reshape(-1) for k in range(plan.n_shells)])
            for s in sorted(set(slots))]
    f = {s: absf[i] for i, s in enumerate(sorted(set(slots)))}
    return (plan.contract(ts, f[slots[0]], f[slots[1]], f[slots[2]], precision="fp64")
            * (box ** 6 / float(ng) ** 3)).cpu().numpy()


@pytest.fixture
def small_levels():
    """Levels of any side: the default rule keeps only sides with >= 40% of the plan grid's
    points (relative rounding errors within 1.6x); these tests want the small ones too."""
    old = os.environ.get("BSK_LEVEL_MIN_POINTS")
    os.environ["BSK_LEVEL_MIN_POINTS"] = "0"
    yield
    if old is None:
        del os.environ["BSK_LEVEL_MIN_POINTS"]
    else:
        os.environ["BSK_LEVEL_MIN_POINTS"] = old


def _shell_r(edges, box):
    kf = TWO_PI / box
    return [int(np.floor(hi / kf * (1.0 + 1e-9))) for _, hi in edges]


@pytest.mark.parametrize("n,box,kmax_kf,num_fields", [(128, 250.0, 32, 1), (256, 500.0, 64, 1),
                                                       (256, 500.0, 64, 2)])
def test_levels_equal_the_single_grid(cuda, small_levels, n, box, kmax_kf, num_fields):
    edges, tri = _case(n, box, kmax_kf, 2, num_fields)
    slots = (0, 0, 1) if num_fields == 2 else (0, 0, 0)
    lev = Plan(n, box, edges)              # grid levels
    one = Plan(n, box, edges, grid="single")
    assert lev.ngrid == one.ngrid
    ts_l, ts_1 = lev.triangles(tri), one.triangles(tri)
    levels = ts_l.levels()
    assert ts_1.levels() == [] and len(levels) >= 1
    # 128^3 (grid 96): the only smaller side, 48, does not pay; 256^3 (grid 192) takes levels
    if n >= 256:
        assert len(levels) >= 2 and levels[0]["ngrid"] < lev.ngrid
    assert sum(lv["bins"] for lv in levels) == len(np.unique(tri, axis=0))
    assert levels[-1]["ngrid"] <= lev.ngrid
    # the assignment rule, restated: every bin on the smallest chosen side that holds it
    r = _shell_r(edges, box)
    sides = [lv["ngrid"] for lv in levels]
    if sides[-1] != lev.ngrid:
        sides.append(lev.ngrid)
    count = dict.fromkeys(sides, 0)
    for t in np.unique(tri, axis=0):
        need, big = sum(r[s] for s in t), max(r[s] for s in t)
        count[next(L for L in sides if need < L and 2 * big < L)] += 1
    assert [count[lv["ngrid"]] for lv in levels] == [lv["bins"] for lv in levels]

    for seed in (1, 2):  # a repaint re-takes every level's spectrum from the plan's
        d1 = synthetic.lognormal_mesh_torch(n, box, seed=seed, device=cuda).contiguous()
        meshes = [d1]
        if num_fields == 2:
            meshes.append((1.5 * d1 + 0.3 * torch.randn_like(d1)).contiguous())
        for p in (lev, one):
            for s, m in enumerate(meshes):
                p.paint(s, m)
        b64_l = lev.measure_b(ts_l, slots=slots, precision="fp64").cpu().numpy()
        b64_1 = one.measure_b(ts_1, slots=slots, precision="fp64").cpu().numpy()
        bx3_l = lev.measure_b(ts_l, slots=slots, precision="bf16x3").cpu().numpy()
        babs = _abs_sum(one, ts_1, box, slots)
        lev.sync_check()
        one.sync_check()
        live = babs > 0
        nrm64 = (np.abs(b64_l - b64_1) / np.where(live, babs, 1.0))[live]
        nrmx3 = (np.abs(bx3_l - b64_1) / np.where(live, babs, 1.0))[live]
        print("levels %s: fp64 max normalised diff %.3g, bf16x3 %.3g"
              % ([lv["ngrid"] for lv in levels], nrm64.max(), nrmx3.max()))
        assert nrm64.max() <= 2e-6
        assert nrmx3.max() <= 6e-6
    lev.close()
    one.close()


def test_level_point_ranges_sum_to_the_whole(cuda, small_levels):
    n, box = 256, 500.0
    edges, tri = _case(n, box, 64, 2)
    p = Plan(n, box, edges)
    ts = p.triangles(tri)
    assert len(ts.levels()) >= 2
    p.paint(0, synthetic.lognormal_mesh_torch(n, box, seed=3, device=cuda).contiguous())
    K = p.ngrid ** 3
    cuts = [0, 128 * (K // 128 // 3), 128 * (2 * K // 128 // 3), K]
    # FP64 sums regroup exactly enough for 1e-12; bf16x3's FP32 slice sums regroup at ~1e-7
    for prec, tol in (("fp64", 1e-12), ("bf16x3", 1e-6)):
        whole = p.measure_b(ts, precision=prec).cpu().numpy()
        parts = sum(p.measure_b_range(ts, a, b, precision=prec).cpu().numpy()
                    for a, b in zip(cuts[:-1], cuts[1:]))
        p.sync_check()
        assert np.abs(parts - whole).max() <= tol * np.abs(whole).max(), prec
    p.close()


def test_default_levels_keep_most_of_the_grid(cuda):
    # the 512^3 headline binning: every level keeps >= 40% of the plan grid's points
    n, box = 512, 1000.0
    edges, tri = _case(n, box, 128, 2)
    p = Plan(n, box, edges)
    levels = p.triangles(tri).levels()
    assert levels and levels[-1]["ngrid"] == p.ngrid
    assert all(lv["ngrid"] ** 3 >= 0.4 * p.ngrid ** 3 for lv in levels)
    assert sum(lv["bins"] for lv in levels) == len(tri)
    p.close()


@pytest.mark.parametrize("kind,num_fields", [("equilateral", 1), ("isosceles", 1),
                                             ("squeezed", 1), ("equilateral", 2),
                                             ("squeezed", 2)])
@pytest.mark.parametrize("min_points", ["0", None])
def test_bin_sets_on_levels_equal_the_single_grid(cuda, kind, num_fields, min_points):
    # the serving mix's bin sets (auto and cross) on grid levels, with the default 40% rule
    # and with levels of any side
    n, box = 256, 500.0
    kf = TWO_PI / box
    spec = dict(kmin=kf, kmax=64 * kf, dk=2 * kf, triangle_type=kind, squeezed_bin_index=0)
    edges, tri = bin_lists(spec, num_fields)
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    slots = (0, 0, 1) if num_fields == 2 else (0, 0, 0)
    old = os.environ.get("BSK_LEVEL_MIN_POINTS")
    if min_points is not None:
        os.environ["BSK_LEVEL_MIN_POINTS"] = min_points
    try:
        lev = Plan(n, box, edges)
        ts_l = lev.triangles(tri)
    finally:
        if old is None:
            os.environ.pop("BSK_LEVEL_MIN_POINTS", None)
        else:
            os.environ["BSK_LEVEL_MIN_POINTS"] = old
    one = Plan(n, box, edges, grid="single")
    ts_1 = one.triangles(tri)
    d1 = synthetic.lognormal_mesh_torch(n, box, seed=5, device=cuda).contiguous()
    meshes = [d1] if num_fields == 1 else [d1, (0.7 * d1 + 0.2 * torch.randn_like(d1))]
    for p in (lev, one):
        for s_, m in enumerate(meshes):
            p.paint(s_, m.contiguous())
    b64_1 = one.measure_b(ts_1, slots=slots, precision="fp64").cpu().numpy()
    babs = _abs_sum(one, ts_1, box, slots)
    live = babs > 0
    for prec, bound in (("fp64", 2e-6), ("bf16x3", 6e-6)):
        b = lev.measure_b(ts_l, slots=slots, precision=prec).cpu().numpy()
        lev.sync_check()
        assert np.all(np.abs(b - b64_1)[live] <= bound * babs[live]), (prec, ts_l.levels())
    lev.close()
    one.close()
