"""GPU path vs the FP64 oracle (and vs bskit's golden grid info), through the C ABI.

Tolerances (stated per test):
* shell mode counts and triangle counts: bit-exact integers;
* k_mean: 1e-12 relative (FP64 fields and sums on both sides);
* B: the GPU fields are FP32 (cuFFT C2R), the oracle's FP64.  For every bin we
  report rel = |B - B_o| / |B_o| and the conditioning-free
  nrm = |B - B_o| / (L^6/N^3 * sum_x |I_i I_j I_l|).  fp64/fp32 must meet
  nrm <= 2e-6 on every bin and bf16x3 nrm <= 4e-6 (each bf16 hi + lo pair
  represents its FP32 value to about 2^-18 relative, and on shells one k_f wide
  an exact emulation of the three bf16 products already reaches 2.0e-6); all
  three must meet rel <= 1e-5 on every bin whose value is at least 10% of its
  absolute sum (|B_o| >= 0.1 * abs sum; below that a 1e-6 normalised error is
  no longer a 1e-5 relative one), and a median rel <= 1e-5 over all bins;
  bf16 (one MMA term) must meet nrm <= 1e-3.
"""
import os

import numpy as np
import pytest
import torch

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from bskit_gb300.engine import Plan
from oracle import bispec_oracle as O

pytestmark = pytest.mark.gpu

TWO_PI = 2 * np.pi


def _cfg0():
    n, box = 64, 100.0
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=16 * kf, dk=3 * kf)
    return n, box, B.generate_bin_edge_list(**kw), B.generate_triangle_bin_list(return_indices=True, **kw)


def _small(n=32, box=100.0, dk=2, kmax_frac=0.25):
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=n * kmax_frac * kf, dk=dk * kf)
    return n, box, B.generate_bin_edge_list(**kw), B.generate_triangle_bin_list(return_indices=True, **kw)


def _abs_sums(fa, fb, fc, tri, box, n):
    return O.triple_sums(np.abs(fa), np.abs(fb), np.abs(fc), tri) * box ** 6 / n ** 3


def _check_b(b, bo, babs, prec):
    err = np.abs(b - bo)
    nrm = err / babs
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = err / np.abs(bo)  # inf / nan on bins with no closed triangle
    well = np.abs(bo) >= 0.1 * babs
    print("%s: max nrm %.3g, max rel(well-conditioned, %d/%d bins) %.3g, median rel %.3g" %
          (prec, nrm.max(), well.sum(), len(bo), rel[well].max() if well.any() else 0,
           np.median(rel)))
    if prec == "bf16":
        assert nrm.max() <= 1e-3
    else:
        assert nrm.max() <= (4e-6 if prec == "bf16x3" else 2e-6)
        assert np.median(rel) <= 1e-5
        if well.any():
            assert rel[well].max() <= 1e-5


@pytest.mark.parametrize("grid", ["native", "reduced"])
def test_mode_counts_exact(cuda, grid):
    for n, box, edges, _ in (_cfg0(), _small(32, 100.0, 2), _small(48, 77.0, 1, 0.5)):
        plan = Plan(n, box, edges, grid=grid)
        assert np.array_equal(plan.mode_counts(), O.shell_mode_counts(n, box, edges))
        plan.close()
    # golden P(k) N_modes 18, 62, 98, 210 at L = 1000
    kf = TWO_PI / 1000.0
    edges = np.array([[0.5 + i, 1.5 + i] for i in range(4)]) * kf
    plan = Plan(512, 1000.0, edges, grid="reduced")
    assert plan.ngrid < 512
    assert plan.mode_counts().tolist() == [18, 62, 98, 210]


def test_mode_counts_match_all_golden_pk_rows(cuda):
    # all 255 rows of bskit's P(k) golden file (shells [i + 0.5, i + 1.5] k_f at 512^3,
    # L = 1000, up to the Nyquist corner): the plan's exact counts on the full grid
    gold = np.loadtxt(os.path.join(os.path.dirname(__file__), "golden",
                                   "ps_nmodes_512.dat")).astype(np.int64)
    kf = TWO_PI / 1000.0
    edges = np.array([[0.5 + i, 1.5 + i] for i in range(len(gold))]) * kf
    plan = Plan(512, 1000.0, edges, grid="native")
    assert np.array_equal(plan.mode_counts(), gold)
    plan.close()


def test_gridinfo_matches_golden_text(cuda):
    up = dict(kmin=0.00314, kmax=0.1, dk=0.00628, num_lowk_bins=3, dk_high=0.01884)
    edges = B.generate_bin_edge_list(**up)
    tri = B.generate_triangle_bin_list(return_indices=True, **up)
    plan = Plan(512, 1000.0, edges, grid="reduced")  # the mesh size of the golden run
    ts = plan.triangles(tri)
    nt, km = plan.gridinfo(ts)
    plan.sync_check()
    nt, km = nt.cpu().numpy(), km.cpu().numpy()
    ed6 = B.triangle_indices_to_edges(edges, tri)
    rows = ['%d %e %e %e %e %e %e %e %e %e %e' % ((t,) + tuple(km[t]) + tuple(ed6[t]) + (nt[t],))
            for t in range(len(tri))]
    import os
    gold = open(os.path.join(os.path.dirname(__file__), "golden",
                             "Lbox1000_512_kf_3kf_3lowkbins.dat")).read().split("\n")[:len(rows)]
    assert rows == gold


@pytest.mark.parametrize("grid", ["native", "reduced"])
def test_gridinfo_exact_vs_oracle(cuda, grid):
    # edges at multiples of k_f: many modes sit exactly on shell edges
    n, box, edges, tri = _small(32, 100.0, 2)
    plan = Plan(n, box, edges, grid=grid)
    ts = plan.triangles(tri)
    nt, km = plan.gridinfo(ts)
    plan.sync_check()
    raw, nto, kmo = O.grid_info(n, box, edges, tri)
    assert np.array_equal(nt.cpu().numpy(), nto)
    km = km.cpu().numpy()
    ok = nto > 0
    assert np.all(np.isnan(km[~ok]))
    assert np.allclose(km[ok], kmo[ok], rtol=1e-12, atol=0)


@pytest.mark.parametrize("n", [32, 40, 48, 56, 96])
def test_fields_match_oracle_native(cuda, n):
    # 32 and 40: the field synthesis with run-time plans (16x2, 8x5); 48 and 96: compile-time
    # plans (16x3, 16x6) whose last pass writes the fields straight from registers; 56 = 8 x 7
    # has no synthesis plan and takes the filter + cuFFT C2R path
    n, box, edges, _ = _small(n, 100.0, 2)
    delta = synthetic.lognormal_mesh(n, box, seed=11)
    plan = Plan(n, box, edges, grid="native")
    plan.paint(0, torch.from_numpy(delta))
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    for s in range(len(edges)):
        f = plan.field(0, s).cpu().numpy().astype(np.float64)
        scale = np.abs(of[s]).max()
        assert np.abs(f - of[s]).max() <= 1e-5 * scale, s


def test_fields_match_oracle_native_192(cuda):
    # the compile-time 16 x 12 plan (the 256^3 workload's contraction grid), 5 shells
    n, box, edges, _ = _small(192, 100.0, 8, 0.25)
    delta = synthetic.lognormal_mesh(n, box, seed=13)
    plan = Plan(n, box, edges, grid="native")
    plan.paint(0, torch.from_numpy(delta))
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    for s in range(len(edges)):
        f = plan.field(0, s).cpu().numpy().astype(np.float64)
        scale = np.abs(of[s]).max()
        assert np.abs(f - of[s]).max() <= 1e-5 * scale, s


@pytest.mark.parametrize("n", [128, 160, 240, 256, 288, 320])
def test_fields_match_oracle_grid_level_sizes(cuda, n):
    # the compile-time plans that grid levels use besides 48 / 96 / 192 / 384 / 480
    # (16x8, 16x2x5, 16x3x5, 16x16, 16x6x3, 16x4x5), shells out to 0.45 N -- a level holds
    # shells of radius up to nearly half its side
    n, box, edges, _ = _small(n, 100.0, n // 12, 0.45)
    delta = synthetic.lognormal_mesh(n, box, seed=17)
    plan = Plan(n, box, edges, grid="native")
    plan.paint(0, torch.from_numpy(delta))
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    for s in range(len(edges)):
        f = plan.field(0, s).cpu().numpy().astype(np.float64)
        scale = np.abs(of[s]).max()
        assert np.abs(f - of[s]).max() <= 1e-5 * scale, s
    plan.close()


def test_fields_match_oracle_480(cuda):
    # the 1024^3 workload's reduced grid (16x6x5 plan, radix-5 last pass over 96 butterflies a
    # line); three shells out to radius 181, beyond the Z pass's register prefetch (128 q_c)
    n, box, edges, _ = _small(480, 100.0, 60, 0.45)
    assert len(edges) == 3
    delta = synthetic.lognormal_mesh_torch(n, box, seed=19, device=cuda).contiguous()
    plan = Plan(n, box, edges, grid="native")
    plan.paint(0, delta)
    got = [plan.field(0, s).cpu().numpy() for s in range(len(edges))]
    plan.sync_check()
    plan.close()
    host = delta.cpu().numpy()
    del delta
    torch.cuda.empty_cache()
    of = O.shell_fields(O.spectrum(host), n, box, edges)
    for s in range(len(edges)):
        scale = np.abs(of[s]).max()
        assert np.abs(got[s].astype(np.float64) - of[s]).max() <= 1e-5 * scale, s


def test_paint_keeps_input(cuda):
    n, box, edges, _ = _small(32, 100.0, 2)
    delta = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=12)).cuda()
    keep = delta.clone()
    plan = Plan(n, box, edges)
    plan.paint(0, delta)
    torch.cuda.synchronize()
    assert torch.equal(delta, keep)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3", "bf16"])
def test_auto_bispectrum_cfg0(cuda, prec):
    n, box, edges, tri = _cfg0()
    delta = synthetic.lognormal_mesh(n, box, seed=0)
    plan = Plan(n, box, edges, grid="reduced")
    plan.paint(0, torch.from_numpy(delta))
    ts = plan.triangles(tri)
    b = plan.measure_b(ts, precision=prec)
    plan.sync_check()
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    bo = O.triple_sums(of, of, of, tri) * box ** 6 / n ** 3
    _check_b(b.cpu().numpy(), bo, _abs_sums(of, of, of, tri, box, n), prec)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3"])
def test_auto_bispectrum_more_shells(cuda, prec):
    # 15 shells, 477 bins: several tensor-core tiles and column ranges
    n, box, edges, tri = _small(64, 100.0, 2, 0.25)
    delta = synthetic.lognormal_mesh(n, box, seed=4)
    plan = Plan(n, box, edges)
    plan.paint(0, torch.from_numpy(delta))
    ts = plan.triangles(tri)
    b = plan.measure_b(ts, precision=prec)
    plan.sync_check()
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    bo = O.triple_sums(of, of, of, tri) * box ** 6 / n ** 3
    _check_b(b.cpu().numpy(), bo, _abs_sums(of, of, of, tri, box, n), prec)


def test_contract_ragged_grid_matches_fp64(cuda):
    # K = 36^3 = 46656 is not a multiple of 128: the tensor-core path loads the sources with
    # per-quarter copies and the column operand from a split whose last chunk is half padding
    kf = TWO_PI / 100.0
    kw = dict(kmin=kf, kmax=16 * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = B.generate_triangle_bin_list(return_indices=True, **kw)
    n, K = len(edges), 36 ** 3
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    fs = [torch.randn((n, K), generator=g, device="cuda") for _ in range(3)]
    plan = Plan(64, 100.0, edges)
    ts = plan.triangles(tri)
    b64 = plan.contract(ts, *fs, precision="fp64").cpu().numpy()
    babs = plan.contract(ts, *[f.abs() for f in fs], precision="fp64").cpu().numpy()
    for prec, bound in (("bf16x3", 4e-6), ("bf16", 1e-3)):
        b = plan.contract(ts, *fs, precision=prec).cpu().numpy()
        assert np.all(np.isfinite(b))
        assert (np.abs(b - b64) / babs).max() <= bound, prec
    plan.sync_check()


def test_empty_set_and_single_shell(cuda):
    # an empty triangle list through every measuring entry point (torch hands out NULL
    # data pointers for empty tensors), then one shell and its one bin (0, 0, 0)
    n, box = 32, 100.0
    kf = TWO_PI / box
    edges = np.array([[2 * kf, 4 * kf]])
    delta = synthetic.lognormal_mesh(n, box, seed=14)
    plan = Plan(n, box, edges)
    plan.paint(0, torch.from_numpy(delta))
    empty = plan.triangles(np.zeros((0, 3), np.int32))
    assert empty.T == 0
    for prec in ("fp64", "fp32", "bf16x3", "bf16"):
        assert plan.measure_b(empty, precision=prec).numel() == 0
    nt, km = plan.gridinfo(empty)
    assert nt.numel() == 0 and tuple(km.shape) == (0, 3)
    f = torch.ones((1, 1024), device="cuda")
    assert plan.contract(empty, f, f, f).numel() == 0
    assert Plan.normalize(nt, nt).numel() == 0
    plan.sync_check()

    tri = np.array([[0, 0, 0]], np.int32)
    ts = plan.triangles(tri)
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    bo = O.triple_sums(of, of, of, tri) * box ** 6 / n ** 3
    babs = _abs_sums(of, of, of, tri, box, n)
    # one bin: the normalised bounds alone (a median over one bin is that bin's relative error)
    for prec, bound in (("fp64", 2e-6), ("fp32", 2e-6), ("bf16x3", 4e-6), ("bf16", 1e-3)):
        b = plan.measure_b(ts, precision=prec)
        plan.sync_check()
        assert (np.abs(b.cpu().numpy() - bo) / babs).max() <= bound, prec
    nt, km = plan.gridinfo(ts)
    plan.sync_check()
    _, nto, kmo = O.grid_info(n, box, edges, tri)
    assert np.array_equal(nt.cpu().numpy(), nto) and nto[0] > 0
    assert np.allclose(km.cpu().numpy(), kmo, rtol=1e-12, atol=0)


@pytest.mark.parametrize("prec", ["fp64", "bf16x3"])
def test_cross_bispectra(cuda, prec):
    n, box = 48, 100.0
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=12 * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    d1 = synthetic.lognormal_mesh(n, box, seed=21)
    d2 = synthetic.noisy_copy(d1, seed=22)
    d3 = synthetic.lognormal_mesh(n, box, seed=23)
    plan = Plan(n, box, edges)
    for s, d in enumerate((d1, d2, d3)):
        plan.paint(s, torch.from_numpy(d))
    f = [O.shell_fields(O.spectrum(d), n, box, edges) for d in (d1, d2, d3)]
    for nf, slots in ((2, (0, 0, 1)), (3, (0, 1, 2))):
        tri = B.generate_triangle_bin_list(num_fields=nf, return_indices=True, **kw)
        ts = plan.triangles(tri)
        b = plan.measure_b(ts, slots=slots, precision=prec)
        plan.sync_check()
        fa, fb, fc = (f[0], f[0], f[1]) if nf == 2 else (f[0], f[1], f[2])
        bo = O.triple_sums(fa, fb, fc, tri) * box ** 6 / n ** 3
        _check_b(b.cpu().numpy(), bo, _abs_sums(fa, fb, fc, tri, box, n), prec)


def test_reduced_grid_equals_native(cuda):
    n, box, edges, tri = _small(64, 100.0, 2, 0.25)
    delta = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=8))
    out = {}
    for grid in ("native", "reduced"):
        plan = Plan(n, box, edges, grid=grid)
        plan.paint(0, delta)
        out[grid] = plan.measure_b(plan.triangles(tri), precision="fp64").cpu().numpy()
        if grid == "reduced":
            assert plan.ngrid < n
    scale = np.abs(out["native"]).max()
    assert np.abs(out["native"] - out["reduced"]).max() <= 1e-6 * scale


def test_plane_wave_known_answer(cuda):
    n, box = 32, TWO_PI
    q = [np.array([3, 0, 0]), np.array([0, 2, 0]), np.array([-3, -2, 0])]
    phi, A = [0.3, -1.1, 0.5], 0.7
    x = np.arange(n) * box / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    delta = sum(A * np.cos(qa[0] * X + qa[1] * Y + qa[2] * Z + p) for qa, p in zip(q, phi))
    shells = np.array([[1.9, 2.1], [2.9, 3.1], [3.5, 3.7]])
    plan = Plan(n, box, shells)
    plan.paint(0, torch.from_numpy(delta.astype(np.float32)))
    ts = plan.triangles([[1, 0, 2]])
    expect = box ** 6 * A ** 3 * np.cos(sum(phi)) / 4.0
    for prec in ("fp64", "fp32", "bf16x3"):
        b = plan.measure_b(ts, precision=prec).cpu().numpy()[0]
        assert abs(b - expect) <= 1e-5 * abs(expect), prec


def test_brute_force_known_answer(cuda):
    n, box = 16, 50.0
    kf = TWO_PI / box
    delta = synthetic.lognormal_mesh(n, box, seed=3)
    shells = np.array([[0.5, 2.5], [1.5, 3.5], [2.5, 4.5]]) * kf
    plan = Plan(n, box, shells)
    plan.paint(0, torch.from_numpy(delta))
    tri = np.array([[2, 1, 1], [2, 1, 0], [1, 1, 1]])
    ts = plan.triangles(tri)
    nt, km = plan.gridinfo(ts)
    b = plan.measure_b(ts, precision="fp64")
    Bn = plan.normalize(b, nt).cpu().numpy()
    nt = nt.cpu().numpy()
    for t, (i, j, l) in enumerate(tri):
        Bd, Nd, k1, k2, k3 = O.bk_binned(delta.astype(np.float64), box, shells[i], shells[j],
                                         shells[l])
        assert nt[t] == Nd
        assert abs(Bn[t] - Bd.real) <= 1e-5 * abs(Bd.real)


def test_duplicate_and_unordered_triangles(cuda):
    n, box, edges, tri = _small(32, 100.0, 2)
    delta = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=9))
    plan = Plan(n, box, edges)
    plan.paint(0, delta)
    base = plan.measure_b(plan.triangles(tri), precision="fp64").cpu().numpy()
    perm = tri[:, [2, 0, 1]]
    dup = np.concatenate([tri[:5], tri[:5], perm[:5]])
    b = plan.measure_b(plan.triangles(dup), precision="fp64").cpu().numpy()
    assert np.allclose(b[:5], base[:5], rtol=1e-12)
    assert np.allclose(b[5:10], base[:5], rtol=1e-12)
    assert np.allclose(b[10:15], base[:5], rtol=1e-9)


def test_slab_ranges_sum_to_whole(cuda):
    n, box, edges, tri = _small(64, 100.0, 2, 0.25)
    delta = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=10))
    plan = Plan(n, box, edges)
    plan.paint(0, delta)
    ts = plan.triangles(tri)
    K = plan.ngrid ** 3
    slab = plan.ngrid ** 2
    for prec in ("fp64", "bf16x3"):
        whole = plan.measure_b(ts, precision=prec).cpu().numpy()
        cut = (plan.ngrid // 3) * slab // 128 * 128
        parts = [plan.measure_b_range(ts, 0, cut, precision=prec),
                 plan.measure_b_range(ts, cut, K, precision=prec)]
        tot = sum(p.cpu().numpy() for p in parts)
        # a different slab cut changes only the FP32 accumulation order of the tensor path
        tol = 1e-12 if prec == "fp64" else 1e-6
        assert np.abs(tot - whole).max() <= tol * np.abs(whole).max(), prec


def test_empty_point_range_is_zero(cuda):
    # a rank whose share of the grid is empty (more ranks than 128-point stages) adds zeros
    n, box, edges, tri = _small(32, 100.0, 2)
    plan = Plan(n, box, edges)
    plan.paint(0, torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=15)))
    ts = plan.triangles(tri)
    for prec in ("fp64", "fp32", "bf16x3"):
        out = torch.full((len(tri),), 7.0, dtype=torch.float64, device="cuda")
        plan.measure_b_range(ts, 256, 256, precision=prec, out=out)
        plan.sync_check()
        assert torch.count_nonzero(out).item() == 0, prec


def test_more_than_64_shells(cuda):
    # 80 shells: a pair whose third shells span more than a tile's 64 columns becomes several
    # GEMM rows, and a pair 65 shells apart takes two source ranges; the tensor-core
    # contraction of random fields against the FP64 one of the same fields
    n_sh, K = 80, 24 ** 3
    kf = TWO_PI / 100.0
    edges = np.array([[0.3 * s, 0.3 * s + 0.3] for s in range(n_sh)]) * kf
    tri = ([(79, 79, l) for l in range(n_sh)] + [(70, 5, l) for l in range(0, n_sh, 2)] +
           [(10, 12, l) for l in range(0, n_sh, 7)] + [(0, 0, 0)])
    tri = np.array(tri, dtype=np.int32)
    plan = Plan(64, 100.0, edges)
    ts = plan.triangles(tri)
    tiles, sum_nc, rows = ts.schedule()
    assert rows == 7 and sum_nc <= 64 * tiles  # (79,79), (70,5), (10,12): two runs each
    g = torch.Generator(device="cuda")
    g.manual_seed(16)
    fs = [torch.randn((n_sh, K), generator=g, device="cuda") for _ in range(3)]
    b64 = plan.contract(ts, *fs, precision="fp64").cpu().numpy()
    babs = plan.contract(ts, *[f.abs() for f in fs], precision="fp64").cpu().numpy()
    want = np.array([np.dot(fs[0][i].double().cpu().numpy() * fs[1][j].double().cpu().numpy(),
                            fs[2][l].double().cpu().numpy()) for i, j, l in tri])
    assert np.abs(b64 - want).max() <= 1e-12 * babs.max()
    for prec, bound in (("bf16x3", 4e-6), ("bf16", 1e-3)):
        b = plan.contract(ts, *fs, precision=prec).cpu().numpy()
        assert np.all(np.isfinite(b))
        assert (np.abs(b - b64) / babs).max() <= bound, prec
    plan.sync_check()


def test_schedule_covers_every_pair(cuda):
    n, box, edges, tri = _small(64, 100.0, 2, 0.25)
    plan = Plan(n, box, edges)
    tiles, sum_nc, rows = plan.triangles(tri).schedule()
    pairs = {(int(i), int(j)) for i, j, _ in tri}
    assert rows == len(pairs)
    assert tiles >= -(-rows // 128) and sum_nc % 8 == 0
    assert len(tri) <= 128 * sum_nc
    plan.close()


def test_mem_budget_refuses_before_allocating(cuda):
    from bskit_gb300 import _lib
    n, box, edges, tri = _small(32, 100.0, 2)
    delta = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=21)).cuda()
    free = Plan(n, box, edges)
    free.paint(0, delta)
    ref = free.measure_b(free.triangles(tri)).cpu().numpy()
    need = free.footprint()
    free.close()
    tight = Plan(n, box, edges, mem_budget=need // 2)
    tight.paint(0, delta)
    ts = tight.triangles(tri)
    before = tight.footprint()
    with pytest.raises(_lib.BskError) as e:
        tight.measure_b(ts)
    assert e.value.code == _lib.BSK_ERR_OOM and "budget" in str(e.value)
    assert tight.footprint() == before  # nothing was allocated
    tight.close()
    roomy = Plan(n, box, edges, mem_budget=need)
    roomy.paint(0, delta)
    # same kernels; only the order of the FP64 atomic sums may differ
    np.testing.assert_allclose(roomy.measure_b(roomy.triangles(tri)).cpu().numpy(), ref,
                               rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    roomy.close()


def _streaming_case():
    # 30 shells of width k_f up to 31 k_f on a 64^3 mesh (native grid): 4 streamed chunks
    n, box = 64, 100.0
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=32 * kf, dk=kf)
    return n, box, kw, B.generate_bin_edge_list(**kw)


@pytest.mark.parametrize("prec,roomy", [("fp32", False), ("bf16x3", False), ("bf16x3", True)])
def test_shell_streaming_under_budget(cuda, prec, roomy):
    n, box, kw, edges = _streaming_case()
    d1 = synthetic.lognormal_mesh(n, box, seed=31)
    d2 = synthetic.noisy_copy(d1, seed=32)
    probe = Plan(n, box, edges)
    probe.paint(0, torch.from_numpy(d1))
    probe.paint(1, torch.from_numpy(d2))
    base = probe.footprint()
    k = probe.ngrid ** 3
    probe.close()
    # room for one 8-shell chunk of three FP32 fields (+ the bf16 split), not for the
    # 30 shells (32 with the FFT-batch padding) of one slot resident; the tight budget
    # leaves no room for the field-synthesis workspace (chunks come from the cuFFT path),
    # the roomy one, just below the resident need, does
    room = 8 * k * (16 if prec == "bf16x3" else 12) + (1 << 20)
    if roomy:
        room = 32 * k * 8 - (4 << 20)
    plan = Plan(n, box, edges, mem_budget=base + room)
    plan.paint(0, torch.from_numpy(d1))
    plan.paint(1, torch.from_numpy(d2))
    f = [O.shell_fields(O.spectrum(d), n, box, edges) for d in (d1, d2)]
    for nf, slots in ((1, (0, 0, 0)), (2, (0, 0, 1))):
        tri = B.generate_triangle_bin_list(num_fields=nf, return_indices=True, **kw)
        b = plan.measure_b(plan.triangles(tri), slots=slots, precision=prec)
        plan.sync_check()
        assert plan.stream_chunk() == 8
        fa, fb, fc = (f[0], f[0], f[0]) if nf == 1 else (f[0], f[0], f[1])
        bo = O.triple_sums(fa, fb, fc, tri) * box ** 6 / n ** 3
        _check_b(b.cpu().numpy(), bo, _abs_sums(fa, fb, fc, tri, box, n), prec)
    assert plan.footprint() <= base + room
    plan.close()


def test_gridinfo_streaming_under_budget(cuda):
    n, box, kw, edges = _streaming_case()
    tri = B.generate_triangle_bin_list(return_indices=True, **kw)
    full = Plan(n, box, edges)
    ts = full.triangles(tri)
    ntri0, kmean0 = (x.cpu().numpy() for x in full.gridinfo(ts))
    base = full.footprint()
    k = full.ngrid ** 3
    full.close()
    spec = 8 * k // n * (n // 2 + 1) * 16
    # one 8-shell chunk of six FP64 fields, not the resident 2 x 32 shells
    plan = Plan(n, box, edges, mem_budget=base + 8 * 6 * 8 * k + spec + (1 << 20))
    ts = plan.triangles(tri)
    ntri, kmean = (x.cpu().numpy() for x in plan.gridinfo(ts))
    plan.sync_check()
    assert plan.stream_chunk() == 8
    assert np.array_equal(ntri, ntri0)
    ok = ntri0 > 0
    # the streamed groups sum the FP64 products in another order than the resident tiles
    np.testing.assert_allclose(kmean[ok], kmean0[ok], rtol=1e-11)
    assert np.isnan(kmean[~ok]).all()
    plan.close()
    # a budget below one chunk is refused before allocating
    from bskit_gb300 import _lib
    tight = Plan(n, box, edges, mem_budget=base + 4 * 6 * 8 * k)
    with pytest.raises(_lib.BskError) as e:
        tight.gridinfo(tight.triangles(tri))
    assert e.value.code == _lib.BSK_ERR_OOM
    tight.close()


def test_cic_compensated_paint(cuda):
    n, box, edges, tri = _small(32, 100.0, 2)
    delta = synthetic.lognormal_mesh(n, box, seed=31)
    plan = Plan(n, box, edges)
    plan.paint(0, torch.from_numpy(delta), cic_nmesh=64)
    ts = plan.triangles(tri)
    b = plan.measure_b(ts, precision="fp64").cpu().numpy()
    of = O.shell_fields(O.cic_compensate(O.spectrum(delta), n, 64), n, box, edges)
    bo = O.triple_sums(of, of, of, tri) * box ** 6 / n ** 3
    babs = _abs_sums(of, of, of, tri, box, n)
    assert np.max(np.abs(b - bo) / babs) <= 2e-6
    plain = Plan(n, box, edges)
    plain.paint(0, torch.from_numpy(delta))
    b0 = plain.measure_b(plain.triangles(tri), precision="fp64").cpu().numpy()
    assert np.max(np.abs(b0 - b) / babs) > 1e-4  # the window correction is not a no-op
