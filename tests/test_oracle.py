"""Pin the FP64 oracle: bskit's golden grid-info outputs, the P(k) mode counts,
the brute-force triangle-counting estimator and analytic plane-wave fields."""
import os

import numpy as np
import pytest

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from oracle import bispec_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
UPSTREAM_BINS = dict(kmin=0.00314, kmax=0.1, dk=0.00628, num_lowk_bins=3, dk_high=0.01884)


def _gridinfo_rows(n):
    edges = B.generate_bin_edge_list(**UPSTREAM_BINS)
    tri = B.generate_triangle_bin_list(return_indices=True, **UPSTREAM_BINS)
    raw, nt, km = O.grid_info(n, 1000.0, edges, tri)
    ed6 = B.triangle_indices_to_edges(edges, tri)
    rows = ['%d %e %e %e %e %e %e %e %e %e %e' % ((t,) + tuple(km[t]) + tuple(ed6[t]) + (nt[t],))
            for t in range(len(tri))]
    return rows, raw, nt


def test_oracle_reproduces_golden_gridinfo_text():
    # bskit examples/tests/output_ref/Lbox1000_512_kf_3kf_3lowkbins.dat: 512^3, L=1000.
    # Largest shell edge is 15.5 k_f < 64/3, so a 64^3 grid gives the same sums.
    rows, raw, nt = _gridinfo_rows(64)
    with open(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins.dat")) as f:
        gold = f.read().split("\n")[:len(rows)]
    assert rows == gold
    assert np.max(np.abs(raw - nt)) < 1e-6
    with open(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins_slow.dat")) as f:
        slow = f.read().split("\n")[:len(rows)]
    assert slow == gold  # bskit's slow and fast grid info agree


def test_oracle_reproduces_golden_subbox_gridinfo():
    # ..._subbox0.dat: L=500, 256^3 subbox, 5 appended runs of the same 59 bins.
    # bskit prints the raw FFT sum as N_tri; where no closed triangle exists it is
    # round-off (0 or -9.06e-14 in bin 29) and bskit's k_mean there is 0/0 -> NaN or
    # round-off garbage.  The exact count rounds to the same integer; the oracle
    # (like the GPU path) reports NaN k_mean for every empty bin.
    d = np.genfromtxt(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins_subbox0.dat"))
    edges = B.generate_bin_edge_list(**UPSTREAM_BINS)
    tri = B.generate_triangle_bin_list(return_indices=True, **UPSTREAM_BINS)
    raw, nt, km = O.grid_info(48, 500.0, edges, tri)
    for blk in range(len(d) // 59):
        last = d[blk * 59:(blk + 1) * 59]
        assert np.array_equal(nt, np.rint(last[:, 10]))
        ok = nt > 0
        rel = np.abs(km[ok] - last[ok, 1:4]) / np.abs(last[ok, 1:4])
        assert rel.max() < 5e-7
        assert np.all(np.isnan(km[~ok]))
        assert np.all(np.abs(last[~ok, 10]) < 1e-6)


def test_mode_counts_match_golden_pk():
    # test_grid_512_1_ps_kf_0.5kf.dat: N_modes of [0.5,1.5]kf, [1.5,2.5]kf, ... at L=1000
    gold = np.loadtxt(os.path.join(GOLD, "ps_modes_512_head.dat"))
    kf = 2 * np.pi / 1000.0
    edges = np.array([[0.5 + i, 1.5 + i] for i in range(len(gold))]) * kf
    counts = O.shell_mode_counts(64, 1000.0, edges)
    assert np.array_equal(counts, gold[:, 2].astype(np.int64))


def test_mode_counts_match_all_golden_pk_rows_inside_the_grid():
    # every shell of radius below 63.5 k_f has the same count on a 128^3 grid as on the
    # golden file's 512^3 one: the first 62 of its 255 rows pin the oracle's predicate
    gold = np.loadtxt(os.path.join(GOLD, "ps_nmodes_512.dat")).astype(np.int64)
    assert len(gold) == 255
    kf = 2 * np.pi / 1000.0
    edges = np.array([[0.5 + i, 1.5 + i] for i in range(62)]) * kf
    assert np.array_equal(O.shell_mode_counts(128, 1000.0, edges), gold[:62])


def test_mode_counts_equal_parseval_definition():
    n, box = 16, 100.0
    kf = 2 * np.pi / box
    edges = np.array([[1, 3], [3, 5], [5, 7.2]]) * kf
    nf = O.number_fields(n, box, edges)
    parseval = np.rint((nf ** 2).sum(axis=(1, 2, 3)) / n ** 3).astype(np.int64)
    assert np.array_equal(parseval, O.shell_mode_counts(n, box, edges))


def test_fft_estimator_equals_brute_force():
    # bk_binned (main.py:834) counts triangles explicitly; edges at half-integers of k_f
    # avoid the closed-vs-half-open edge difference between the two estimators.
    n, box = 16, 50.0
    kf = 2 * np.pi / box
    delta = synthetic.lognormal_mesh(n, box, seed=3).astype(np.float64)
    for b0, b1, b2 in [((2.5, 4.5), (1.5, 3.5), (1.5, 3.5)),
                       ((3.5, 5.5), (2.5, 4.5), (0.5, 2.5)),
                       ((2.5, 3.5), (2.5, 3.5), (2.5, 3.5))]:
        bins = [np.array(b) * kf for b in (b0, b1, b2)]
        Bd, Nd, k1, k2, k3 = O.bk_binned(delta, box, *bins)
        shells = np.array(bins)
        tri = np.array([[0, 1, 2]])
        bu = O.bispectrum_unnormalized([delta], box, shells, tri)
        raw, nt, km = O.grid_info(n, box, shells, tri)
        assert nt[0] == Nd
        assert abs(bu[0] / nt[0] - Bd.real) <= 1e-9 * abs(Bd.real)
        assert abs(Bd.imag) <= 1e-9 * abs(Bd.real) + 1e-12
        assert np.allclose(km[0], [k1, k2, k3], rtol=1e-12)


def test_plane_wave_known_answer():
    # delta = sum_a A cos(q_a.x + phi_a) with q1+q2+q3 = 0 in three distinct shells:
    # B_unnorm of bin (s1, s2, s3) = L^6 * A^3 cos(phi1+phi2+phi3) / 4 (pmesh normalisation).
    n, box = 16, 2 * np.pi
    q = [np.array([3, 0, 0]), np.array([0, 2, 0]), np.array([-3, -2, 0])]
    phi = [0.3, -1.1, 0.5]
    A = 0.7
    x = np.arange(n) * box / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    delta = sum(A * np.cos(qa[0] * X + qa[1] * Y + qa[2] * Z + p) for qa, p in zip(q, phi))
    shells = np.array([[2.9, 3.1], [1.9, 2.1], [3.5, 3.7]])  # |q| = 3, 2, sqrt(13)
    bu = O.bispectrum_unnormalized([delta], box, shells, np.array([[0, 1, 2]]))
    expect = box ** 6 * A ** 3 * np.cos(sum(phi)) / 4.0
    assert abs(bu[0] - expect) < 1e-9 * abs(expect)


def test_lognormal_generator_matches_restatement():
    a = synthetic.lognormal_mesh(24, 100.0, seed=5)
    b = O.lognormal_mesh_reference(24, 100.0, seed=5)
    assert a.dtype == np.float32 and np.array_equal(a, b)
    assert abs(float(a.mean())) < 0.05
