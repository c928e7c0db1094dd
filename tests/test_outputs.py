"""Result-file tools vs bskit's own golden outputs (examples/tests/output_ref)."""
import os

import numpy as np

from bskit_gb300 import outputs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_combine_reproduces_golden_text(tmp_path):
    # examples/tests/scripts/test_process_bs_output.sh: KMAX=0.085
    out = tmp_path / "comb.dat"
    outputs.combine_bispectrum_files(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins.dat"),
                                     os.path.join(GOLD, "test_grid_512_1_unnormbs_kf_3kf_3lowbins.dat"),
                                     0.085, str(out))
    gold = open(os.path.join(GOLD, "test_grid_512_1_bs_comb_kf_3kf_3lowbins.dat")).read()
    assert out.read_text() == gold


def test_combined_equals_slow_path_at_print_precision():
    comb = np.loadtxt(os.path.join(GOLD, "test_grid_512_1_bs_comb_kf_3kf_3lowbins.dat"))
    slow = np.loadtxt(os.path.join(GOLD, "test_grid_512_1_bs_kf_3kf_3lowbins_slow.dat"))
    # slow-path B vs fast-path B / N_tri: bskit's two algorithms agree to print precision
    assert np.allclose(comb[:, 10], slow[:, 10], rtol=2e-6)
    assert np.array_equal(comb[:, 11], slow[:, 11])


def test_combine_checks_index_and_edges():
    info = np.loadtxt(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins.dat"))
    b = np.loadtxt(os.path.join(GOLD, "test_grid_512_1_unnormbs_kf_3kf_3lowbins.dat"))
    bad = b.copy()
    bad[3, 0] = 99
    try:
        outputs.combine_arrays(info, bad, 1.0)
        raise AssertionError("index mismatch not detected")
    except ValueError as e:
        assert "index mismatch" in str(e)
    bad = b.copy()
    bad[5, 2] *= 1.02
    try:
        outputs.combine_arrays(info, bad, 1.0)
        raise AssertionError("edge mismatch not detected")
    except ValueError as e:
        assert "bound mismatch" in str(e)
    # k_max cut: rows stop one before the first bin with k1_min > k_max
    k1 = info[:, 4]
    kmax = 0.05
    first = np.where(k1 > kmax)[0][0]
    assert len(outputs.combine_arrays(info, b, kmax)) == first - 1


def test_transform_bininfo_rescales_k(tmp_path):
    src = os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins.dat")
    out = tmp_path / "t.dat"
    b = outputs.transform_bininfo_file(src, str(out), 1000.0, 500.0)
    a = np.loadtxt(src)
    assert np.allclose(b[:, 1:10], 2 * a[:, 1:10]) and np.array_equal(b[:, 10], a[:, 10])
    assert np.allclose(np.loadtxt(str(out)), b, rtol=1e-6)
