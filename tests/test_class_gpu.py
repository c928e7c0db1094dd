"""The drop-in FFTBispectrum class end to end on the GPU, against bskit's golden
files and the FP64 oracle.

* ``measure_gridinfo_faster(out_file=...)`` and ``measure_bispectrum(meas_type=
  'grid_info', out_file=...)`` on bskit's own test binning (L = 1000, Nmesh 512,
  k_f-wide low-k bins then 3 k_f): the written files equal
  examples/tests/output_ref/Lbox1000_512_kf_3kf_3lowkbins.dat and its _slow twin
  character for character (rows written by main.py:2098-2106 and 1760-1772);
* ``measure_bispectrum_faster`` (unnormalised B, main.py:1784-1938) and
  ``measure_bispectrum(meas_type='full')`` (B / N_tri, main.py:1637-1780) on a 64^3
  lognormal mesh: the returned values and the rows written to ``out_file`` against
  the oracle (counts exact, k_mean 1e-12 relative, B within the bf16x3 bound of
  tests/test_gpu_parity.py: |B - B_o| <= 4e-6 of the absolute sum).
"""
import os

import numpy as np
import pytest

from bskit_gb300 import FFTBispectrum
from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from oracle import bispec_oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
GOLDEN_BINS = dict(kmin=0.00314, kmax=0.1, dk=0.00628, num_lowk_bins=3, dk_high=0.01884)


def _lines(path):
    with open(path) as f:
        return f.read().splitlines()


def test_class_gridinfo_files_match_golden(cuda, tmp_path):
    mesh = np.zeros((512,) * 3, dtype=np.float32)  # grid information needs no field values
    fb = FFTBispectrum(mesh, BoxSize=1000.0, for_grid_info_only=True, **GOLDEN_BINS)
    fast = tmp_path / "fast.dat"
    res = fb.measure_gridinfo_faster(out_file=str(fast))
    assert len(res["N_tri"]) == 59
    assert _lines(fast) == _lines(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins.dat"))
    slow = tmp_path / "slow.dat"
    fb2 = FFTBispectrum(mesh, BoxSize=1000.0, for_grid_info_only=True, **GOLDEN_BINS)
    fb2.measure_bispectrum(meas_type="grid_info", out_file=str(slow))
    assert _lines(slow) == _lines(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins_slow.dat"))
    fb.close()
    fb2.close()


def _rows(path):
    return np.array([[float(v) for v in line.split()] for line in _lines(path)])


@pytest.mark.parametrize("num_fields", [1, 2])
def test_class_measurements_match_oracle(cuda, tmp_path, num_fields):
    n, box = 64, 100.0
    kf = 2 * np.pi / box
    kw = dict(kmin=kf, kmax=16 * kf, dk=3 * kf)
    d1 = synthetic.lognormal_mesh(n, box, seed=0)
    meshes = [d1]
    extra = {}
    if num_fields == 2:
        d2 = synthetic.noisy_copy(d1, seed=3)
        meshes.append(d2)
        extra["second"] = d2
    edges = B.generate_bin_edge_list(**kw)
    tri = B.generate_triangle_bin_list(num_fields=num_fields, return_indices=True, **kw)

    # oracle: unnormalised B, its absolute sum, N_tri and k_mean
    fields = [O.shell_fields(O.spectrum(m), n, box, edges) for m in meshes]
    fa, fc = fields[0], fields[-1]
    scale = box ** 6 / float(n) ** 3
    bo = O.triple_sums(fa, fa, fc, tri) * scale
    babs = O.triple_sums(np.abs(fa), np.abs(fa), np.abs(fc), tri) * scale
    _, nto, kmo = O.grid_info(n, box, edges, tri)

    fb = FFTBispectrum(d1, BoxSize=box, **kw, **extra)
    f_fast = tmp_path / "fast.dat"
    res = fb.measure_bispectrum_faster(out_file=str(f_fast))
    assert np.array_equal(res["index"], np.arange(len(tri)))
    assert np.all(np.abs(res["B"] - bo) <= 4e-6 * babs)
    rows = _rows(f_fast)
    assert np.array_equal(rows[:, 0], np.arange(len(tri)))
    np.testing.assert_allclose(rows[:, 1:7], B.triangle_indices_to_edges(edges, tri), rtol=1e-6)
    np.testing.assert_allclose(rows[:, 7], res["B"], rtol=1e-6)  # %e: 7 significant digits

    # bskit keeps B and grid information in separate measurement objects: its 'b' dict
    # stores k_mean as one value per bin for B and three per bin for grid information
    # (main.py:1888 and 2070), which one dict cannot mix
    fb_gi = FFTBispectrum(d1, BoxSize=box, for_grid_info_only=True, **kw, **extra)
    gi = fb_gi.measure_gridinfo_faster()
    assert np.array_equal(gi["N_tri"], nto)
    live = nto > 0
    np.testing.assert_allclose(gi["k_mean"][live], kmo[live], rtol=1e-12)

    fb_slow = FFTBispectrum(d1, BoxSize=box, **kw, **extra)
    f_full = tmp_path / "full.dat"
    full = fb_slow.measure_bispectrum(meas_type="full", out_file=str(f_full))
    assert np.array_equal(full["N_tri"], nto)
    with np.errstate(divide="ignore", invalid="ignore"):
        b_norm = bo / nto
        bound = 4e-6 * babs / nto
    assert np.all(np.abs(full["B"][live] - b_norm[live]) <= bound[live])
    rows = _rows(f_full)
    assert rows.shape == (len(tri), 12)
    assert np.array_equal(rows[:, 11], nto)
    np.testing.assert_allclose(rows[live, 10], full["B"][live], rtol=1e-6)
    fb.close()
    fb_gi.close()
    fb_slow.close()
