"""Sub-box requests (bskit's field_subbox_pm + measure_subbox_bs_fast.py workflow).

CPU: the sub-box index map against bskit's own function (golden fixture) and
the nearest-grid-point cut.  GPU (through the C ABI): every sub-box's B against
the FP64 oracle on the cut-out array (bf16x3 tolerances of test_gpu_parity: nrm
<= 4e-6, rel <= 1e-5 on well-conditioned bins, median rel <= 1e-5), the sub-box grid
information against bskit's golden ``_subbox0.dat``, and the full-mesh CIC
deconvolution against the oracle (1e-5 of the field's max).
"""
import json
import os

import numpy as np
import pytest
import torch

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from bskit_gb300.mesh import ArrayMesh
from bskit_gb300.subbox import field_subbox, subbox_index_to_multiindex
from oracle import bispec_oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TWO_PI = 2 * np.pi


def test_subbox_multiindex_matches_reference():
    ref = json.load(open(os.path.join(GOLD, "subbox_multiindex.json")))
    for n, rows in ref.items():
        n = int(n)
        got = [subbox_index_to_multiindex(i, n).tolist() for i in range(n ** 3)]
        assert got == rows


def test_field_subbox_is_the_block():
    a = np.arange(12 ** 3, dtype=np.float32).reshape(12, 12, 12)
    sub = field_subbox((1, 0, 2), 3, ArrayMesh(a, 30.0))
    assert sub.Nmesh == 4
    assert np.allclose(sub.attrs['BoxSize'], 10.0)
    assert np.array_equal(sub.numpy(), a[4:8, 0:4, 8:12])
    t = field_subbox((1, 0, 2), 3, ArrayMesh(torch.from_numpy(a), 30.0))
    assert np.array_equal(t.numpy(), a[4:8, 0:4, 8:12])


def _check(b, bo, babs):
    err = np.abs(b - bo)
    nrm = err / babs
    rel = err / np.abs(bo)
    well = np.abs(bo) >= 0.1 * babs
    assert nrm.max() <= 4e-6
    assert np.median(rel) <= 1e-5
    if well.any():
        assert rel[well].max() <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("cross", [False, True])
def test_subbox_bispectra_match_oracle(cuda, cross):
    from bskit_gb300.subbox import SubboxBispectrum
    n_full, box_full, nsub = 64, 100.0, 2
    d1 = synthetic.lognormal_mesh(n_full, box_full, seed=41)
    d2 = synthetic.noisy_copy(d1, seed=42) if cross else None
    n, box = n_full // nsub, box_full / nsub
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=8 * kf, dk=2 * kf)
    sb = SubboxBispectrum(ArrayMesh(d1, box_full), nsub, second=None if d2 is None else
                          ArrayMesh(d2, box_full), **kw)
    res = sb.measure(subboxes=[0, 5, 7], meas_type='unnorm_b_value')
    edges = B.generate_bin_edge_list(**kw)
    tri = np.asarray(sb.k_indices)
    for i, r in res.items():
        a, b, c = (int(v) * n for v in subbox_index_to_multiindex(i, nsub))
        fa = O.shell_fields(O.spectrum(d1[a:a + n, b:b + n, c:c + n]), n, box, edges)
        fc = fa if d2 is None else O.shell_fields(O.spectrum(d2[a:a + n, b:b + n, c:c + n]), n,
                                                  box, edges)
        bo = O.triple_sums(fa, fa, fc, tri) * box ** 6 / n ** 3
        babs = O.triple_sums(np.abs(fa), np.abs(fa), np.abs(fc), tri) * box ** 6 / n ** 3
        _check(r['B'], bo, babs)
    sb.close()


@pytest.mark.gpu
def test_subbox_gridinfo_matches_golden(cuda, tmp_path):
    # bskit's Lbox1000_512_kf_3kf_3lowkbins_subbox0.dat: sub-box 0 of a 512^3, L = 1000
    # mesh cut 2 per side; grid information only, so the mesh is never read
    from bskit_gb300.subbox import SubboxBispectrum
    up = dict(kmin=0.00314, kmax=0.1, dk=0.00628, num_lowk_bins=3, dk_high=0.01884)
    sb = SubboxBispectrum(ArrayMesh(torch.empty((512,) * 3), 1000.0), 2, **up)
    res = sb.measure(subboxes=[0], meas_type='grid_info',
                     out_file_prefix=str(tmp_path / "sub"))
    sb.close()
    d = np.genfromtxt(os.path.join(GOLD, "Lbox1000_512_kf_3kf_3lowkbins_subbox0.dat"))[:59]
    nt, km = res[0]['N_tri'], res[0]['k_mean']
    assert np.array_equal(nt, np.rint(d[:, 10]))
    ok = nt > 0
    assert (np.abs(km[ok] - d[ok, 1:4]) / np.abs(d[ok, 1:4])).max() < 5e-7
    assert np.all(np.isnan(km[~ok]))
    written = np.genfromtxt(str(tmp_path / "sub_subbox0.dat"))
    assert np.array_equal(written[:, 10], nt)


@pytest.mark.gpu
def test_compensate_cic_matches_oracle(cuda):
    from bskit_gb300.engine import compensate_cic
    n = 48
    d = synthetic.lognormal_mesh(n, 100.0, seed=43)
    got = compensate_cic(torch.from_numpy(d).cuda(), 96).cpu().numpy()
    ref = O.c2r(O.cic_compensate(O.spectrum(d), n, 96), n)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_subbox_with_cic_matches_oracle(cuda):
    from bskit_gb300.subbox import SubboxBispectrum
    n_full, box_full, nsub = 64, 100.0, 2
    d = synthetic.lognormal_mesh(n_full, box_full, seed=44)
    n, box = n_full // nsub, box_full / nsub
    kf = TWO_PI / box
    kw = dict(kmin=kf, kmax=8 * kf, dk=2 * kf)
    sb = SubboxBispectrum(ArrayMesh(d, box_full, compensate_cic=128), nsub, **kw)
    r = sb.measure(subboxes=[3], meas_type='unnorm_b_value')[3]
    comp = O.c2r(O.cic_compensate(O.spectrum(d), n_full, 128), n_full)
    a, b, c = (int(v) * n for v in subbox_index_to_multiindex(3, nsub))
    edges = B.generate_bin_edge_list(**kw)
    tri = np.asarray(sb.k_indices)
    f = O.shell_fields(O.spectrum(comp[a:a + n, b:b + n, c:c + n]), n, box, edges)
    bo = O.triple_sums(f, f, f, tri) * box ** 6 / n ** 3
    babs = O.triple_sums(np.abs(f), np.abs(f), np.abs(f), tri) * box ** 6 / n ** 3
    _check(r['B'], bo, babs)
    sb.close()
