"""Bin-list generators vs outputs of bskit's own generators (tests/golden/bins_reference.json,
made by tests/golden/make_fixtures.py from bskit/main.py:1008-1389)."""
import hashlib
import json
import os

import numpy as np
import pytest

from bskit_gb300 import bins as B

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "bins_reference.json")) as _f:
    CASES = json.load(_f)["cases"]


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _kw(p):
    return dict(kmin=p["kmin"], kmax=p["kmax"], dk=p["dk"],
                num_lowk_bins=p.get("num_lowk_bins", 0), dk_high=p.get("dk_high", -1.0))


def _generate(name, kw, return_indices):
    if name.startswith("all_nf"):
        return B.generate_triangle_bin_list(num_fields=int(name[-1]), return_indices=return_indices, **kw)
    if name == "equilateral":
        return B.generate_equilateral_triangle_bin_list(return_indices=return_indices, **kw)
    if name.startswith("squeezed"):
        return B.generate_squeezed_triangle_bin_list(squeezed_bin_index=int(name.split("_")[1]),
                                                     return_indices=return_indices, **kw)
    _, m, t = name.split("_")
    return B.generate_isosceles_triangle_bin_list(isos_mult=float(m), isos_tol=float(t),
                                                  return_indices=return_indices, **kw)


@pytest.mark.parametrize("case", CASES, ids=[c["params"]["name"] for c in CASES])
def test_bin_edges_bit_exact(case):
    e = B.generate_bin_edge_list(**_kw(case["params"]))
    assert np.array_equal(e, np.array(case["bin_edges"]))
    gm = [B.geometric_k_mean(a, b) for a, b in e]
    assert gm == case["geometric_k_mean"]


@pytest.mark.parametrize("case", CASES, ids=[c["params"]["name"] for c in CASES])
def test_triangle_lists_bit_exact(case):
    kw = _kw(case["params"])
    for name, ref in case["lists"].items():
        E = np.asarray(_generate(name, kw, False), dtype=np.float64)
        I = np.asarray(_generate(name, kw, True), dtype=np.int64)
        assert list(E.shape) == ref["edges_shape"], name
        assert _digest(E) == ref["edges_sha256"], name
        assert _digest(I) == ref["idx_sha256"], name
        if "idx" in ref:
            assert I.tolist() == ref["idx"]


def test_headline_counts():
    kf = 2 * np.pi / 1000.0
    idx = B.generate_triangle_bin_list(kmin=kf, kmax=128 * kf, dk=2 * kf, return_indices=True)
    assert len(idx) == 24305
    assert np.all(idx[:, 0] >= idx[:, 1]) and np.all(idx[:, 1] >= idx[:, 2])
    e = B.generate_bin_edge_list(kf, 128 * kf, 2 * kf)
    assert len(e) == 63  # arange drops the last shell below kmax


def test_errors_match_reference():
    with pytest.raises(ValueError, match="kmin must be > 0"):
        B.generate_bin_edge_list(-1., 1., 0.1)
    with pytest.raises(ValueError, match="kmax must be > 0"):
        B.generate_bin_edge_list(0.1, 0., 0.1)
    with pytest.raises(ValueError, match="dk must be > 0"):
        B.generate_bin_edge_list(0.1, 1., 0.)
    with pytest.raises(ValueError, match="dk_high"):
        B.generate_bin_edge_list(0.1, 1., 0.1, num_lowk_bins=2)
    with pytest.raises(ValueError, match="num_fields"):
        B.generate_triangle_bin_list(0.1, 1., 0.1, num_fields=4)
    with pytest.raises(NotImplementedError, match="Mu binning"):
        B.generate_triangle_bin_list(0.1, 1., 0.1, dmu=0.1)
    with pytest.raises(ValueError, match="isos_mult"):
        B.generate_isosceles_triangle_bin_list(0.1, 1., 0.1, isos_mult=0.5)


def test_indices_edges_consistent():
    kw = dict(kmin=0.05, kmax=1.0, dk=0.05, num_lowk_bins=4, dk_high=0.15)
    e = B.generate_bin_edge_list(**kw)
    for nf in (1, 2, 3):
        idx = B.generate_triangle_bin_list(num_fields=nf, return_indices=True, **kw)
        edg = B.generate_triangle_bin_list(num_fields=nf, **kw)
        assert np.array_equal(B.triangle_indices_to_edges(e, idx), edg)
