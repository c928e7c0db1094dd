"""The measurement scripts' command lines (no GPU).

``python -m bskit_gb300.measure`` takes bskit's script arguments
(scripts/measure/measure_bs_fast.py:58-111, measure_bs_slow.py,
measure_subbox_bs_fast.py:60-113).  The measurement classes are replaced by recorders
here, so these tests check what the command line turns into -- the bigfile meshes read,
the binning keywords, the method called and its index range and output file -- not the
GPU arithmetic, which the GPU tests cover through the same classes.
"""
import io

import numpy as np
import pytest

from bskit_gb300 import bispectrum, measure, subbox

from test_bigfile import write_block

CALLS = []


class FakeFFTBispectrum(object):
    def __init__(self, source, **kw):
        CALLS.append(("init", source, kw))

    def __getattr__(self, name):
        def method(**kw):
            CALLS.append((name, kw))
        return method

    def close(self):
        pass


class FakeSubbox(object):
    def __init__(self, source, nsub, **kw):
        CALLS.append(("subbox_init", source, nsub, kw))

    def measure(self, **kw):
        CALLS.append(("subbox_measure", kw))

    def close(self):
        pass


@pytest.fixture
def grids(tmp_path, monkeypatch):
    CALLS.clear()
    monkeypatch.setattr(bispectrum, "FFTBispectrum", FakeFFTBispectrum)
    monkeypatch.setattr(subbox, "SubboxBispectrum", FakeSubbox)
    paths = []
    for i in range(2):
        root = tmp_path / ("snap%d" % i)
        root.mkdir()
        grid = np.random.default_rng(i).standard_normal((16,) * 3).astype(np.float32)
        write_block(str(root), "Field", grid, {"BoxSize": np.array([500.0] * 3),
                                               "Nmesh": np.array([16] * 3, np.int64),
                                               "ndarray.shape": np.array([16] * 3, np.int64)})
        paths.append((str(root), grid))
    return paths


def _run(kind, args):
    return measure.run(kind, [str(a) for a in args], out=io.StringIO())


def test_fast_bispectrum_command(grids, tmp_path):
    (p1, g1), (p2, g2) = grids
    out = tmp_path / "b.dat"
    _run("bs_fast", ["bigfile_grid", p1, 16, 64, 500.0, 3, 40, out, "--snap_prefix2", p2,
                     "--k_bin_info", 0.0126, 0.1, 0.0126, "--high_k_bin_info", 3, 0.0252,
                     "-cic", "-pu", 1000.0])
    (tag, src, kw), (name, mkw) = CALLS
    assert tag == "init" and np.array_equal(src.numpy(), g1) and src.compensate_cic == 64
    assert np.array_equal(kw["second"].numpy(), g2) and kw["third"] is None
    assert kw["Nmesh"] == 16 and np.array_equal(kw["BoxSize"], [500.0] * 3)
    assert (kw["kmin"], kw["kmax"], kw["dk"]) == (0.0126, 0.1, 0.0126)
    assert (kw["num_lowk_bins"], kw["dk_high"]) == (3, 0.0252)
    assert kw["pos_units_mpcoverh"] == 1000.0 and kw["triangle_type"] == "all"
    assert kw["for_grid_info_only"] is False and kw["precision"] == "bf16x3"
    assert name == "measure_bispectrum_faster"
    assert mkw == dict(imin=3, imax=40, out_file=str(out), verbose=0)


def test_fast_gridinfo_and_triangle_types(grids, tmp_path):
    (p1, _), _ = grids
    _run("bs_fast", ["bigfile_grid", p1, 16, 16, 500.0, 0, 10, tmp_path / "g.dat",
                     "--k_bin_info", 0.01, 0.1, 0.02, "--meas_type", "grid_info",
                     "--triangle_type", "isosceles", "--isos_mult", 2, "--precision", "fp32"])
    (_, src, kw), (name, _) = CALLS
    assert src.compensate_cic is None
    assert kw["for_grid_info_only"] is True and kw["precision"] == "fp32"
    assert (kw["triangle_type"], kw["isos_mult"], kw["isos_tol"]) == ("isosceles", 2.0, 0.1)
    assert name == "measure_gridinfo_faster"
    CALLS.clear()
    _run("bs_fast", ["bigfile_grid", p1, 16, 16, 500.0, 0, 10, tmp_path / "s.dat",
                     "--k_bin_info", 0.01, 0.1, 0.02, "--triangle_type", "squeezed",
                     "--squeezed_bin_index", 1])
    assert CALLS[0][2]["squeezed_bin_index"] == 1


def test_slow_command_defaults_to_full(grids, tmp_path):
    (p1, _), _ = grids
    _run("bs_slow", ["bigfile_grid", p1, 16, 16, 500.0, 0, 5, tmp_path / "f.dat",
                     "--k_bin_info", 0.01, 0.1, 0.02])
    name, mkw = CALLS[1]
    assert name == "measure_bispectrum" and mkw["meas_type"] == "full"
    assert (mkw["imin"], mkw["imax"]) == (0, 5)


def test_subbox_command(grids, tmp_path):
    (p1, g1), _ = grids
    prefix = str(tmp_path / "sb")
    _run("subbox_bs_fast", ["bigfile_grid", p1, 16, 16, 500.0, 2, 0, 7, 1, 3, prefix,
                            "--k_bin_info", 0.02, 0.2, 0.04])
    (tag, src, nsub, kw), (name, mkw) = CALLS
    assert tag == "subbox_init" and nsub == 2 and np.array_equal(src.numpy(), g1)
    assert kw["BoxSize"] == 500.0 and kw["kmin"] == 0.02
    assert name == "subbox_measure"
    assert list(mkw["subboxes"]) == [1, 2, 3]  # the end index is inclusive, as bskit's loop
    assert (mkw["imin"], mkw["imax"], mkw["meas_type"]) == (0, 7, "unnorm_b_value")
    assert mkw["out_file_prefix"] == prefix


def test_reference_errors(grids, tmp_path):
    (p1, _), (p2, _) = grids
    base = ["bigfile_grid", p1, 16, 16, 500.0, 0, 5, tmp_path / "e.dat"]
    with pytest.raises(RuntimeError):  # neither a bin file nor kmin/kmax/dk
        _run("bs_fast", base)
    kbins = tmp_path / "bins.txt"
    np.savetxt(kbins, np.ones((6, 2)))
    with pytest.raises(RuntimeError):  # both
        _run("bs_fast", base + ["--k_bin_file", kbins, "--k_bin_info", 0.01, 0.1, 0.02])
    with pytest.raises(ValueError):  # isosceles without its multiplier
        _run("bs_fast", base + ["--k_bin_info", 0.01, 0.1, 0.02, "--triangle_type",
                                "isosceles"])
    with pytest.raises(ValueError):  # third mesh without a second
        _run("bs_fast", base + ["--k_bin_info", 0.01, 0.1, 0.02, "--snap_prefix3", p2])
    with pytest.raises(NotImplementedError):  # particle catalogs need nbodykit
        _run("bs_fast", ["gadget"] + base[1:] + ["--k_bin_info", 0.01, 0.1, 0.02])
    with pytest.raises(SystemExit):  # argparse: unknown measurement type
        _run("bs_fast", base + ["--k_bin_info", 0.01, 0.1, 0.02, "--meas_type", "full"])
    assert measure.main(["nonsense"]) == 2
    # a k-bin file is passed through as k_edges (rows k1_lo..k3_hi, one column per bin)
    CALLS.clear()
    _run("bs_slow", base + ["--k_bin_file", kbins])
    assert CALLS[0][2]["k_edges"].shape == (2, 6)


@pytest.mark.gpu
def test_fast_command_runs_on_the_gpu(cuda, tmp_path):
    # the real classes: the command's output file holds the class's own rows (the FP64
    # contraction's sums may differ in the last bits between runs: 2e-6 on 7 printed digits)
    n, box = 32, 100.0
    grid = np.random.default_rng(3).standard_normal((n,) * 3).astype(np.float32)
    root = tmp_path / "snap"
    root.mkdir()
    write_block(str(root), "Field", grid, {"BoxSize": np.array([box] * 3),
                                           "ndarray.shape": np.array([n] * 3, np.int64)})
    kf = 2 * np.pi / box
    out = tmp_path / "cli.dat"
    _run("bs_fast", ["bigfile_grid", root, n, n, box, 0, 30, out, "--k_bin_info",
                     repr(kf), repr(8 * kf), repr(2 * kf), "--precision", "fp64"])
    direct = tmp_path / "direct.dat"
    fb = bispectrum.FFTBispectrum(grid, BoxSize=box, kmin=kf, kmax=8 * kf, dk=2 * kf,
                                  precision="fp64")
    fb.measure_bispectrum_faster(imin=0, imax=30, out_file=str(direct))
    fb.close()
    a, b = np.loadtxt(out), np.loadtxt(direct)
    assert a.shape == b.shape and a.shape[0] > 1
    assert np.array_equal(a[:, :7], b[:, :7])
    assert np.allclose(a[:, 7], b[:, 7], rtol=2e-6, atol=0)
