"""Generate the golden fixtures used by the CPU test-suite.

This script runs ONLY where the upstream bskit sources are mounted (it is not
run by the tests).  It imports ``bskit/main.py`` from the upstream checkout
with stub modules standing in for nbodykit / pmesh (absent here; only the
pure-numpy bin generators are exercised) and the ``np.float = float`` shim
that numpy>=1.24 needs for ``bskit/main.py:1381``.  It then writes:

* ``bins_reference.json``  -- outputs of the upstream bin-list generators
  (``generate_bin_edge_list`` main.py:1008, ``generate_triangle_bin_list``
  main.py:1272, ``generate_equilateral/squeezed/isosceles_triangle_bin_list``
  main.py:1074/1121/1181) for a set of parameter combinations: full arrays
  for small lists, (shape, sha256 of the float64/int64 bytes, first/last rows)
  for large ones.
* ``subbox_multiindex.json`` -- ``subbox_index_to_multiindex`` (main.py:54)
  for every sub-box index at nsub_per_side = 1..4.
* copies of the upstream golden grid-info outputs
  (``examples/tests/output_ref/Lbox1000_512_kf_3kf_3lowkbins*.dat``) and the
  first rows of the P(k) golden file that carry shell mode counts.

Usage:  python tests/golden/make_fixtures.py /path/to/bskit-checkout
"""
import hashlib
import importlib.util
import json
import os
import shutil
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    class _Dummy:
        def __init__(self, *a, **k):
            pass

    class _Comm:
        rank = 0
        size = 1

        def gather(self, x):
            return [x]

        def bcast(self, x):
            return x

    class _CurrentMPIComm:
        @staticmethod
        def get():
            return _Comm()

    nbk = mod("nbodykit")
    mod("nbodykit.lab")
    fftpower = mod("nbodykit.algorithms.fftpower", FFTBase=_Dummy)
    mod("nbodykit.algorithms", fftpower=fftpower)
    nbk.setup_logging = lambda *a, **k: None
    nbk.style = None
    nbk.CurrentMPIComm = _CurrentMPIComm
    mod("nbodykit.meshtools", SlabIterator=_Dummy)
    mod("pmesh")
    mod("pmesh.pm", ParticleMesh=_Dummy, RealField=_Dummy, ComplexField=_Dummy)
    mod("pmesh.window", Affine=_Dummy)


def load_reference(ref_root):
    _install_stubs()
    if not hasattr(np, "float"):
        np.float = float  # bskit/main.py:1381 uses the removed alias
    spec = importlib.util.spec_from_file_location(
        "bskit_reference_main", os.path.join(ref_root, "bskit", "main.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def _pack(edges, idx, full_limit=400):
    edges = np.asarray(edges, dtype=np.float64)
    idx = np.asarray(idx, dtype=np.int64)
    out = {
        "T": int(len(idx)),
        "edges_shape": list(edges.shape),
        "edges_sha256": _digest(edges),
        "idx_sha256": _digest(idx),
    }
    if len(idx) <= full_limit:
        out["edges"] = edges.tolist()
        out["idx"] = idx.tolist()
    else:
        out["edges_head"] = edges[:5].tolist()
        out["edges_tail"] = edges[-5:].tolist()
        out["idx_head"] = idx[:5].tolist()
        out["idx_tail"] = idx[-5:].tolist()
    return out


def bin_cases():
    """Parameter sets: the benchmark workloads plus the upstream test binning
    and a few edge cases (high-k width switch, odd ranges)."""
    cases = []
    two_pi = 2.0 * np.pi

    def kf(L):
        return two_pi / L

    # 64^3, L=100, dk=3kf, kf..kNyq/2
    cases.append(dict(name="mesh64_L100_dk3", kmin=kf(100), kmax=16 * kf(100), dk=3 * kf(100)))
    # 256^3, L=500, dk=2kf, kf..kNyq/2
    cases.append(dict(name="mesh256_L500_dk2", kmin=kf(500), kmax=64 * kf(500), dk=2 * kf(500)))
    # 512^3, L=1000, dk=2kf, kf..kNyq/2 (the 24305-bin all-triangle set)
    cases.append(dict(name="mesh512_L1000_dk2", kmin=kf(1000), kmax=128 * kf(1000), dk=2 * kf(1000)))
    # 1024^3, L=2000, dk=4kf, kf..0.3 kNyq
    cases.append(dict(name="mesh1024_L2000_dk4", kmin=kf(2000), kmax=0.3 * 512 * kf(2000), dk=4 * kf(2000)))
    # serving sizes, L=100, dk=2kf to kNyq/2
    for n in (64, 128):
        cases.append(dict(name="serve%d_L100_dk2" % n, kmin=kf(100), kmax=n / 4 * kf(100), dk=2 * kf(100)))
    # upstream example-test binning (examples/tests/scripts/test_measure_bs_faster.sh:22-26)
    cases.append(dict(name="upstream_test", kmin=0.00314, kmax=0.1, dk=0.00628,
                      num_lowk_bins=3, dk_high=0.01884))
    # small odd case with a high-k width switch
    cases.append(dict(name="small_highk", kmin=0.05, kmax=1.0, dk=0.05, num_lowk_bins=4, dk_high=0.15))
    cases.append(dict(name="tiny", kmin=0.3, kmax=1.9, dk=0.4))
    return cases


def main(ref_root):
    ref = load_reference(ref_root)
    out = {"cases": []}
    for c in bin_cases():
        kw = dict(kmin=c["kmin"], kmax=c["kmax"], dk=c["dk"],
                  num_lowk_bins=c.get("num_lowk_bins", 0), dk_high=c.get("dk_high", -1.0))
        rec = {"params": c}
        rec["bin_edges"] = ref.generate_bin_edge_list(**kw).tolist()
        nb = len(rec["bin_edges"])
        big = c["name"] in ("mesh512_L1000_dk2", "mesh1024_L2000_dk4", "mesh256_L500_dk2")
        lists = {}
        for nf in (1, 2, 3):
            if big and nf > 1 and c["name"] != "mesh256_L500_dk2":
                continue
            e = ref.generate_triangle_bin_list(num_fields=nf, **kw)
            i = ref.generate_triangle_bin_list(num_fields=nf, return_indices=True, **kw)
            lists["all_nf%d" % nf] = _pack(e, i)
        e = ref.generate_equilateral_triangle_bin_list(**kw)
        i = ref.generate_equilateral_triangle_bin_list(return_indices=True, **kw)
        lists["equilateral"] = _pack(e, i)
        for sq in sorted({0, 1, min(2, nb - 2)}):
            e = ref.generate_squeezed_triangle_bin_list(squeezed_bin_index=sq, **kw)
            i = ref.generate_squeezed_triangle_bin_list(squeezed_bin_index=sq, return_indices=True, **kw)
            lists["squeezed_%d" % sq] = _pack(e, i)
        for mult, tol in ((2.0, 0.1), (1.5, 0.2), (3.0, 0.05)):
            e = ref.generate_isosceles_triangle_bin_list(isos_mult=mult, isos_tol=tol, **kw)
            i = ref.generate_isosceles_triangle_bin_list(isos_mult=mult, isos_tol=tol,
                                                         return_indices=True, **kw)
            lists["isosceles_%g_%g" % (mult, tol)] = _pack(e, i)
        rec["lists"] = lists
        # geometric_k_mean (main.py:408) on every shell
        rec["geometric_k_mean"] = [float(ref.geometric_k_mean(a, b)) for a, b in rec["bin_edges"]]
        out["cases"].append(rec)
        print(c["name"], nb, {k: v["T"] for k, v in lists.items()})

    with open(os.path.join(HERE, "bins_reference.json"), "w") as f:
        json.dump(out, f, indent=0)

    # subbox_index_to_multiindex (main.py:54) for every sub-box of nsub = 1..4
    sub = {str(n): [ref.subbox_index_to_multiindex(i, n).tolist() for i in range(n ** 3)]
           for n in (1, 2, 3, 4)}
    with open(os.path.join(HERE, "subbox_multiindex.json"), "w") as f:
        json.dump(sub, f)

    src = os.path.join(ref_root, "examples", "tests", "output_ref")
    for name in ("Lbox1000_512_kf_3kf_3lowkbins.dat", "Lbox1000_512_kf_3kf_3lowkbins_slow.dat",
                 "Lbox1000_512_kf_3kf_3lowkbins_subbox0.dat",
                 # unnormalised B and its combination with the grid info (pins the combine tool)
                 "test_grid_512_1_unnormbs_kf_3kf_3lowbins.dat",
                 "test_grid_512_1_bs_comb_kf_3kf_3lowbins.dat",
                 "test_grid_512_1_bs_kf_3kf_3lowbins_slow.dat"):
        shutil.copyfile(os.path.join(src, name), os.path.join(HERE, name))
    # first rows of the P(k) golden file: k_mean, P, N_modes for [0.5,1.5]kf, [1.5,2.5]kf...
    with open(os.path.join(src, "test_grid_512_1_ps_kf_0.5kf.dat")) as f:
        rows = [next(f) for _ in range(12)]
    with open(os.path.join(HERE, "ps_modes_512_head.dat"), "w") as f:
        f.writelines(rows)
    # the N_modes column of every row: shells [i + 0.5, i + 1.5] kf, i = 0..254, at 512^3
    pk = np.loadtxt(os.path.join(src, "test_grid_512_1_ps_kf_0.5kf.dat"))
    with open(os.path.join(HERE, "ps_nmodes_512.dat"), "w") as f:
        f.write("# N_modes of shells [i + 0.5, i + 1.5] k_f, i = 0..%d, Nmesh 512, L 1000 "
                "(test_grid_512_1_ps_kf_0.5kf.dat, third column)\n" % (len(pk) - 1))
        f.writelines("%d\n" % int(round(v)) for v in pk[:, 2])
    # they are the exact closed-shell counts of the full 512^3 grid: |q|^2 is an integer, so
    # [n - 1/2, n + 1/2] k_f holds the modes with n^2 - n + 1 <= |q|^2 <= n^2 + n
    q = np.fft.fftfreq(512, 1.0 / 512).astype(np.int64)
    r2max = 3 * 256 ** 2
    yz = np.bincount((q[:, None] ** 2 + q[None, :] ** 2).ravel(), minlength=r2max + 1)
    hist = np.zeros(r2max + 1, dtype=np.int64)
    for qx in q:
        hist[qx * qx:] += yz[:r2max + 1 - qx * qx]
    cum = np.concatenate([[0], np.cumsum(hist)])
    exact = [cum[n * n + n + 1] - cum[n * n - n + 1] for n in range(1, len(pk) + 1)]
    assert np.array_equal(np.array(exact), np.rint(pk[:, 2]).astype(np.int64))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
