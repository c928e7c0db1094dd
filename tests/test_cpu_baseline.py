"""The timed CPU baseline does the reference's work (no GPU).

``oracle.cpu_baseline.ReferenceCPU`` times bskit's fast path on the host cores from a
bounded sample.  A timing means something only if the sampled work is the real work, so
on a small mesh this checks that its shell field is the masked inverse FFT of the oracle
(bskit/main.py:1846-1861) and that its slab-parallel triangle sums, added over slabs,
are the whole-grid sums np.sum(I_a * I_b * I_c) (main.py:1875-1879).
"""
import numpy as np

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from oracle import bispec_oracle as O
from oracle.cpu_baseline import ReferenceCPU


def test_sampled_work_is_the_reference_work():
    n, box = 32, 100.0
    kf = 2 * np.pi / box
    # edges at half-integer multiples of k_f: no mode sits on an edge, so the baseline's
    # and the oracle's |k| roundings cannot disagree about membership
    kw = dict(kmin=0.5 * kf, kmax=8.5 * kf, dk=2 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = B.generate_triangle_bin_list(return_indices=True, **kw)
    delta = synthetic.lognormal_mesh(n, box, seed=3)
    ref = ReferenceCPU(delta, box, edges, tri, n_tri_sample=6, processes=2)
    try:
        est = ref.step()
        assert est > 0 and ref.last["sample_seconds"] > 0
        of = O.shell_fields(O.spectrum(delta), n, box, edges)[ref.shell]
        f0 = ref.fields[0].astype(np.float64)
        assert np.abs(f0 - of).max() <= 1e-5 * np.abs(of).max()
        f = ref.fields.astype(np.float64)
        want = np.array([np.sum(f[a] * f[b] * f[c]) for a, b, c in ref.loc])
        scale = np.array([np.sum(np.abs(f[a] * f[b] * f[c])) for a, b, c in ref.loc])
        # float32 products and pairwise float32 sums against float64 ones
        assert np.all(np.abs(ref.last["sums"] - want) <= 1e-5 * scale)
        assert ref.T == len(tri) and len(ref.loc) == 6
    finally:
        ref.close()
