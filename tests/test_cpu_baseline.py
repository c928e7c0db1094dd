"""The timed CPU baseline does the reference's work (no GPU).

``oracle.cpu_baseline.ReferenceCPU`` times bskit's fast path on the host cores, in full
or from a bounded sample.  A timing means something only if the timed work is the real
work, so on a small mesh this checks that its shell fields are the masked inverse FFTs of
the oracle (bskit/main.py:1846-1861) and that its slab-parallel triangle sums, added over
slabs, are the whole-grid sums np.sum(I_a * I_b * I_c) (main.py:1875-1879): for the
stratified sample of ``step()`` (each sampled bin once, on its own three shells) and for
``full_run()``.
"""
import numpy as np

from bskit_gb300 import bins as B
from bskit_gb300 import synthetic
from oracle import bispec_oracle as O
from oracle.cpu_baseline import ReferenceCPU, stratified_shells


def _case():
    n, box = 32, 100.0
    kf = 2 * np.pi / box
    # edges at half-integer multiples of k_f: no mode sits on an edge, so the baseline's
    # and the oracle's |k| roundings cannot disagree about membership
    kw = dict(kmin=0.5 * kf, kmax=12.5 * kf, dk=1 * kf)
    edges = B.generate_bin_edge_list(**kw)
    tri = B.generate_triangle_bin_list(return_indices=True, **kw)
    delta = synthetic.lognormal_mesh(n, box, seed=3)
    return n, box, edges, tri, delta


def test_stratified_shells_span_the_range():
    s = stratified_shells(63, 18)
    assert len(s) == 18 and s[0] == 0 and s[-1] == 62
    assert stratified_shells(10, 18) == list(range(10))


def test_sampled_work_is_the_reference_work():
    n, box, edges, tri, delta = _case()
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    ref = ReferenceCPU(delta, box, edges, tri, sample_shells=5, processes=2)
    try:
        done = []
        for _ in range(len(ref.shells)):
            est = ref.step()
            assert est > 0 and ref.last["sample_seconds"] > 0
            k = ref.k - 1
            s = ref.shells[k]
            f = ref.fields[ref.slot[s]].astype(np.float64)
            assert np.abs(f - of[s]).max() <= 1e-5 * np.abs(of[s]).max()
            for (a, b, c), v in zip(ref.by_step[k], ref.last["sums"]):
                want = np.sum(of[a] * of[b] * of[c])
                scale = np.sum(np.abs(of[a] * of[b] * of[c]))
                # float32 fields, products and sums against the float64 oracle
                assert abs(v - want) <= 1e-5 * scale
                done.append((a, b, c))
        # every bin inside the sampled shells was summed exactly once, on distinct shells
        inside = [tuple(t) for t in tri if set(t) <= set(ref.shells)]
        assert sorted(done) == sorted(inside) and len(done) == len(ref.sample) > 0
        assert ref.T == len(tri)
    finally:
        ref.close()


def test_full_run_sums_every_bin():
    n, box, edges, tri, delta = _case()
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    ref = ReferenceCPU(delta, box, edges, tri, processes=3, full=True)
    try:
        secs, sums = ref.full_run()
        assert secs > 0 and len(sums) == len(tri)
        want = O.triple_sums(of, of, of, tri)
        scale = O.triple_sums(np.abs(of), np.abs(of), np.abs(of), tri)
        assert np.all(np.abs(sums - want) <= 1e-5 * scale)
    finally:
        ref.close()
