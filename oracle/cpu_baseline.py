"""Timed CPU restatement of bskit's fast path -- TEST/BENCH INFRASTRUCTURE ONLY.

Only bench.py's ``cpu_baseline`` leg, its ``--impl reference`` arm and ``tests/``
(which check that the sampled work is the reference's work) use this module.
It times, on the host cores, the reference algorithm of
``FFTBispectrum.measure_bispectrum_faster`` (bskit/main.py:1846-1879) the way
bskit runs it under MPI:

* one inverse FFT per shell of the masked float32 spectrum (pmesh's parallel
  c2r; here scipy's pocketfft on the P host cores, ``scipy.fft.irfftn(...,
  workers=P)``, numpy's single-threaded ``np.fft.irfftn`` when scipy is
  absent), main.py:1846-1861;
* per triangle bin ``np.sum(I_a * I_b * I_c)`` on float32 fields,
  main.py:1875, computed slab-parallel by P host threads (numpy releases the
  interpreter lock in its array loops) that each sum their own x-slab, followed
  by a host-side sum -- bskit's MPI slab decomposition with gather+bcast,
  main.py:1878-1879.

``full_run()`` runs the whole workload (every shell, every bin) and times it:
for 256^3 and smaller grids.  A 512^3, 24 305-bin run takes core-hours, so
``step()`` times a bounded sample instead: a stratified subset of the shells
(spread over the whole k range) is transformed one shell per step, and each
step sums the workload's bins whose three shells are all among the shells
transformed so far and that include the new one -- every sampled bin once,
on its own three shell fields.  The per-bispectrum estimate is
    n_shells * mean(t_c2r) + t_r2c + T * (sampled triangle time / sampled bins),
labelled "extrapolated".
"""
import concurrent.futures as cf
import os
import time

import numpy as np


def _slab_sums(f, x0, x1, triples):
    out = np.empty(len(triples), dtype=np.float64)
    for t, (a, b, c) in enumerate(triples):
        out[t] = np.sum(f[a, x0:x1] * f[b, x0:x1] * f[c, x0:x1])
    return out


def _irfftn(spec, n, workers):
    try:
        import scipy.fft as sf
        return sf.irfftn(spec, s=(n, n, n), axes=(0, 1, 2), workers=workers)
    except ImportError:
        return np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2))


def stratified_shells(n_shells, m):
    """m shell indices spread evenly over [0, n_shells) (all of them when m >= n_shells)."""
    if m >= n_shells:
        return list(range(n_shells))
    return sorted(set(int(round(v)) for v in np.linspace(0, n_shells - 1, m)))


class ReferenceCPU(object):
    """bskit's fast-path algorithm on the host cores.

    ``delta`` is the real float32 mesh (host), ``triples`` the workload's full
    (T, 3) index list.  ``sample_shells`` is the number of shells the sampled
    steps transform (a stratified subset; the sampled bins are the workload's
    bins inside it).
    """

    def __init__(self, delta, box, shell_edges, triples, sample_shells=18, processes=None,
                 full=False):
        self.n = n = delta.shape[0]
        self.box = box
        self.edges = np.asarray(shell_edges, dtype=np.float64)
        self.triples = np.asarray(triples, dtype=np.int64).reshape(-1, 3)
        self.T = len(self.triples)
        self.P = processes or os.cpu_count() or 1
        t0 = time.perf_counter()
        try:
            import scipy.fft as sf
            self.dhat = sf.rfftn(delta.astype(np.float32), workers=self.P) / float(n) ** 3
        except ImportError:
            self.dhat = np.fft.rfftn(delta.astype(np.float32)) / float(n) ** 3
        self.t_r2c = time.perf_counter() - t0
        kf = 2 * np.pi / box
        q = np.fft.fftfreq(n, 1.0 / n) * kf
        qz = np.arange(n // 2 + 1) * kf
        self.kk = ((q[:, None, None] * q[:, None, None] + q[None, :, None] * q[None, :, None])
                   + qz[None, None, :] * qz[None, None, :]) ** 0.5
        self.shells = (list(range(len(self.edges))) if full
                       else stratified_shells(len(self.edges), sample_shells))
        self.slot = {s: k for k, s in enumerate(self.shells)}
        self.fields = np.empty((len(self.shells), n, n, n), dtype=np.float32)
        inside = np.isin(self.triples, self.shells).all(axis=1)
        self.sample = self.triples[inside]
        # the step at which each sampled bin becomes complete (its last shell transformed)
        order = {s: k for k, s in enumerate(self.shells)}
        last = np.array([max(order[int(v)] for v in t) for t in self.sample], dtype=np.int64)
        self.by_step = [self.sample[last == k] for k in range(len(self.shells))]
        self.bounds = np.linspace(0, n, self.P + 1).astype(int)
        self.pool = cf.ThreadPoolExecutor(max_workers=self.P)
        self.k = 0
        self.t_c2r = []
        self.t_tri = 0.0
        self.n_tri = 0
        self.last = {}

    def _transform(self, s):
        n = self.n
        lo, hi = self.edges[s]
        t0 = time.perf_counter()
        m = self.dhat * ((self.kk <= hi) & (self.kk >= lo))
        self.fields[self.slot[s]] = _irfftn(m.astype(np.complex64), n, self.P) * float(n) ** 3
        return time.perf_counter() - t0

    def _sums(self, tri):
        if len(tri) == 0:
            return np.zeros(0), 0.0
        loc = np.array([[self.slot[int(v)] for v in t] for t in tri], dtype=np.int64)
        t0 = time.perf_counter()
        parts = list(self.pool.map(lambda i: _slab_sums(self.fields, self.bounds[i],
                                                        self.bounds[i + 1], loc),
                                   range(self.P)))
        dt = time.perf_counter() - t0
        return np.sum(parts, axis=0), dt  # the host-side sum over slabs (main.py:1878-1879)

    def step(self):
        """Transform the next sampled shell, sum the bins it completes; return the
        extrapolated seconds per bispectrum from everything timed so far."""
        k = self.k % len(self.shells)
        t_fft = self._transform(self.shells[k])
        sums, t_tri = self._sums(self.by_step[k])
        self.k += 1
        self.t_c2r.append(t_fft)
        self.t_tri += t_tri
        self.n_tri += len(self.by_step[k])
        per_tri = self.t_tri / self.n_tri if self.n_tri else 0.0
        est = len(self.edges) * float(np.mean(self.t_c2r)) + self.t_r2c + self.T * per_tri
        self.last = {"t_c2r_s": t_fft, "t_triangle_sample_s": t_tri,
                     "sample_seconds": t_fft + t_tri, "bins_this_step": len(self.by_step[k]),
                     "sums": sums, "bins_timed": self.n_tri}
        return est

    def full_run(self):
        """Every shell and every bin of the workload (built with full=True): the measured
        seconds of one bispectrum, and the unnormalised triangle sums (no L^6/N^3 factor)."""
        assert len(self.shells) == len(self.edges), "build with full=True"
        t0 = time.perf_counter()
        for s in self.shells:
            self._transform(s)
        sums, _ = self._sums(self.triples)
        return time.perf_counter() - t0 + self.t_r2c, sums

    def describe(self):
        return ("bskit fast-path algorithm in numpy float32 on %d host cores: c2r per shell "
                "(scipy pocketfft, %d threads), x-slab parallel triangle sums on %d threads; "
                "sample: %d of %d shells (stratified over the k range), "
                "the %d of %d bins inside them, one shell per step, each bin summed once on its "
                "own three shell fields; r2c %.2f s; extrapolated to the full workload"
                % (self.P, self.P, self.P, len(self.shells), len(self.edges), len(self.sample),
                   self.T, self.t_r2c))

    def close(self):
        self.pool.shutdown(wait=True)
        self.fields = None
