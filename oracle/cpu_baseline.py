"""Timed CPU restatement of bskit's fast path -- TEST/BENCH INFRASTRUCTURE ONLY.

Only bench.py's ``cpu_baseline`` leg, its ``--impl reference`` arm and ``tests/``
(which check that the sampled work is the reference's work) use this module.
It times, on the host cores, the reference algorithm of
``FFTBispectrum.measure_bispectrum_faster`` (bskit/main.py:1846-1879) the way
bskit runs it under MPI:

* one inverse FFT per shell of the masked float32 spectrum (pmesh c2r; here
  numpy's pocketfft, ``np.fft.irfftn``), main.py:1846-1861;
* per triangle bin ``np.sum(I_a * I_b * I_c)`` on float32 fields,
  main.py:1875, computed slab-parallel by P worker processes
  (``OMP_NUM_THREADS=1`` each) that each sum their own x-slab, followed by a
  host-side sum -- bskit's MPI slab decomposition with gather+bcast,
  main.py:1878-1879.

A full 512^3, 24 305-bin run takes core-hours, so the timing is a bounded
sample: one shell FFT (credited with perfect P-way scaling, as pfft would
give bskit) and a stratified sample of triangle bins, extrapolated to the
whole workload.  The sample size is part of the returned record.
"""
import multiprocessing as mp
import os
import time

import numpy as np

_FIELDS = None


def _init_worker(shm_name, shape):
    global _FIELDS
    from multiprocessing import shared_memory
    os.environ["OMP_NUM_THREADS"] = "1"
    shm = shared_memory.SharedMemory(name=shm_name)
    _FIELDS = (shm, np.ndarray(shape, dtype=np.float32, buffer=shm.buf))


def _slab_sums(args):
    x0, x1, triples = args
    f = _FIELDS[1]
    out = np.empty(len(triples), dtype=np.float64)
    for t, (a, b, c) in enumerate(triples):
        out[t] = np.sum(f[a, x0:x1] * f[b, x0:x1] * f[c, x0:x1])
    return out


class ReferenceCPU(object):
    """bskit's fast-path algorithm on the host cores, timed on bounded samples.

    ``delta`` is the real float32 mesh (host), ``triples`` the workload's full
    (T, 3) index list.  The per-unit costs do not depend on which shells are
    involved (every shell field is a dense N^3 array, every triangle sum
    touches 3 N^3 floats), so one step times: the c2r of one masked shell and
    ``n_tri_sample`` slab-parallel triangle sums over three shell fields (the
    transformed shell and two shifted copies).  The mesh r2c is timed once in
    ``__init__``.  ``step()`` returns the extrapolated seconds per bispectrum
        n_shells * t_c2r / P + t_r2c / P + T * t_tri / n_tri_sample.
    """

    def __init__(self, delta, box, shell_edges, triples, n_tri_sample=24, processes=None):
        from multiprocessing import shared_memory
        self.n = n = delta.shape[0]
        self.box = box
        self.edges = np.asarray(shell_edges, dtype=np.float64)
        self.T = len(triples)
        self.P = processes or os.cpu_count() or 1
        self.n_tri_sample = n_tri_sample
        t0 = time.perf_counter()
        self.dhat = np.fft.rfftn(delta.astype(np.float32)) / float(n) ** 3
        self.t_r2c = time.perf_counter() - t0
        kf = 2 * np.pi / box
        q = np.fft.fftfreq(n, 1.0 / n) * kf
        qz = np.arange(n // 2 + 1) * kf
        self.kk = ((q[:, None, None] * q[:, None, None] + q[None, :, None] * q[None, :, None])
                   + qz[None, None, :] * qz[None, None, :]) ** 0.5
        self.shm = shared_memory.SharedMemory(create=True, size=3 * n ** 3 * 4)
        self.fields = np.ndarray((3, n, n, n), dtype=np.float32, buffer=self.shm.buf)
        combos = [(a, b, c) for a in range(3) for b in range(a + 1) for c in range(b + 1)]
        self.loc = np.array(combos)[np.arange(n_tri_sample) % len(combos)]
        self.bounds = np.linspace(0, n, self.P + 1).astype(int)
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(self.P, initializer=_init_worker,
                             initargs=(self.shm.name, self.fields.shape))
        self.pool.map(_slab_sums, [(0, 1, self.loc[:1])] * self.P)  # start the workers
        self.shell = len(self.edges) // 2
        self.last = {}

    def step(self):
        n = self.n
        lo, hi = self.edges[self.shell]
        t0 = time.perf_counter()
        m = self.dhat * ((self.kk <= hi) & (self.kk >= lo))
        self.fields[0] = np.fft.irfftn(m.astype(np.complex64), s=(n, n, n),
                                       axes=(0, 1, 2)) * float(n) ** 3
        t_fft = time.perf_counter() - t0
        self.fields[1] = np.roll(self.fields[0], 1, axis=0)
        self.fields[2] = np.roll(self.fields[0], 2, axis=1)
        t0 = time.perf_counter()
        parts = self.pool.map(_slab_sums, [(self.bounds[i], self.bounds[i + 1], self.loc)
                                           for i in range(self.P)])
        t_tri = time.perf_counter() - t0
        sums = np.sum(parts, axis=0)  # the host-side sum over slabs (main.py:1878-1879)
        est = len(self.edges) * t_fft / self.P + self.t_r2c / self.P + self.T * t_tri / len(self.loc)
        self.last = {"t_c2r_s": t_fft, "t_triangle_sample_s": t_tri, "sample_seconds": t_fft + t_tri,
                     "sums": sums}
        return est

    def describe(self):
        return ("bskit fast-path algorithm in numpy float32 on %d host processes (x-slab "
                "parallel triangle sums, OMP_NUM_THREADS=1); per step: c2r of 1 of %d shells "
                "+ %d of %d triangle sums, r2c timed once (%.2f s); FFT cost credited with "
                "perfect %d-way scaling; extrapolated to the full workload"
                % (self.P, len(self.edges), len(self.loc), self.T, self.t_r2c, self.P))

    def close(self):
        try:
            self.pool.close()
            self.pool.join()
        finally:
            self.shm.close()
            self.shm.unlink()
