"""Continuous-batching bispectrum server.

A request is one bispectrum job: a real N^3 mesh (optionally a second one for a
cross bispectrum <AAB>), a box size, a bin specification (bskit's triangle
types) and a precision.  The server

* keeps engine state resident per (Nmesh, BoxSize, shell list): plans whose
  spectra, shell fields and cuFFT plans stay allocated, the triangle sets of
  every bin set seen, and their grid information (triangle counts, k_mean),
  computed once;
* admits work by HBM footprint: a group of engine instances for a shell set is
  created only when its measured footprint fits in the budget (idle groups of
  other shell sets are evicted, least recently used first);
* batches requests that share a bin set into one captured CUDA graph per batch
  size (paint -> shell fields -> contraction -> normalisation -> device-to-host
  copy of B for every request of the batch, as parallel graph branches);
* runs batches of different groups on different CUDA streams, so requests
  that arrive while others are on the GPU start as soon as a group and memory
  are free and their work overlaps on the device;
* records arrival, dispatch and completion times (p50 / p99 latency).

The scheduling logic (``Scheduler``) is independent of CUDA; ``EngineBackend``
drives the GPU and ``tests/test_serving.py`` also runs the scheduler against a
simulated backend.
"""
import collections
import time

import numpy as np

from . import bins as _bins

TRIANGLE_TYPES = ("all", "equilateral", "squeezed", "isosceles")
PRECISIONS = ("bf16x3", "fp32", "bf16", "fp64")


class Request(object):
    """One bispectrum job.

    mesh / second : float32 N^3 arrays (host numpy or torch, ideally pinned)
    spec : dict of bskit bin arguments: kmin, kmax, dk, triangle_type and, as
        needed, num_lowk_bins, dk_high, squeezed_bin_index, isos_mult, isos_tol
    """

    def __init__(self, rid, mesh, box, spec, second=None, precision="bf16x3", arrival=0.0):
        # checked here, at submission: a bad request must not fail later inside a batch
        for m in (mesh, second):
            if m is not None and (len(m.shape) != 3 or len(set(m.shape)) != 1):
                raise ValueError("meshes must be cubic N^3 arrays")
        if second is not None and tuple(second.shape) != tuple(mesh.shape):
            raise ValueError("the second mesh must have the first mesh's shape")
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % (PRECISIONS,))
        self.rid = rid
        self.mesh = mesh
        self.second = second
        self.box = float(box)
        self.spec = dict(spec)
        self.precision = precision
        self.arrival = float(arrival)
        self.t_dispatch = None
        self.t_done = None
        self.B = None
        self.N_tri = None
        self.k_mean = None
        self.B_unnorm = None

    @property
    def nmesh(self):
        return int(self.mesh.shape[0])

    @property
    def num_fields(self):
        return 2 if self.second is not None else 1

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def bin_lists(spec, num_fields=1):
    """(shell edges (n, 2), triangle indices (T, 3)) of a bin specification."""
    t = spec.get("triangle_type", "all")
    kw = dict(kmin=spec["kmin"], kmax=spec["kmax"], dk=spec["dk"],
              num_lowk_bins=spec.get("num_lowk_bins", 0), dk_high=spec.get("dk_high", -1.))
    edges = _bins.generate_bin_edge_list(**kw)
    if t == "all":
        tri = _bins.generate_triangle_bin_list(num_fields=num_fields, return_indices=True, **kw)
    elif t == "equilateral":
        tri = _bins.generate_equilateral_triangle_bin_list(return_indices=True, **kw)
    elif t == "squeezed":
        tri = _bins.generate_squeezed_triangle_bin_list(
            squeezed_bin_index=spec.get("squeezed_bin_index", 0), return_indices=True, **kw)
    elif t == "isosceles":
        tri = _bins.generate_isosceles_triangle_bin_list(
            isos_mult=spec.get("isos_mult", 2.0), isos_tol=spec.get("isos_tol", 0.1),
            return_indices=True, **kw)
    else:
        raise ValueError("triangle_type must be one of %s" % (TRIANGLE_TYPES,))
    return edges, np.asarray(tri, dtype=np.int32).reshape(-1, 3)


class Job(object):
    """Scheduler view of a request: its shell-set key and bin-set key."""

    def __init__(self, req):
        self.req = req
        self.edges, self.tri = bin_lists(req.spec, req.num_fields)
        self.shell_key = (req.nmesh, req.box, self.edges.tobytes())
        self.bin_key = self.shell_key + (self.tri.tobytes(), req.num_fields, req.precision)


class Scheduler(object):
    """Admission, batching and dispatch; knows nothing about CUDA.

    backend must provide:
      group_footprint(job, size) -> bytes of a new group of ``size`` instances
      create_group(job, size) -> group handle (with .size, .shell_key)
      destroy_group(group)
      launch(group, jobs) -> batch handle (asynchronous)
      poll(batch) -> True when finished (results written into the requests)
    """

    def __init__(self, backend, mem_budget, max_batch=4, max_groups=4, clock=time.perf_counter):
        self.backend = backend
        self.mem_budget = int(mem_budget)
        self.max_batch = int(max_batch)
        self.max_groups = int(max_groups)   # per shell set
        self.clock = clock
        self.pending = collections.OrderedDict()   # bin_key -> deque of jobs (FIFO)
        self.groups = []                           # all resident groups
        self.busy = {}                             # group -> (batch, jobs)
        self.last_used = {}
        self.used = 0
        self.done = []
        self.log = []

    # -------------------------------------------------------------- intake
    def submit(self, req):
        job = Job(req)
        self.pending.setdefault(job.bin_key, collections.deque()).append(job)
        return job

    def n_pending(self):
        return sum(len(q) for q in self.pending.values())

    def idle(self):
        return not self.busy and self.n_pending() == 0

    # -------------------------------------------------------------- admission
    def _free_group(self, shell_key):
        for g in self.groups:
            if g.shell_key == shell_key and g not in self.busy:
                return g
        return None

    def _evict_for(self, need):
        """Destroy idle groups (least recently used first) until ``need`` bytes fit."""
        idle = [g for g in self.groups if g not in self.busy]
        idle.sort(key=lambda g: self.last_used.get(g, 0.0))
        while self.used + need > self.mem_budget and idle:
            g = idle.pop(0)
            self.backend.destroy_group(g)
            self.groups.remove(g)
            self.used -= g.footprint
            self.log.append(("evict", g.shell_key[:2]))
        return self.used + need <= self.mem_budget

    def _admit_group(self, job):
        if sum(1 for g in self.groups if g.shell_key == job.shell_key) >= self.max_groups:
            return None
        size = self.max_batch
        while size >= 1:
            need = self.backend.group_footprint(job, size)
            if self.used + need <= self.mem_budget or self._evict_for(need):
                g = self.backend.create_group(job, size)
                g.footprint = need
                self.groups.append(g)
                self.used += need
                self.log.append(("admit", job.shell_key[:2], size, need))
                return g
            size //= 2
        return None

    # -------------------------------------------------------------- main step
    def step(self):
        """Retire finished batches, then dispatch as much pending work as fits."""
        now = self.clock()
        for g, (batch, jobs) in list(self.busy.items()):
            if self.backend.poll(batch):
                t = self.clock()
                for j in jobs:
                    j.req.t_done = t
                    self.done.append(j.req)
                del self.busy[g]
                self.last_used[g] = t
        # oldest waiting request first
        order = sorted(self.pending.keys(), key=lambda k: self.pending[k][0].req.arrival
                       if self.pending[k] else float("inf"))
        for key in order:
            q = self.pending[key]
            while q:
                g = self._free_group(q[0].shell_key)
                if g is None:
                    g = self._admit_group(q[0])
                if g is None:
                    break
                jobs = [q.popleft() for _ in range(min(g.size, len(q)))]
                t = self.clock()
                for j in jobs:
                    j.req.t_dispatch = t
                self.busy[g] = (self.backend.launch(g, jobs), jobs)
                self.last_used[g] = t
            if not q:
                del self.pending[key]
        return now

    def run(self, requests, realtime=True, poll_sleep=0.0):
        """Feed requests at their arrival times (seconds after start) and serve them all."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = self.clock()
        i = 0
        while i < len(reqs) or not self.idle():
            now = self.clock() - t0
            while i < len(reqs) and (reqs[i].arrival <= now or not realtime):
                reqs[i].arrival += t0
                self.submit(reqs[i])
                i += 1
            self.step()
            if poll_sleep:
                time.sleep(poll_sleep)
        return reqs


def latency_stats(reqs):
    lat = np.array([r.latency for r in reqs if r.latency is not None]) * 1e3
    if len(lat) == 0:
        return {}
    t_first = min(r.arrival for r in reqs)
    t_last = max(r.t_done for r in reqs if r.t_done is not None)
    return {"requests": int(len(lat)), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "max_ms": float(lat.max()), "throughput_rps": len(lat) / (t_last - t_first)}


class _Instance(object):
    pass


class _Group(object):
    def __init__(self, shell_key, size):
        self.shell_key = shell_key
        self.size = size
        self.footprint = 0


class EngineBackend(object):
    """Drives the CUDA engine: one plan per instance, graphs per (bin set, batch size)."""

    def __init__(self, device=None, use_graphs=True):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.use_graphs = use_graphs
        self.gridinfo = {}      # bin_key -> (ntri, kmean) device tensors
        self.probe = {}         # shell_key -> measured footprint of one instance

    # -------------------------------------------------------------- resources
    def _new_instance(self, job):
        from .engine import Plan
        torch = self.torch
        req = job.req
        inst = _Instance()
        inst.plan = Plan(req.nmesh, req.box, job.edges, device=self.device)
        n = req.nmesh
        inst.dmesh = [torch.empty((n, n, n), dtype=torch.float32, device=self.device)
                      for _ in range(2)]
        inst.tsets = {}
        inst.out = {}
        return inst

    def _warm(self, inst, job):
        """One eager run so that every lazily allocated buffer exists before capture."""
        torch = self.torch
        slots = (0, 0, 1) if job.req.num_fields == 2 else (0, 0, 0)
        for s in range(job.req.num_fields):
            inst.dmesh[s].zero_()
            inst.plan.paint(s, inst.dmesh[s])
        ts = self._tset(inst, job)
        inst.plan.measure_b(ts, slots=slots, precision=job.req.precision)
        torch.cuda.synchronize(self.device)

    def _tset(self, inst, job):
        ts = inst.tsets.get(job.bin_key)
        if ts is None:
            ts = inst.plan.triangles(job.tri)
            inst.tsets[job.bin_key] = ts
        return ts

    def group_footprint(self, job, size):
        fp = self.probe.get((job.shell_key, job.req.num_fields))
        if fp is None:
            inst = self._new_instance(job)
            self._warm(inst, job)
            fp = inst.plan.footprint() + 2 * job.req.nmesh ** 3 * 4
            self.probe[(job.shell_key, job.req.num_fields)] = fp
            inst.plan.close()
        return fp * size

    def create_group(self, job, size):
        torch = self.torch
        g = _Group(job.shell_key, size)
        g.instances = [self._new_instance(job) for _ in range(size)]
        g.streams = [torch.cuda.Stream(device=self.device) for _ in range(size)]
        g.graphs = {}
        return g

    def destroy_group(self, g):
        for inst in g.instances:
            inst.plan.close()
        g.instances = []
        g.graphs = {}

    # -------------------------------------------------------------- grid info
    def _gridinfo(self, inst, job):
        gi = self.gridinfo.get(job.bin_key)
        if gi is None:
            ts = self._tset(inst, job)
            gi = inst.plan.gridinfo(ts)
            inst.plan.sync_check()
            self.gridinfo[job.bin_key] = gi
        return gi

    # -------------------------------------------------------------- execution
    def _enqueue(self, inst, job, ntri):
        """paint -> fields -> contraction -> normalise -> D2H, on the current stream."""
        plan = inst.plan
        slots = (0, 0, 1) if job.req.num_fields == 2 else (0, 0, 0)
        ts = self._tset(inst, job)
        for s in range(job.req.num_fields):
            plan.paint(s, inst.dmesh[s])
        b = plan.measure_b(ts, slots=slots, precision=job.req.precision)
        bn = plan.normalize(b, ntri)
        key = job.bin_key
        out = inst.out.get(key)
        if out is None:
            T = len(job.tri)
            out = (self.torch.empty(T, dtype=self.torch.float64).pin_memory(),
                   self.torch.empty(T, dtype=self.torch.float64).pin_memory())
            inst.out[key] = out
        out[0].copy_(bn, non_blocking=True)
        out[1].copy_(b, non_blocking=True)
        return out

    def _graph(self, g, jobs):
        """Captured graph running len(jobs) pipelines of one bin set as parallel branches."""
        torch = self.torch
        key = (jobs[0].bin_key, len(jobs))
        gr = g.graphs.get(key)
        if gr is not None:
            return gr
        for inst in g.instances[:len(jobs)]:
            self._warm(inst, jobs[0])
        ntri = self._gridinfo(g.instances[0], jobs[0])[0]
        for inst in g.instances[:len(jobs)]:
            self._enqueue(inst, jobs[0], ntri)  # allocate pinned outputs eagerly
        torch.cuda.synchronize(self.device)
        graph = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(device=self.device)
        with torch.cuda.graph(graph, stream=cap, capture_error_mode="thread_local"):
            fork = torch.cuda.current_stream()
            start = torch.cuda.Event()
            start.record(fork)
            ends = []
            for k, inst in enumerate(g.instances[:len(jobs)]):
                s = g.streams[k]
                s.wait_event(start)
                with torch.cuda.stream(s):
                    self._enqueue(inst, jobs[0], ntri)
                    e = torch.cuda.Event()
                    e.record(s)
                    ends.append(e)
            for e in ends:
                fork.wait_event(e)
        g.graphs[key] = graph
        return graph

    def launch(self, g, jobs):
        torch = self.torch
        stream = g.streams[0]
        ntri, kmean = self._gridinfo(g.instances[0], jobs[0])
        # capture (first batch of this bin set and size only) before the meshes are staged:
        # the warm-up run of the capture overwrites the instances' mesh buffers
        graph = self._graph(g, jobs) if self.use_graphs else None
        # host -> device copies of the batch's meshes (from the requests' own buffers)
        with torch.cuda.stream(stream):
            for inst, job in zip(g.instances, jobs):
                inst.dmesh[0].copy_(torch.as_tensor(job.req.mesh), non_blocking=True)
                if job.req.num_fields == 2:
                    inst.dmesh[1].copy_(torch.as_tensor(job.req.second), non_blocking=True)
        if graph is not None:
            with torch.cuda.stream(stream):
                graph.replay()
        else:
            with torch.cuda.stream(stream):
                for inst, job in zip(g.instances, jobs):
                    self._enqueue(inst, job, ntri)
        done = torch.cuda.Event()
        done.record(stream)
        return (done, g, jobs, kmean, ntri)

    def poll(self, batch):
        done, g, jobs, kmean, ntri = batch
        if not done.query():
            return False
        u = jobs[0].req.spec.get("pos_units_mpcoverh", 1.0)
        nt = ntri.cpu().numpy()
        km = kmean.cpu().numpy()
        for inst, job in zip(g.instances, jobs):
            out = inst.out[job.bin_key]
            job.req.B = out[0].numpy().copy() * u ** 6
            job.req.B_unnorm = out[1].numpy().copy() * u ** 6
            job.req.N_tri = nt
            job.req.k_mean = km / u
        return True


def make_server(mem_budget=None, max_batch=4, max_groups=4, device=None, use_graphs=True):
    """Scheduler + CUDA backend; mem_budget defaults to 80% of the free device memory."""
    import torch
    backend = EngineBackend(device=device, use_graphs=use_graphs)
    if mem_budget is None:
        free, _ = torch.cuda.mem_get_info(backend.device)
        mem_budget = int(0.8 * free)
    return Scheduler(backend, mem_budget, max_batch=max_batch, max_groups=max_groups)
