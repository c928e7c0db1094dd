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
  other shell sets are evicted, least recently used first; groups admitted by
  ``prepare`` only when the requesting shell set has no group at all);
* batches requests of one shell set -- one N_grid, box and shell list -- whatever
  their bin sets (all / equilateral / squeezed / isosceles, auto or cross) and
  precisions: a batch of up to ``max_batch`` such requests runs on the instances
  of one group, request k on instance k;
* runs every request as a CUDA graph (paint -> shell fields -> contraction ->
  normalisation -> device-to-host copy of B) captured once per (instance, bin
  set): ``Scheduler.prepare`` captures them ahead of the stream for the
  configurations it is given, so no capture sits on the dispatch path of a
  prepared configuration (a configuration first seen in the stream is captured
  when first dispatched);
* replays the graphs of a batch on the group's per-instance streams, and batches
  of different groups on theirs, so requests that arrive while others are on the
  GPU start as soon as an instance and memory are free and their work overlaps on
  the device;
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
    """Scheduler view of a request: its shell-set key (the batching key) and bin-set key."""

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
        self.pending = collections.OrderedDict()   # shell_key -> deque of jobs (FIFO)
        self.groups = []                           # all resident groups
        self.busy = {}                             # group -> (batch, jobs)
        self.last_used = {}
        self.used = 0
        self.done = []
        self.log = []

    # -------------------------------------------------------------- intake
    def submit(self, req):
        job = Job(req)
        self.pending.setdefault(job.shell_key, collections.deque()).append(job)
        return job

    def prepare(self, requests, groups=None):
        """Admit up to ``groups`` (default max_groups) groups per shell set of the given
        configurations and capture, on every instance, the graph of every bin set among
        them, before any request is served."""
        jobs = [Job(r) for r in requests]
        per_shell = collections.OrderedDict()
        for j in jobs:
            per_shell.setdefault(j.shell_key, []).append(j)
        want = self.max_groups if groups is None else int(groups)
        for key, js in per_shell.items():
            while sum(1 for g in self.groups if g.shell_key == key) < want:
                g = self._admit_group(js[0])
                if g is None:
                    break
                g.pinned = True  # prepared ahead: never evicted to make room for another group
            for g in self.groups:
                if g.shell_key == key:
                    for j in js:
                        self.backend.prepare(g, j)
        return jobs

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

    def _evict_for(self, need, pinned_too=False):
        """Destroy idle groups (least recently used first) until ``need`` bytes fit.  Groups
        admitted by ``prepare`` are kept unless ``pinned_too``."""
        idle = [g for g in self.groups if g not in self.busy
                and (pinned_too or not getattr(g, "pinned", False))]
        if self.used - sum(g.footprint for g in idle) + need > self.mem_budget:
            return False  # would not fit even with all of them gone: destroy nothing
        idle.sort(key=lambda g: self.last_used.get(g, 0.0))
        while self.used + need > self.mem_budget and idle:
            g = idle.pop(0)
            self.backend.destroy_group(g)
            self.groups.remove(g)
            self.used -= g.footprint
            self.log.append(("evict", g.shell_key[:2]))
        return self.used + need <= self.mem_budget

    def _admit_group(self, job):
        have = sum(1 for g in self.groups if g.shell_key == job.shell_key)
        if have >= self.max_groups:
            return None
        sizes = []
        size = self.max_batch
        while size >= 1:
            sizes.append(size)
            size //= 2
        # the largest group that fits, evicting only groups not admitted by ``prepare``; a
        # shell set with no group at all may then take prepared groups' memory, one that has
        # a group waits for it instead
        for pinned_too in ((False, True) if have == 0 else (False,)):
            for size in sizes:
                need = self.backend.group_footprint(job, size)
                if self.used + need <= self.mem_budget or self._evict_for(need, pinned_too):
                    g = self.backend.create_group(job, size)
                    g.footprint = need
                    self.groups.append(g)
                    self.used += need
                    self.log.append(("admit", job.shell_key[:2], size, need))
                    return g
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
        # the shell set whose oldest request waits longest first; a batch takes that set's
        # requests in arrival order, whatever their bin sets
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
                self.log.append(("batch", key[:2], len(jobs), len({j.bin_key for j in jobs})))
                self.busy[g] = (self.backend.launch(g, jobs), jobs)
                self.last_used[g] = t
            if not q:
                del self.pending[key]
        return now

    def close(self):
        """Wait for the batches in flight, then destroy every group (device memory, graphs)."""
        while self.busy:
            self.step()
        for g in list(self.groups):
            self.backend.destroy_group(g)
        self.groups = []
        self.used = 0
        if hasattr(self.backend, "close"):
            self.backend.close()

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
    """Drives the CUDA engine: one plan per instance, one graph per (instance, bin set)."""

    def __init__(self, device=None, use_graphs=True):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.use_graphs = use_graphs
        self.gridinfo = {}      # bin_key -> (ntri, kmean) device tensors
        self.probe = {}         # shell_key -> measured footprint of one instance
        self.captures = 0       # graphs captured (prepare + dispatch)
        self.captures_at_dispatch = 0
        self.captures_at_dispatch_by_n = {}

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
        inst.graphs = {}
        inst.warm = set()
        return inst

    def _warm(self, inst, job):
        """One eager run so that every lazily allocated buffer exists before capture."""
        if job.bin_key in inst.warm:
            return
        torch = self.torch
        slots = (0, 0, 1) if job.req.num_fields == 2 else (0, 0, 0)
        for s in range(job.req.num_fields):
            inst.dmesh[s].zero_()
            inst.plan.paint(s, inst.dmesh[s])
        ts = self._tset(inst, job)
        inst.plan.measure_b(ts, slots=slots, precision=job.req.precision)
        torch.cuda.synchronize(self.device)
        inst.warm.add(job.bin_key)

    def _tset(self, inst, job):
        ts = inst.tsets.get(job.bin_key)
        if ts is None:
            ts = inst.plan.triangles(job.tri)
            inst.tsets[job.bin_key] = ts
        return ts

    def group_footprint(self, job, size):
        fp = self.probe.get(job.shell_key)
        if fp is None:
            # an instance serves auto and cross requests of its shell set alike: measure it
            # with both field slots built
            inst = self._new_instance(job)
            self._warm(inst, job)
            inst.dmesh[1].zero_()
            inst.plan.paint(1, inst.dmesh[1])
            inst.plan.measure_b(self._tset(inst, job), slots=(0, 0, 1),
                                precision=job.req.precision)
            self.torch.cuda.synchronize(self.device)
            fp = inst.plan.footprint() + 2 * job.req.nmesh ** 3 * 4
            self.probe[job.shell_key] = fp
            inst.plan.close()
        return fp * size

    def create_group(self, job, size):
        torch = self.torch
        g = _Group(job.shell_key, size)
        g.instances = [self._new_instance(job) for _ in range(size)]
        g.streams = [torch.cuda.Stream(device=self.device) for _ in range(size)]
        return g

    def destroy_group(self, g):
        for inst in g.instances:
            inst.graphs = {}
            inst.out = {}
            inst.dmesh = []
            inst.plan.close()
        g.instances = []

    def close(self):
        self.gridinfo.clear()
        self.torch.cuda.synchronize(self.device)
        self.torch.cuda.empty_cache()

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

    def _graph(self, inst, stream, job):
        """The instance's captured pipeline for the job's bin set (captured on first use)."""
        torch = self.torch
        graph = inst.graphs.get(job.bin_key)
        if graph is not None:
            return graph
        self._warm(inst, job)
        ntri = self._gridinfo(inst, job)[0]
        self._enqueue(inst, job, ntri)  # allocate the pinned outputs eagerly
        torch.cuda.synchronize(self.device)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream, capture_error_mode="thread_local"):
            self._enqueue(inst, job, ntri)
        inst.graphs[job.bin_key] = graph
        self.captures += 1
        return graph

    def prepare(self, g, job):
        """Capture the job's bin-set graph on every instance of the group (ahead of serving)."""
        if not self.use_graphs:
            for inst in g.instances:
                self._warm(inst, job)
                self._gridinfo(inst, job)
            return
        for inst, stream in zip(g.instances, g.streams):
            self._graph(inst, stream, job)

    def launch(self, g, jobs):
        torch = self.torch
        done = []
        for k, job in enumerate(jobs):
            inst, stream = g.instances[k], g.streams[k]
            ntri, kmean = self._gridinfo(inst, job)
            graph = None
            if self.use_graphs:
                if job.bin_key not in inst.graphs:
                    self.captures_at_dispatch += 1
                    n = job.req.nmesh
                    self.captures_at_dispatch_by_n[n] = self.captures_at_dispatch_by_n.get(n, 0) + 1
                # capture before this request's mesh is staged: the capture's warm-up run
                # overwrites the instance's mesh buffers
                graph = self._graph(inst, stream, job)
            with torch.cuda.stream(stream):
                inst.dmesh[0].copy_(torch.as_tensor(job.req.mesh), non_blocking=True)
                if job.req.num_fields == 2:
                    inst.dmesh[1].copy_(torch.as_tensor(job.req.second), non_blocking=True)
                if graph is not None:
                    graph.replay()
                else:
                    self._enqueue(inst, job, ntri)
                e = torch.cuda.Event()
                e.record(stream)
            done.append((e, inst, job, ntri, kmean))
        return done

    def poll(self, batch):
        if not all(e.query() for e, _, _, _, _ in batch):
            return False
        for _, inst, job, ntri, kmean in batch:
            u = job.req.spec.get("pos_units_mpcoverh", 1.0)
            out = inst.out[job.bin_key]
            job.req.B = out[0].numpy().copy() * u ** 6
            job.req.B_unnorm = out[1].numpy().copy() * u ** 6
            job.req.N_tri = ntri.cpu().numpy()
            job.req.k_mean = kmean.cpu().numpy() / u
        return True


def make_server(mem_budget=None, max_batch=4, max_groups=4, device=None, use_graphs=True):
    """Scheduler + CUDA backend; mem_budget defaults to 80% of the free device memory."""
    import torch
    backend = EngineBackend(device=device, use_graphs=use_graphs)
    if mem_budget is None:
        free, _ = torch.cuda.mem_get_info(backend.device)
        mem_budget = int(0.8 * free)
    return Scheduler(backend, mem_budget, max_batch=max_batch, max_groups=max_groups)
