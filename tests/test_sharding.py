"""Multi-rank host logic of the sharded bispectrum, as 2 gloo ranks on CPU: the
point partition covers the grid exactly once and the all-reduced partial sums
equal the oracle's whole-grid sums."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from bskit_gb300.sharding import point_range


def test_point_range_partition():
    for n in (64 ** 3, 40 ** 3, 14 ** 3, 1000):
        for world in (1, 2, 3, 4, 7):
            cuts = [point_range(n, r, world) for r in range(world)]
            assert cuts[0][0] == 0 and cuts[-1][1] == n
            for (a0, a1), (b0, b1) in zip(cuts, cuts[1:]):
                assert a1 == b0 and a0 <= a1
            assert all(c[0] % 128 == 0 for c in cuts)


class _FakePlan(object):
    def __init__(self, ngrid):
        self.ngrid = ngrid


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, result_q):
    import torch
    import torch.distributed as dist

    from bskit_gb300 import bins, synthetic
    from bskit_gb300.sharding import sharded_measure_b
    from oracle import bispec_oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, box = 16, 100.0
    kf = 2 * np.pi / box
    kw = dict(kmin=kf, kmax=4 * kf, dk=kf)
    edges = bins.generate_bin_edge_list(**kw)
    tri = bins.generate_triangle_bin_list(return_indices=True, **kw)
    delta = synthetic.lognormal_mesh(n, box, seed=2)
    f = O.shell_fields(O.spectrum(delta), n, box, edges).reshape(len(edges), -1)

    def partial(k0, k1):
        return torch.tensor([np.dot(f[i, k0:k1] * f[j, k0:k1], f[l, k0:k1]) for i, j, l in tri],
                            dtype=torch.float64)

    total = sharded_measure_b(_FakePlan(n), None, partial_fn=partial)
    full = O.triple_sums(O.shell_fields(O.spectrum(delta), n, box, edges),
                         O.shell_fields(O.spectrum(delta), n, box, edges),
                         O.shell_fields(O.spectrum(delta), n, box, edges), tri)
    result_q.put((rank, float(np.max(np.abs(total.numpy() - full) / np.abs(full).max()))))
    dist.destroy_process_group()


def test_two_rank_gloo_reduce_matches_oracle():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    res = dict(q.get(timeout=5) for _ in range(2))
    for p in procs:
        assert p.exitcode == 0
    assert res[0] < 1e-12 and res[1] < 1e-12


class _FakeShardPlan(object):
    """The bench's shard step on CPU: point-range partial sums of the oracle's fields."""

    def __init__(self, fields, tri):
        self.f = fields
        self.tri = tri
        self.ngrid = round(fields.shape[1] ** (1.0 / 3.0))

    def measure_b_range(self, tset, k0, k1, slots=(0, 0, 0), precision="bf16x3"):
        import torch
        f = self.f
        return torch.tensor([np.dot(f[i, k0:k1] * f[j, k0:k1], f[l, k0:k1])
                             for i, j, l in self.tri], dtype=torch.float64)

    @staticmethod
    def normalize(b, ntri):
        return b / ntri


def _bench_worker(rank, world, port, result_q):
    import sys

    import torch
    import torch.distributed as dist

    from bskit_gb300 import bins, synthetic
    from oracle import bispec_oracle as O

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, box = 16, 100.0
    kf = 2 * np.pi / box
    kw = dict(kmin=kf, kmax=4 * kf, dk=kf)
    edges = bins.generate_bin_edge_list(**kw)
    tri = bins.generate_triangle_bin_list(return_indices=True, **kw)
    delta = synthetic.lognormal_mesh(n, box, seed=2)
    of = O.shell_fields(O.spectrum(delta), n, box, edges)
    _, ntri, _ = O.grid_info(n, box, edges, tri)
    plan = _FakeShardPlan(of.reshape(len(edges), -1), tri)
    got = bench.shard_step(plan, None, torch.tensor(ntri), "bf16x3").numpy()
    want = O.triple_sums(of, of, of, tri) / ntri
    ok = ntri > 0
    result_q.put((rank, float(np.max(np.abs(got[ok] - want[ok]) / np.abs(want[ok]).max()))))
    dist.destroy_process_group()


def test_bench_shard_step_two_gloo_ranks():
    # bench.py --shard's step: each rank its point range, one all-reduce, the divide by N_tri
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_bench_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    res = dict(q.get(timeout=5) for _ in range(2))
    for p in procs:
        assert p.exitcode == 0
    assert res[0] < 1e-12 and res[1] < 1e-12
