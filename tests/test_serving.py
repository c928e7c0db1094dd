"""Serving: scheduler logic on CPU with a simulated backend, and on the GPU the
same results for every request alone and in a concurrent mix."""
import numpy as np
import pytest

from bskit_gb300 import serving


class FakeClock(object):
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-4
        return self.t


class FakeGroup(serving._Group):
    pass


class FakeBackend(object):
    """Instances cost 10 units of memory per mesh cell side; a batch takes 5 polls."""

    def __init__(self):
        self.created = []
        self.destroyed = []
        self.launched = []
        self.order = []
        self.prepared = []

    def group_footprint(self, job, size):
        return 10 * job.req.nmesh * size

    def create_group(self, job, size):
        g = FakeGroup(job.shell_key, size)
        self.created.append((job.req.nmesh, size))
        return g

    def destroy_group(self, g):
        self.destroyed.append(g.shell_key[0])

    def launch(self, g, jobs):
        self.launched.append((g.shell_key[0], len(jobs)))
        self.order.extend(j.req.rid for j in jobs)
        return {"left": 5, "jobs": jobs}

    def prepare(self, g, job):
        self.prepared.append((g.shell_key[0], job.req.spec["triangle_type"]))

    def poll(self, batch):
        batch["left"] -= 1
        if batch["left"] > 0:
            return False
        for j in batch["jobs"]:
            j.req.B = np.full(len(j.tri), float(j.req.rid))
        return True


def _req(rid, n, t="all", arrival=0.0, cross=False):
    kf = 2 * np.pi / 100.0
    mesh = np.zeros((n, n, n), np.float32)
    spec = dict(kmin=kf, kmax=n / 4 * kf, dk=2 * kf, triangle_type=t)
    return serving.Request(rid, mesh, 100.0, spec, second=mesh if cross else None, arrival=arrival)


def test_batches_mix_bin_sets_of_one_shell_set_in_arrival_order():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=10 ** 6, max_batch=4, max_groups=3, clock=FakeClock())
    reqs = [_req(i, 32, "all" if i % 2 == 0 else "equilateral", arrival=1e-3 * i)
            for i in range(10)]
    sch.run(reqs, realtime=False)
    assert all(r.B is not None and r.B[0] == r.rid for r in reqs)
    # one shell set (both bin sets share the shells): batches of up to max_batch requests
    # that mix the bin sets, dispatched in arrival order
    assert all(1 <= k <= 4 for _, k in be.launched)
    assert sum(k for _, k in be.launched) == 10
    assert be.order == list(range(10))
    mixed = [e for e in sch.log if e[0] == "batch" and e[3] > 1]
    assert mixed, "no batch held two bin sets"
    # groups are per shell set; busy groups scale out
    assert all(c == (32, 4) for c in be.created) and 1 <= len(be.created) <= 3
    lat = serving.latency_stats(reqs)
    assert lat["requests"] == 10 and lat["p99_ms"] >= lat["p50_ms"]


def test_prepare_admits_groups_and_captures_every_bin_set_ahead():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=10 ** 6, max_batch=2, max_groups=2, clock=FakeClock())
    cfg = [_req(0, 16, "all"), _req(1, 16, "equilateral"), _req(2, 32, "squeezed")]
    sch.prepare(cfg)
    # two groups per shell set, every bin set of the set captured on each
    assert sorted(be.created) == [(16, 2), (16, 2), (32, 2), (32, 2)]
    assert sorted(be.prepared) == sorted([(16, "all"), (16, "equilateral")] * 2 +
                                         [(32, "squeezed")] * 2)
    reqs = [_req(i, 16, "all" if i % 2 else "equilateral") for i in range(6)]
    sch.run(reqs, realtime=False)
    assert len(be.created) == 4 and all(r.B is not None for r in reqs)


def test_prepared_groups_are_kept_unless_a_shell_set_has_no_group():
    be = FakeBackend()
    # 32^3 groups of 2 cost 640, 64^3 ones 1280: the budget holds two 32^3 groups and one 64^3
    sch = serving.Scheduler(be, mem_budget=2600, max_batch=2, max_groups=2, clock=FakeClock())
    sch.prepare([_req(0, 32)])
    sch.prepare([_req(1, 64)], groups=1)
    assert sorted(be.created) == [(32, 2), (32, 2), (64, 2)] and sch.used == 2560
    # more 64^3 work than its prepared group takes at once: no second 64^3 group evicts the
    # prepared 32^3 groups; the requests wait for the prepared group
    reqs = [_req(10 + i, 64) for i in range(6)]
    sch.run(reqs, realtime=False)
    assert all(r.B is not None for r in reqs)
    assert be.destroyed == [] and len(be.created) == 3
    # a shell set with no group at all may still take a prepared group's memory
    r = _req(20, 128)
    sch.run([r], realtime=False)
    assert r.B is not None and be.created[-1] == (128, 2)
    assert sorted(be.destroyed) == [32, 32, 64]


def test_no_eviction_for_a_group_that_cannot_fit_and_smaller_groups_tried_first():
    be = FakeBackend()
    # a 64^3 group of 4 (2560) cannot fit a 2000 budget even in an empty server; a group of
    # 2 (1280) fits beside the prepared 16^3 group of 4 (640): it is admitted, and the
    # prepared group is not destroyed on the way by the attempt at 4
    sch = serving.Scheduler(be, mem_budget=2000, max_batch=4, max_groups=1, clock=FakeClock())
    sch.prepare([_req(0, 16)])
    r = _req(1, 64)
    sch.run([r], realtime=False)
    assert r.B is not None
    assert be.created == [(16, 4), (64, 2)] and be.destroyed == []


def test_admission_by_footprint_and_eviction():
    be = FakeBackend()
    # room for one group of 2 instances of N=32 (640) but not two groups of N=32 and N=64
    sch = serving.Scheduler(be, mem_budget=1000, max_batch=2, clock=FakeClock())
    reqs = [_req(0, 32), _req(1, 32), _req(2, 64), _req(3, 32)]
    sch.run(reqs, realtime=False)
    assert all(r.B is not None for r in reqs)
    assert sch.used <= 1000
    assert ("evict", (32, 100.0)) in sch.log
    sizes = [s for _, s in be.created]
    assert max(sizes) <= 2


def test_group_cap_per_shell_set():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=10 ** 6, max_batch=2, max_groups=1, clock=FakeClock())
    reqs = [_req(i, 16) for i in range(7)]
    sch.run(reqs, realtime=False)
    assert be.created == [(16, 2)]
    assert all(r.B is not None for r in reqs)


def test_requests_never_exceed_budget_wait_instead():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=700, max_batch=2, clock=FakeClock())
    reqs = [_req(i, 64, arrival=0.0) for i in range(5)]   # one instance of 64 costs 640
    sch.run(reqs, realtime=False)
    assert all(r.B is not None for r in reqs)
    assert be.created == [(64, 1)]
    assert all(k == 1 for _, k in be.launched)


def test_close_finishes_batches_in_flight_then_destroys_every_group():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=10 ** 6, max_batch=2, max_groups=2, clock=FakeClock())
    reqs = [_req(i, n, arrival=0.0) for i, n in enumerate((32, 32, 32, 64))]
    for r in reqs:
        sch.submit(r)
    sch.step()  # dispatch: batches in flight, none polled to completion yet
    assert sch.busy
    sch.close()
    assert not sch.busy and sch.groups == [] and sch.used == 0
    assert sorted(be.destroyed) == sorted(n for n, _ in be.created)
    # the batches in flight were retired with their results, not dropped
    assert sum(k for _, k in be.launched) >= 2
    assert sum(r.B is not None for r in reqs) == sum(k for _, k in be.launched)


def test_bad_requests_rejected_at_submission():
    kf = 2 * np.pi / 100.0
    spec = dict(kmin=kf, kmax=4 * kf, dk=2 * kf)
    cube = np.zeros((16,) * 3, np.float32)
    for kw in (dict(mesh=np.zeros((16, 16, 8), np.float32)),
               dict(mesh=np.zeros((16, 16), np.float32)),
               dict(mesh=cube, second=np.zeros((8,) * 3, np.float32)),
               dict(mesh=cube, precision="fp16")):
        with pytest.raises(ValueError):
            serving.Request(0, box=100.0, spec=spec, **kw)
    with pytest.raises(ValueError):  # an unknown triangle type fails when submitted
        serving.Scheduler(FakeBackend(), 1 << 30).submit(
            serving.Request(0, cube, 100.0, dict(spec, triangle_type="obtuse")))


def test_cross_requests_have_their_own_bin_set():
    be = FakeBackend()
    sch = serving.Scheduler(be, mem_budget=10 ** 6, max_batch=4, clock=FakeClock())
    a, c = _req(0, 32), _req(1, 32, cross=True)
    ja, jc = serving.Job(a), serving.Job(c)
    assert ja.bin_key != jc.bin_key and len(jc.tri) > len(ja.tri)
    sch.run([a, c], realtime=False)
    assert a.B is not None and c.B is not None


@pytest.mark.gpu
def test_mixed_stream_equals_each_request_alone(cuda):
    import torch

    from bskit_gb300 import synthetic
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(12):
        n = int(rng.choice([32, 48]))
        box = 100.0
        kf = 2 * np.pi / box
        t = ["all", "equilateral", "squeezed"][i % 3]
        spec = dict(kmin=kf, kmax=n / 4 * kf, dk=2 * kf, triangle_type=t)
        mesh = torch.from_numpy(synthetic.lognormal_mesh(n, box, seed=100 + i)).pin_memory()
        second = None
        if i % 4 == 3:
            second = torch.from_numpy(synthetic.noisy_copy(mesh.numpy(), seed=200 + i)).pin_memory()
        reqs.append(serving.Request(i, mesh, box, spec, second=second, arrival=0.0))
    mixed = serving.make_server(mem_budget=40 << 30, max_batch=3)
    mixed.run([serving.Request(r.rid, r.mesh, r.box, r.spec, r.second) for r in reqs],
              realtime=False)
    # batches of one N mix bin sets (all / equilateral / squeezed, auto and cross)
    assert any(e[0] == "batch" and e[3] > 1 for e in mixed.log)
    got = {r.rid: r for r in mixed.done}
    for r in reqs:
        alone = serving.make_server(mem_budget=40 << 30, max_batch=1, use_graphs=False)
        alone.run([r], realtime=False)
        m = got[r.rid]
        assert np.array_equal(m.N_tri, r.N_tri)
        scale = np.abs(r.B_unnorm).max()
        assert np.abs(m.B_unnorm - r.B_unnorm).max() <= 1e-12 * scale
