"""Point-range sharding of one bispectrum across GPUs.

bskit splits every sum over the grid into MPI x-slabs and combines the local
sums with gather + bcast (bskit/main.py:1875-1879).  Here each rank paints the
full mesh (replicated FFTs), contracts only its contiguous range of
contraction-grid points (``Plan.measure_b_range``) and the FP64 partial vectors
are summed with one all-reduce -- the only exchange of the path (T doubles).
"""
import torch


def point_range(n_points, rank, world, align=128):
    """[k0, k1) of rank's share of n_points; interior bounds are multiples of ``align``
    (the tensor-core path consumes 128-point stages)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")

    def bound(r):
        if r >= world:
            return n_points
        return (n_points * r // world) // align * align

    return bound(rank), bound(rank + 1)


def allreduce_partials(partial, group=None):
    """Sum FP64 partial vectors over the process group (in place); returns the tensor."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(partial, op=dist.ReduceOp.SUM, group=group)
    return partial


def sharded_measure_b(plan, tset, slots=(0, 0, 0), precision="bf16x3", group=None,
                      partial_fn=None):
    """Unnormalised B of ``tset`` with the grid points split over the group's ranks.

    ``partial_fn(k0, k1)`` computes one rank's partial vector; by default it is
    ``plan.measure_b_range`` on the plan's device.
    """
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    n_points = plan.ngrid ** 3
    k0, k1 = point_range(n_points, rank, world)
    if partial_fn is None:
        part = plan.measure_b_range(tset, k0, k1, slots=slots, precision=precision)
    else:
        part = partial_fn(k0, k1)
    part = torch.as_tensor(part, dtype=torch.float64)
    return allreduce_partials(part, group)
