"""View sharding for batched and differentiable passes across ranks (one GPU per rank).

Views are independent, so each rank renders a contiguous range of them with no exchange on the
data path.  The only collective is the sum of per-vertex gradients of a differentiable batch
(every rank's views see the same mesh); images and losses stay on their rank or are gathered on
the host.  A single frame does not shard: N ranks render N independent replicas.
"""


def view_range(num_views, rank, world):
    """[begin, end) of the views rank `rank` of `world` renders: contiguous, sizes differ by at
    most one, earlier ranks take the larger share."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    base, extra = divmod(int(num_views), int(world))
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def allreduce_gradients(tensors, group=None):
    """Sums gradients (e.g. positions, colours, UVs of the shared mesh) over all ranks in place."""
    import torch.distributed as dist
    for t in tensors:
        if t is not None:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors
