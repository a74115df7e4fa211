"""Multi-GPU rendering as replicas: every rank holds the whole scene (the
accelerator and path state fit one GB300 many times over), renders a
disjoint range of sample indices, and the films are summed once at the end
-- the only exchange the path has (one all-reduce of W x H x 4 floats).
Ray casts need no exchange at all: each rank casts its own rays."""
import torch
import torch.distributed as dist


def sample_range(total_spp, rank, world):
    """Contiguous share [start, start + count) of total_spp sample indices."""
    base, extra = divmod(int(total_spp), int(world))
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def reduce_film(image, group=None):
    """Sums the (R, G, B, weight) films of all ranks in place."""
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(image, op=dist.ReduceOp.SUM, group=group)
    return image


def render_sharded(render, total_spp, rank, world, group=None):
    """render(sample_start, spp) -> film tensor of this rank's samples;
    returns the film of all total_spp samples (identical on every rank)."""
    # checked from the arguments every rank has, so all ranks raise together
    # and none is left waiting in the all-reduce
    if int(total_spp) < int(world):
        raise ValueError("more ranks (%d) than samples (%d)" % (world, total_spp))
    start, count = sample_range(total_spp, rank, world)
    return reduce_film(render(start, count), group)
