"""Sharding of a render across ranks (one process per GPU).

Paths are independent, so ranks take disjoint, contiguous ranges of sample indices of the same
frame (e8g_render_params.sample_offset) and the frame is their sample-weighted mean: the only
exchange is one sum of the image at the end. Ranks render the same scene (replicated).
"""


def sample_range(spp_total, rank, world):
    """(first sample, sample count) of `rank` when spp_total samples are split over `world` ranks."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, rem = divmod(spp_total, world)
    count = base + (1 if rank < rem else 0)
    first = rank * base + min(rank, rem)
    return first, count


def combine(img, count, spp_total, group=None):
    """Combine per-rank means (img over `count` samples) into the frame mean, in place, with one
    all-reduce over `group` (torch.distributed)."""
    import torch.distributed as dist
    img.mul_(float(count) / float(spp_total))
    dist.all_reduce(img, op=dist.ReduceOp.SUM, group=group)
    return img
