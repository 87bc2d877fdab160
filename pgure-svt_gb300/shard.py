"""Frame sharding across processes.

Output frames are independent windows (pguresvt.hpp:90-167 builds each from
its own slice of the sequence), so N processes each denoise a contiguous
range of output frames with pgsvt_params.frame_begin / frame_end and no data
exchange; the only collective is gathering the frames (or, in bench.py, the
maximum of the per-rank times).
"""


def shard_frames(nframes, world, rank):
    """Contiguous [begin, end) output frames of `rank` out of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(nframes, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def gather_frames(local, begin, end, group=None):
    """All-gather the frames [begin, end) of every rank into one array.

    `local` is the rank's full-shape result with only its frames filled
    (the library zeroes the others); torch.distributed sums them."""
    import numpy as np
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(local))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
