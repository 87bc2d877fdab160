"""World-size-2 gloo run on CPU of the frame-sharded path: each rank denoises
its frames with the oracle (frame_begin/frame_end) and the gathered sequence
equals the single-process result; the bench's max-over-ranks timing reduce
runs on the same group."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, X, kw, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import __graft_entry__ as entry
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pkg = entry.load_package()
    O = entry.load_oracle()
    b, e = pkg.shard.shard_frames(X.shape[2], world, rank)
    Y, est, _ = O.denoise(X, n_jobs=2, frame_begin=b, frame_end=e, **kw)
    Yall = pkg.shard.gather_frames(Y, b, e)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)  # bench.py's max over ranks
    if rank == 0:
        np.save(out, Yall)
        assert t.item() == world
    dist.destroy_process_group()


def test_shard_frames_cover_every_frame(pkg):
    for n, w in [(200, 8), (30, 4), (7, 3), (5, 5)]:
        ranges = [pkg.shard.shard_frames(n, w, r) for r in range(w)]
        assert ranges[0][0] == 0 and ranges[-1][1] == n
        assert all(ranges[i][1] == ranges[i + 1][0] for i in range(w - 1))


def test_two_rank_gloo_matches_single_process(pkg, oracle, tmp_path):
    noisy, _, _ = pkg.synth.workload("plain_64", seed=6, side=24, nt=17)
    kw = dict(traj_length=15, block_size=4, motion_window=5, median_size=-1, optimize_pgure=0,
              lambda_=0.2)
    Y1, _, _ = oracle.denoise(noisy, n_jobs=2, **kw)
    out = str(tmp_path / "y.npy")
    mp.start_processes(_worker, args=(2, _free_port(), noisy, kw, out), nprocs=2, join=True,
                       start_method="spawn")
    np.testing.assert_array_equal(np.load(out), Y1)
