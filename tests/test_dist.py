"""The multi-rank path of bench.py on CPU with gloo, world size 2: each rank
renders its own frame (weak scaling, no data-path collective), the step time
is the slowest rank's, and the rate counts every rank's rays."""
import importlib.util
import os
import pathlib
import socket

import numpy as np
import torch.multiprocessing as mp

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import torch
    import torch.distributed as tdist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    bench = _bench()
    ng = importlib.import_module("nerf-tf2_gb300")
    o, d, _, _ = ng.synthetic.frame_rays(bench.rank_frame_seed(rank), H=16, W=16, focal=22.2)
    my_ms = 10.0 * (rank + 1)                       # rank 1 is the slower one
    slowest = bench.max_over_ranks(my_ms, world, torch.device("cpu"))
    rate = bench.whole_job_rate(world, o.shape[0], slowest)
    out[rank] = (float(o[0, 0]), float(d[5, 1]), slowest, rate)
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_ranks_gloo():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        r0, r1 = out[0], out[1]
    assert (r0[0], r0[1]) != (r1[0], r1[1])         # different cameras: independent shards
    assert r0[2] == r1[2] == 20.0                   # both report the slowest rank's time
    assert np.isclose(r0[3], 2 * 256 / 0.020) and r0[3] == r1[3]


def test_single_rank_helpers():
    bench = _bench()
    import torch
    assert bench.max_over_ranks(12.5, 1, torch.device("cpu")) == 12.5
    assert bench.whole_job_rate(1, 640000, 200.0) == 3.2e6
    assert bench.rank_frame_seed(3) == 3
