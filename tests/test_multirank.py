"""The N > 1 host logic of bench.py, as world_size-2 gloo ranks on the CPU:
each rank is a replica with its own inputs, and the job's step time is the
slowest rank's (the timing rule the multi-GPU bench applies)."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    step_ms = 10.0 + 7.5 * rank
    got = bench.max_over_ranks(step_ms, dist, "cpu")
    u0, p = bench.CONFIGS[2]["inputs"](64, bench.replica_seed(rank))
    out[rank] = (got, float(p[1].sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step_and_distinct_replicas():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 17.5
    assert res[0][1] != res[1][1]  # rank-seeded replicas


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
    assert np.array_equal(bench.CONFIGS[2]["inputs"](8, bench.replica_seed(0))[0],
                          bench.CONFIGS[2]["inputs"](8, 2024)[0])
