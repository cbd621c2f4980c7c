"""The multi-rank host logic on CPU: two gloo ranks, as torchrun would start."""
import os

import numpy as np
import torch.multiprocessing as mp


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from rustspice_gb300 import ranks
    from rustspice_gb300 import workloads as wl
    B = wl.inverter_batch(16, 3, seed=ranks.shard_seed(rank))
    lengths = [int(c.node_count) for c in B.circuits]
    step_ms = 10.0 + 5.0 * rank
    q.put((rank, lengths, ranks.max_over_ranks(step_ms), B.ninst))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict()
    for _ in range(2):
        r, lengths, mx, ninst = q.get(timeout=120)
        out[r] = (lengths, mx, ninst)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1] == out[1][1] == 15.0           # max over ranks
    assert out[0][2] == out[1][2] == 16 * 3         # equal per-rank work (weak scaling)
    assert out[0][0] != out[1][0]                    # distinct instances per rank


def test_rank0_keeps_single_gpu_workload():
    from rustspice_gb300 import ranks
    assert ranks.shard_seed(0) == 3
    assert len({ranks.shard_seed(r) for r in range(8)}) == 8
