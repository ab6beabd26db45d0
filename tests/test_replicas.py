"""The N-GPU path of bench.py is N independent replicas (one model per GPU,
no collective on the data path): the host logic -- rank environment, the
max-over-ranks time and the whole-job rate -- on two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    r, w, loc = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    ms = 10.0 + 5.0 * rank  # each replica's device time for its K steps
    dist.barrier()
    worst = bench.reduce_max_sum([ms], w)[0]
    out.put((r, w, loc, worst))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == 15.0 for r in res)  # both ranks see the max over ranks
    # whole-job rate: every replica updates E elements per step
    E, steps = 1000, 20
    assert E * steps * 2 / (res[0][3] / 1000.0) == pytest.approx(2.0 * E * steps / 0.015)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.reduce_max_sum([3.5], 1) == [3.5]
