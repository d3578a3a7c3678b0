"""bench.py under torchrun runs one independent replica per rank (the path has
no cross-colony exchange): ranks meet only at the barrier and the max-over-ranks
of the timed region.  Exercised here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, pg = bench.dist_setup()
    assert pg is not None and pg.get_backend() == "gloo"
    ms = 100.0 + 7.0 * r                 # this rank's timed region
    bench.dist_barrier(pg)
    ms_max = bench.dist_max(pg, ms)
    q.put((r, w, ms_max, bench.aggregate_value(1000, w, 10, ms_max)))
    pg.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_share_only_the_max_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 107.0 for o in out)
    # whole-job throughput: both replicas' cells over the slowest rank's time
    assert out[0][3] == pytest.approx(1000 * 2 * 10 / 0.107)
