"""The multi-GPU path is replicas only: independent scene sets per rank, no
collective on the data path.  bench.py's aggregation (units summed over
ranks, device time max over ranks) is checked here on CPU with two gloo
ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_env() == (ws, rank, rank)
        # rank r processed 1000 (r + 1) units in 10 (r + 1) ms
        rate, ms, units = bench.job_rate(1000 * (rank + 1), 10.0 * (rank + 1), ws, "cpu")
        out.put((rank, rate, ms, units))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregate_is_sum_over_max():
    ws = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(out.get(timeout=10) for _ in range(ws))
    for rank, rate, ms, units in got:
        assert units == 3000.0            # 1000 + 2000 units over both ranks
        assert ms == 20.0                 # the slower rank's time
        assert rate == pytest.approx(3000.0 / 0.020)


def test_single_rank_needs_no_process_group():
    import bench
    rate, ms, units = bench.job_rate(500, 4.0, 1, "cpu")
    assert (rate, ms, units) == (500 / 0.004, 4.0, 500)
