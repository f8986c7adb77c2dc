"""The multi-process path of a run on N GPUs, on CPU: two gloo ranks.

Each rank runs an independent halo (replicas: the step has no exchange between
halos), the timing is the maximum over ranks, and the job's rate counts every rank's
particle-steps over that time.  The oracle steps each rank's own halo, so the test
needs no GPU.
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from nsphere_gb300 import ics
    from nsphere_gb300.replicas import job_rate, max_over_ranks, rank_env, replica_seed
    from oracle.oracle import Oracle

    r_, l_, w_ = rank_env()
    assert (r_, l_, w_) == (rank, rank, world)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # the rank's own halo, stepped by the oracle
    n = 2000
    state = ics.plummer(n, seed=replica_seed(1, rank))
    orc = Oracle()
    p = orc.params(dt=1e-3)
    cur = orc.sort(*state)
    for _ in range(3):
        cur = orc.step_kdk(p, *cur)
    ms = 10.0 + 5.0 * rank                      # a rank-dependent "elapsed time"
    ms_max = max_over_ranks(ms, world)
    rate = job_rate(n * 3, world, ms_max)
    np.savez(os.path.join(out_dir, "rank%d.npz" % rank), r=cur[0], ids=cur[3], ms_max=ms_max, rate=rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_run_independent_replicas(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    from oracle import build_oracle

    build_oracle.build_oracle()
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(120)
        assert pr.exitcode == 0
    a, b = (np.load(tmp_path / ("rank%d.npz" % r)) for r in range(2))
    # the timing is the slowest rank's, on every rank; the rate counts both ranks
    assert float(a["ms_max"]) == float(b["ms_max"]) == 15.0
    assert float(a["rate"]) == pytest.approx(2 * 2000 * 3 / 0.015)
    # the replicas are different halos, each a valid sorted state
    assert not np.array_equal(a["r"], b["r"])
    for s in (a, b):
        assert np.all(np.diff(s["r"]) >= 0) and np.array_equal(np.sort(s["ids"]), np.arange(2000))
