"""Multi-GPU runs are independent replicas (cars never interact): the host
bookkeeping of bench.py's N-rank path, exercised with two gloo ranks on CPU.
Each rank gets its own sim seed; the only collectives are a barrier and the
maximum of the per-rank times."""
import multiprocessing
import os
import socket

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import oracle as O
    import warporacer3d_gb300 as W
    from warporacer3d_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = replicas.topology()
    seconds = 1.0 + 0.5 * r  # the slowest rank sets the job's time
    slowest = replicas.max_over_ranks(seconds, dist)
    sim = O.Sim(W.track("flat"), 32, replicas.replica_seed(42, r), beams=8)
    sim.reset()
    dist.barrier()
    queue.put((r, w, local, slowest, replicas.whole_job_rate(1000, w, slowest), sim.state.copy()))
    dist.destroy_process_group()


def test_two_rank_replicas_on_gloo():
    ctx = multiprocessing.get_context("spawn")
    queue, port = ctx.Queue(), _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, m0, rate0, s0), (r1, w1, l1, m1, rate1, s1) = results
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert m0 == m1 == 1.5 and rate0 == rate1 == 2000 / 1.5
    assert not np.array_equal(s0, s1), "replicas spawn different cars"


def test_single_process_defaults():
    from warporacer3d_gb300 import replicas
    saved = {k: os.environ.pop(k, None) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    try:
        assert replicas.topology() == (0, 1, 0)
        assert replicas.max_over_ranks(3.25) == 3.25 and replicas.whole_job_rate(10, 1, 2.0) == 5.0
    finally:
        os.environ.update({k: v for k, v in saved.items() if v is not None})
