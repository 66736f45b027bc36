"""Host logic of the N-replica run on CPU: two gloo processes."""
import os
import socket

import pytest

from decomp_mpi_gb300.replicas import Replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    r = Replicas()
    r.init("gloo")
    r.barrier()
    # rank-dependent "durations": the slowest replica sets the job's time
    mx = r.max([10.0 + rank, 5.0 - rank])
    sm = r.sum([1.0, float(rank)])
    r.barrier()
    r.close()
    out.put((rank, r.leader, mx, sm))


def test_single_replica_without_launcher():
    r = Replicas(env={})
    assert (r.world, r.rank, r.local_rank, r.leader) == (1, 0, 0, True)
    r.init("gloo")  # no process group for one replica
    r.barrier()
    assert r.max([3.0, 4.0]) == [3.0, 4.0]
    assert r.sum([3.0]) == [3.0]
    r.close()


def test_gpu_index_follows_visible_devices():
    r = Replicas(env={"LOCAL_RANK": "1", "WORLD_SIZE": "2", "RANK": "1"})
    assert r.gpu_index(env={"CUDA_VISIBLE_DEVICES": "4,6"}) == "6"
    assert r.gpu_index(env={}) == "1"


@pytest.mark.timeout(120)
def test_two_replicas_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [x[1] for x in res] == [True, False]
    for _, _, mx, sm in res:
        assert mx == [11.0, 5.0]
        assert sm == [2.0, 1.0]
