"""The replica path of bench.py on CPU: two gloo ranks (127.0.0.1), each
running its own replica of a small workload on the oracle, then the bench's
barrier and max-over-ranks timing.  Replicas exchange nothing on the data
path, so each rank's result must equal a single-process run."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _replica(seed):
    import oracle
    from conftest import permalloy, seeded_m
    from nmag import mesh
    msh = mesh.box_mesh(3, 3, 2, 2.0)
    om = oracle.OracleMesh(msh.points, msh.simplices, nthreads=1)
    sim = oracle.OracleSim(om, permalloy(0.5).coefficients("nmag"), nthreads=1)   # one thread: bit-reproducible
    return sim.rk4(seeded_m(len(msh.points), seed=seed, noise=0.3), 0.05, 5)


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "nmag-src_gb300"), os.path.join(root, "oracle"), root, os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    m = _replica(100 + rank)
    bench.barrier(world)
    t = bench.max_over_ranks(0.5 + rank, world)
    np.save(os.path.join(out, "rank%d.npy" % rank), np.concatenate([[t], m.reshape(-1)]))
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    for rank in range(world):
        d = np.load(os.path.join(str(tmp_path), "rank%d.npy" % rank))
        assert d[0] == 1.5                       # max over ranks of 0.5 + rank
        assert np.array_equal(d[1:], _replica(100 + rank).reshape(-1))   # independent replicas
