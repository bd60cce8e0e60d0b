"""Several ranks (gloo on the CPU, world size 2): the host side of the
multi-GPU arrangement.  Each rank assembles its own shard of independent
meshes (here with the oracle); nothing on the data path is exchanged, and the
job's time is the slowest rank's.  The shards' results equal a one-process
run of the same meshes."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from cm_gb300 import distributed as D
from cm_gb300 import mesh as M


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard_residual_norms(rank):
    import oracle
    norms = []
    meshes, stretches = D.rank_batch_meshes(3, rank, edge_range=(1, 3))
    for i, (m, s) in enumerate(zip(meshes, stretches)):
        x = M.deformed_state(m, stretch=s, shear=0.0, noise=0.02, pressure=-1.0, seed=i)
        r = np.zeros(x.size)
        oracle.EquationsSet(m, nthreads=1).residual_evaluate(x, r)
        norms.append(float(np.linalg.norm(r)))
    return norms, sum(m.ne for m in meshes)


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    t = D.max_over_ranks(0.25 * (rank + 1), dist)
    norms, ne = _shard_residual_norms(rank)
    total = D.sum_over_ranks(ne, dist)
    np.save(os.path.join(outdir, "rank%d.npy" % rank), np.array([t, total, ne] + norms))
    dist.destroy_process_group()


def test_two_rank_shards_without_data_exchange(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [np.load(os.path.join(str(tmp_path), "rank%d.npy" % r)) for r in range(world)]
    # the job time is the slowest rank's, known to every rank
    assert all(r[0] == 0.5 for r in res)
    # the total work is the sum of the shards
    assert all(r[1] == res[0][2] + res[1][2] for r in res)
    # the shards are different problems, and each equals a one-process run
    assert not np.array_equal(res[0][3:], res[1][3:])
    for rank in range(world):
        norms, ne = _shard_residual_norms(rank)
        assert ne == res[rank][2]
        assert np.array_equal(np.array(norms), res[rank][3:])


def test_single_process_reductions_are_identity():
    assert D.max_over_ranks(3.5) == 3.5
    assert D.sum_over_ranks(7) == 7
    a, _ = D.rank_batch_meshes(2, 0, edge_range=(1, 2))
    b, _ = M.batch_meshes(2, seed=0, edge_range=(1, 2))
    assert [m.ne for m in a] == [m.ne for m in b]


@pytest.mark.skipif(not torch.distributed.is_available(), reason="torch.distributed missing")
def test_rank0_shard_is_the_single_gpu_batch():
    a, sa = D.rank_batch_meshes(4, 0)
    b, sb = M.batch_meshes(4, seed=0)
    assert sa == sb and all(np.array_equal(x.X, y.X) for x, y in zip(a, b))
