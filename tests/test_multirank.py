"""gloo tests of the run sharding used for more than one GPU: the ranks
compute disjoint blocks of runs with the CPU restatement, the blocks are
gathered (tensor all_gather) and the proximity is applied to the full label
matrix; the result must equal one process computing every run.  World size 2
with 6 runs, and world size 3 with 2 runs (one rank's block is empty)."""

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KW = dict(cycles=8, landmarks=10000, splitting=0, graph_neighbors=50, folds=10, knn_k=10)
SEED, RUNS = 1234, 6


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_matrix(orc):
    class Part:
        pass

    def fn(x, graph, first_run, runs, **kw):
        gi, gd = graph
        r = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=SEED, runs=runs, first_run=first_run,
                                         threads=2, materialize=0, **kw)
        p = Part()
        p.res, p.acc, p.v, p.run_hashes, p.run_counters, p.cycle_diag = (
            r.res, r.acc, r.v, r.hashes, r.run_counters, r.cycle_diag)
        return p
    return fn


def _worker(rank, world, port, out_path, runs):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from kodama_gb300 import datasets
    from kodama_gb300.distributed import kodama_matrix_sharded
    from oracle import oracle as orc
    x = datasets.spirals()[0].astype(np.float32)
    graph = orc.exact_knn(x, 50, threads=2)
    r = kodama_matrix_sharded(x, runs=runs, graph=graph, matrix_fn=_oracle_matrix(orc),
                              dissimilarity_fn=lambda i, d, res: orc.dissimilarity(i, d, res), dist=dist, **KW)
    if rank == 0:
        np.savez(out_path, res=r.res, acc=r.acc, v=r.v, hashes=r.run_hashes, counters=r.run_counters,
                 diag=r.cycle_diag, kidx=r.knn_idx, kdist=r.knn_dist)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,runs", [(2, RUNS), (3, 2)])
def test_sharded_runs_equal_single_process(orc, tmp_path, world, runs):
    out = str(tmp_path / "sharded.npz")
    mp.start_processes(_worker, args=(world, _free_port(), out, runs), nprocs=world, join=True,
                       start_method="spawn")
    got = np.load(out)
    from kodama_gb300 import datasets
    x = datasets.spirals()[0].astype(np.float32)
    gi, gd = orc.exact_knn(x, 50, threads=2)
    ref = orc.kodama_matrix_graph_data(x, gi, gd, 0, seed=SEED, runs=runs, threads=2, materialize=1, **KW)
    assert np.array_equal(got["res"], ref.res)
    assert np.array_equal(got["acc"], ref.acc)
    assert np.array_equal(got["v"], ref.v)
    assert np.array_equal(got["hashes"], ref.hashes)
    assert np.array_equal(got["counters"], ref.run_counters)
    assert np.array_equal(got["diag"], ref.cycle_diag)
    assert np.array_equal(got["kidx"], ref.knn_idx)
    assert np.array_equal(got["kdist"], ref.knn_dist)


def test_shard_blocks_cover_runs():
    from kodama_gb300.distributed import shard
    for runs in (1, 5, 100, 101):
        for world in (1, 2, 3, 8):
            ids = []
            for rank in range(world):
                first, count = shard(runs, world, rank)
                ids += list(range(first, first + count))
            assert ids == list(range(1, runs + 1))
