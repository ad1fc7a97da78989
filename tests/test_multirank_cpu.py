"""The multi-GPU form on CPU: two gloo ranks (127.0.0.1).

bench.py runs one replica of the workload per GPU ("replicas only": the path
needs no exchange between GPUs) and reports all ranks' pairs over the slowest
rank's time.  Checked here without a GPU: the max-over-ranks reduction the
bench uses, and that replicas of the same seeded network give identical
forces on every rank (the oracle stands in for the per-rank GPU call).
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    import __graft_entry__ as graft
    pkg = graft.load_package()
    oracle, _ = graft.load_oracle()
    import ddd_gb300.synth as synth
    t = bench.max_over_ranks(10.0 + rank, dist, "cpu")
    p, b, _ = synth.make("cpu512", seed=3, num_loops=16)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    k5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / 0.72, 0.28 / (4 * np.pi) / 0.72])
    F = oracle.segseg_ser(k5, net)
    mine = torch.from_numpy(np.ascontiguousarray(F).ravel())
    got = [torch.zeros_like(mine) for _ in range(ws)]
    dist.all_gather(got, mine)
    same = all(torch.equal(g, got[0]) for g in got)
    dist.barrier()
    dist.destroy_process_group()
    np.save(os.path.join(out_dir, "rank%d.npy" % rank), np.array([t, float(same)]))


def test_two_rank_replicas(tmp_path, oracle):
    port = _free_port()
    ctx = torch.multiprocessing.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        t, same = np.load(tmp_path / ("rank%d.npy" % r))
        assert t == 11.0  # every rank sees the slowest rank's time
        assert same == 1.0  # replicas agree bit for bit
