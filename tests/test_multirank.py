"""N > 1: assets shard across ranks with no data-path collective (bench.py
under torchrun).  Two gloo ranks on CPU check that the shards partition the
asset list, that each rank's oracle step of its shard equals the same assets
stepped in one process, and that the timing reduction takes the max."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    for p in (root, os.path.join(root, "realtime-vulkan-hair_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      RVH_DIST_BACKEND="gloo")
    import bench
    from oracle import oracle_ctypes as O
    from rvh import configs
    r, w = bench.dist_init()
    specs = configs.batched(n_assets=9, scale=0.01, seed=41)
    mine = bench.shard(specs, r, w)
    states = []
    for s in mine:
        st = s.records.astype(np.float64)
        O.run(st, s.n_points, s.rest, s.params, [s.frame(k) for k in range(2)], s.colliders, 2)
        states.append(st)
    idx = [i for i in range(len(specs)) if i % w == r]
    np.savez(os.path.join(out_dir, "rank%d.npz" % r), idx=np.array(idx),
             **{"s%d" % i: st for i, st in zip(idx, states)})
    t = bench.max_over_ranks(float(r + 1), w)
    bench.barrier(w)
    with open(os.path.join(out_dir, "max%d.txt" % r), "w") as f:
        f.write(repr(t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_assets_without_collectives(tmp_path, librvh):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    from oracle import oracle_ctypes as O
    from rvh import configs
    specs = configs.batched(n_assets=9, scale=0.01, seed=41)
    got = {}
    for r in range(2):
        d = np.load(tmp_path / ("rank%d.npz" % r))
        for i in d["idx"]:
            assert int(i) not in got
            got[int(i)] = d["s%d" % i]
        assert float(open(tmp_path / ("max%d.txt" % r)).read()) == 2.0
    assert sorted(got) == list(range(9))
    for i, s in enumerate(specs):
        st = s.records.astype(np.float64)
        O.run(st, s.n_points, s.rest, s.params, [s.frame(k) for k in range(2)], s.colliders, 2)
        assert np.array_equal(st, got[i])
