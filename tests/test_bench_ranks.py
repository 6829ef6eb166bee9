"""Replica bookkeeping of ``bench.py --gpus N`` on CPU: two ``gloo`` ranks take
disjoint seeded batches and agree on the slowest rank's time (the whole-job
clock), with no other collective on the data path."""

import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        r, w, _ = bench.dist_env()
        seeds = bench.rank_seeds(r, 4)
        slowest = bench.max_over_ranks(10.0 * (r + 1))
        q.put((r, w, seeds, slowest))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:2] for r in res] == [(0, 2), (1, 2)]
    assert res[0][2] == [0, 1, 2, 3] and res[1][2] == [4, 5, 6, 7]
    assert all(r[3] == 20.0 for r in res)


def test_max_over_ranks_without_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.rank_seeds(0, 3) == [0, 1, 2]


def test_launch_traffic_scales_with_batch():
    sys.path.insert(0, ROOT)
    import json
    import bench
    recs = json.load(open(os.path.join(ROOT, 'profiles', 'traffic.json')))
    kernels = [k for k, v in recs.items() if isinstance(v, dict)]
    assert 'batch_sle_kernel' in kernels
    for k in kernels:
        rec = recs[k]
        full, note = bench.launch_traffic(rec['solves'], k)
        assert full == rec['bytes'] and 'scaled' not in note and k in note
        part, note = bench.launch_traffic(rec['solves'] // 5, k)
        assert abs(part - full * (rec['solves'] // 5) / rec['solves']) < 1.0 and 'scaled' in note
    assert bench.launch_traffic(10, 'no_such_kernel')[0] is None
