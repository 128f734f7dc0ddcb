"""The multi-GPU path is replicas only: each rank decodes its own streams
and the job reports the slowest rank.  Two gloo ranks on the CPU exercise the
barrier and max-over-ranks plumbing bench.py uses, each rank decoding its
replica with the CPU oracle."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root), str(root / "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    import ebiv_oracle
    from govid_gb300 import ebiv

    r, w, dist = bench.dist_init(2)
    spec = ebiv.SceneSpec(width=96, height=64, seed=3 + r, sprites=2)
    cont = ebiv.encode_scene(spec, 4, qp=22, gop=4, tiles=(1, 1), fast=True)
    pk = [p.data for p in ebiv.Reader(cont).packets()]
    bench.barrier(dist)
    ok = sum(1 for s, _ in ebiv_oracle.decode_all(pk) if s == 0)
    elapsed = bench.max_over_ranks(dist, float(rank + 1))
    q.put((r, w, ok, elapsed))
    dist.destroy_process_group()


def test_two_rank_replicas():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 4 for o in out)
    assert all(o[3] == 2.0 for o in out)  # max over ranks
