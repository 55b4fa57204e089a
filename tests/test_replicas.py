"""The multi-process (replicas) layer on CPU: two gloo ranks deal the q-points
round-robin, rank 0 writes every q once in global order, and the timing
reduction takes the maximum over the ranks.  The GPU solve is replaced by a
host function; the layer itself is the one the driver and the benchmark use."""
import os
import socket

import numpy as np
import pytest

from parphom_gb300 import replicas


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, nq, batch, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    group = replicas.init_group(world, rank)
    q = np.arange(nq * 3, dtype=np.float64).reshape(nq, 3)
    calls = []

    def solve(qb):
        calls.append(len(qb))
        assert len(qb) <= batch
        return [{"s": float(r.sum()), "rank": rank} for r in qb]

    written = []

    def write(t, r):
        written.append((t, r["s"], r["rank"]))

    n = replicas.run_sharded(q, batch, solve, write if rank == 0 else None, world, rank, group)
    tmax = replicas.max_over_ranks(float(rank + 1), world, group)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.array([n, tmax, len(calls)], dtype=np.float64))
    if rank == 0:
        np.save(os.path.join(out_dir, "written.npy"), np.array(written, dtype=np.float64).reshape(-1, 3))
    dist.destroy_process_group()


@pytest.mark.parametrize("nq,batch", [(7, 2), (5, 8), (1, 1)])
def test_two_ranks_gloo(tmp_path, nq, batch):
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(2, _free_port(), nq, batch, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    written = np.load(tmp_path / "written.npy")
    q = np.arange(nq * 3, dtype=np.float64).reshape(nq, 3)
    assert written[:, 0].astype(int).tolist() == list(range(nq))      # every q once, in order
    np.testing.assert_array_equal(written[:, 1], q.sum(axis=1))       # the owner's result
    assert written[:, 2].astype(int).tolist() == [t % 2 for t in range(nq)]  # q[r::2] on rank r
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    assert r0[0] + r1[0] == nq
    assert r0[1] == r1[1] == 2.0                                      # max over ranks


def _worker_dies(rank, world, port, out_dir):
    import time

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    group = replicas.init_group(world, rank, timeout_s=20.0)
    q = np.zeros((6, 3))

    def solve(qb):
        if rank == 1:
            os._exit(3)   # a rank that dies between two gatherings
        return [0.0] * len(qb)

    t0 = time.time()
    try:
        replicas.run_sharded(q, 1, solve, (lambda t, r: None) if rank == 0 else None, world, rank, group)
        status = "finished"
    except Exception as e:   # the surviving rank learns of it from its collective
        status = type(e).__name__
    with open(os.path.join(out_dir, f"status{rank}.txt"), "w") as f:
        f.write(f"{status} {time.time() - t0:.1f}")


def test_dead_rank_fails_the_gathering(tmp_path):
    import torch.multiprocessing as mp

    ctx = mp.start_processes(_worker_dies, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=False,
                             start_method="spawn")
    for p in ctx.processes:
        p.join(120)
        if p.is_alive():   # our own child, by its handle
            p.kill()
    status, dt = (tmp_path / "status0.txt").read_text().split()
    assert status != "finished"
    assert float(dt) < 60.0
    assert not (tmp_path / "status1.txt").exists()


def test_one_rank_writes_in_order():
    q = np.random.default_rng(0).standard_normal((11, 3))
    out = []
    n = replicas.run_sharded(q, 4, lambda qb: [float(r[0]) for r in qb], lambda t, r: out.append((t, r)))
    assert n == 11
    assert [t for t, _ in out] == list(range(11))
    assert [r for _, r in out] == [float(v) for v in q[:, 0]]


def test_shard_and_rounds():
    assert replicas.shard(7, 1, 3).tolist() == [1, 4]
    assert replicas.rounds(7, 2, 2) == 2 and replicas.rounds(0, 2, 2) == 0 and replicas.rounds(5, 2, 8) == 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)
    with pytest.raises(ValueError):
        replicas.rounds(4, 1, 0)
