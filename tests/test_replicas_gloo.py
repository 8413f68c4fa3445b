"""Replica bookkeeping across two ranks with the gloo backend on CPU: the
maximum of per-rank times reaches every rank, instance shards cover each
instance exactly once, and the barrier returns.  This is the only
cross-rank logic of a run on several GPUs (no collective on the data path)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, size, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from nbots_gb300 import replicas as R
    r, s = R.init("gloo")
    assert (r, s) == (rank, size)
    R.barrier()
    mx = R.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank])
    items = list(R.shard(96, r, s))
    out.put((rank, mx, items))
    R.finalize()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, mx, _ in res:
        assert mx == [2.0, 10.0, 0.5]
    covered = sorted(i for _, _, items in res for i in items)
    assert covered == list(range(96))
    assert len(res[0][2]) == len(res[1][2]) == 48


def test_single_rank_is_identity():
    from nbots_gb300 import replicas as R
    assert R.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    assert list(R.shard(5, 0, 1)) == [0, 1, 2, 3, 4]
    assert [len(R.shard(10, r, 3)) for r in range(3)] == [3, 3, 4]
