"""The multi-GPU path of bench.py: independent replicas (or shares of the
scenes) per rank with no exchange on the data path; the job's time is the
slowest rank's and its work the sum over ranks.  Run here as two gloo ranks
on the CPU."""
import importlib.util
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        ms = [3.0, 7.5][rank]
        updates = [1000, 2500][rank]
        share = b.rank_share(list(range(10)), rank, world)
        out.put((rank, b.rank_total(ms, "max", dist, device="cpu"), b.rank_total(updates, "sum", dist, device="cpu"),
                 share, b.rank_total(len(share), "sum", dist, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_like_replicas():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, ms, upd, share, nshare in res:
        assert ms == 7.5 and upd == 3500.0  # slowest rank, total work
        assert nshare == 10.0               # every scene on exactly one rank
    assert sorted(res[0][3] + res[1][3]) == list(range(10))
    assert not set(res[0][3]) & set(res[1][3])


def test_single_process_passes_values_through():
    b = _bench()
    assert b.rank_total(4.0, "max") == 4.0
    assert b.rank_share([1, 2, 3], 0, 1) == [1, 2, 3]
