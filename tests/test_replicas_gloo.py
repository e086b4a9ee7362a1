"""The replica harness of bench.py on the CPU: two ranks over gloo (the path
`bench.py --gpus N` takes under torchrun). Each rank is an independent replica;
the only collectives are the barrier and the maximum of the per-rank timings."""
import importlib.util
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as tmp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    b = _bench()
    r, w, local, pg = b.dist_setup(world)
    assert (r, w, local) == (rank, world, rank) and pg is not None
    b.barrier(pg)
    # the slowest rank's time is the job's time
    t = b.max_over_ranks(pg, 1.5 + rank)
    out.put((rank, t))
    pg.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]


def test_single_process_needs_no_process_group():
    b = _bench()
    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK") if k in os.environ}
    try:
        r, w, local, pg = b.dist_setup(1)
        assert (r, w, local, pg) == (0, 1, 0, None)
        assert b.max_over_ranks(pg, 3.25) == 3.25
    finally:
        os.environ.update(env)
