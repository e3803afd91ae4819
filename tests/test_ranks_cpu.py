"""bench.py's whole-job figures with several ranks (gloo, two CPU processes):
the job's time is the slowest rank's (ranks_max) and its units are every
rank's own batch added up (ranks_sum); with one process both pass the value
through.  The GPU run takes the same calls over NCCL."""
import importlib.util
import multiprocessing as mp
import os
import socket

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _load_bench()
        # rank r ran its steps in 10 + r ms and processed 100 + r contacts
        out.put((rank, bench.ranks_max(10.0 + rank, "cpu"), bench.ranks_sum(100 + rank, "cpu")))
    finally:
        dist.destroy_process_group()


def test_two_ranks_slowest_time_and_summed_units():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 11.0, 201), (1, 11.0, 201)]


def test_one_process_passes_through():
    bench = _load_bench()
    assert bench.ranks_max(3.5, "cpu") == 3.5
    assert bench.ranks_sum(7, "cpu") == 7
