"""The replicas' timing reduction of bench.py over two gloo ranks on the CPU: the
whole-job figures are the slowest rank's time and the sum of all ranks' proposals
(the path under torchrun with one rank per GPU; no exchange happens in the timed
work itself)."""
import importlib.util
import os
import socket

import torch.multiprocessing as mp

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(_ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_ms, nprop = _bench().combine_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
        out.put((rank, t_ms, nprop))
    finally:
        dist.destroy_process_group()


def test_slowest_time_and_all_proposals_over_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 15.0, 3000.0), (1, 15.0, 3000.0)]
