"""bench.py on N > 1 ranks: independent replicas (the path has no exchange step), and the job's
time is the slowest rank's, so whole-job throughput = the units all ranks processed / that time.
Two gloo ranks on the CPU run the reduction bench.py uses."""
import os
import socket


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    dist.barrier()
    got = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    single = bench.max_over_ranks(3.0, 1, "cpu")  # one rank: no collective
    q.put((rank, got, single))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_time_on_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=150) for _ in procs]
    for p in procs:
        p.join(timeout=30)
    assert all(p.exitcode == 0 for p in procs)
    assert sorted(results) == [(0, 15.0, 3.0), (1, 15.0, 3.0)]
