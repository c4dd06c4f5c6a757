"""The N-GPU harness of bench.py (independent replicas: one solve per rank, a
host barrier, the maximum time over ranks) on two CPU processes over gloo."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.init_dist()
    bench.barrier(w)
    v = bench.allmax(w, 10.0 + r)  # each rank's "time"; the line reports the slowest
    bench.barrier(w)
    q.put((r, w, v))
    bench._pg.destroy_process_group()


def test_two_rank_barrier_and_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 11.0), (1, 2, 11.0)]


def test_reference_arm_does_no_work_off_rank_zero(capsys):
    sys.path.insert(0, ROOT)
    import bench
    # rank 1 of the reference arm returns before reading its arguments and prints nothing
    bench.run_reference(None, 1)
    assert capsys.readouterr().out == ""
