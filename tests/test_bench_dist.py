"""bench.py's multi-rank path (replicas, no data-path collective) on CPU:
two gloo ranks agree on the max step time and count every rank's columns."""
import multiprocessing as mp
import os
import socket


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    dist = bench.init_dist(2, "gloo")
    t = bench.max_over_ranks(1.5 if rank == 0 else 4.0, dist)
    bench.barrier(dist)
    ws, r, _ = bench.dist_env()
    q.put((rank, t, ws))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [4.0, 4.0]
    assert all(o[2] == 2 for o in out)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(2.5, None) == 2.5
