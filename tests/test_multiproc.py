"""The N>1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).  Every
rank solves the same instance (replicas, no data-path collective): each
rank builds its workload with bench.rank_workload, solves it (here with the
oracle, on the CPU), and bench.replica_check gathers the per-rank work
counts and objective and finds them identical; the step time is reduced as
the max over ranks, with barriers around the timed region."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    from oracle.oracle import Oracle, set_threads

    w, r, _ = bench.dist_env()
    dist = bench.dist_init(w, use_cuda=False)
    bench.dist_barrier(dist)
    inst = bench.rank_workload(config=1)  # the small configuration: the same instance on every rank
    set_threads(1)
    _, st = Oracle.from_instance(inst).solve(mode=2, maxiter=200, eps=inst.eps)
    rep = bench.replica_check(dist, st, "cpu")
    step = 0.5 + rank  # this rank's local step time
    mx = bench.dist_max(dist, step, "cpu")
    bench.dist_barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, mx, inst.P.tobytes(), rep))


def test_two_ranks_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, m0, b0, rep0), (r1, w1, m1, b1, rep1) = out
    assert (r0, r1) == (0, 1) and w0 == w1 == 2
    assert m0 == m1 == 1.5  # max over ranks
    assert b0 == b1  # the same instance on both ranks
    assert rep0 == rep1 and rep0["identical"] and len(rep0["per_rank"]) == 2
    assert rep0["per_rank"][0]["cg"] > 0 and rep0["per_rank"][0]["outer"] > 0


def test_replica_summary_flags_different_work():
    """A rank whose counts or objective differ makes `identical` false."""
    sys.path.insert(0, ROOT)
    import bench

    same = bench.replica_summary([(3, 10, 4, 0.5), (3, 10, 4, 0.5)])
    assert same["identical"] and same["per_rank"][1] == {"outer": 3, "cg": 10, "ls_evals": 4, "L": 0.5}
    assert not bench.replica_summary([(3, 10, 4, 0.5), (3, 11, 4, 0.5)])["identical"]
    assert not bench.replica_summary([(3, 10, 4, 0.5), (3, 10, 4, 0.5000000001)])["identical"]
    one = bench.replica_check(None, {"outer": 3, "cg": 10, "ls_evals": 4, "L": 0.5}, "cpu")
    assert one["identical"] and len(one["per_rank"]) == 1
