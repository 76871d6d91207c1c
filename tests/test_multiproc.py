"""The N>1 path of bench.py on CPU: two ranks over gloo (127.0.0.1), one
independent instance per rank (seed = rank, no data-path collective), the
step time reduced as the max over ranks, barriers around the timed region."""
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
    from pqdts_gb300 import synth

    w, r, _ = bench.dist_env()
    dist = bench.dist_init(w, use_cuda=False)
    bench.dist_barrier(dist)
    step = 0.5 + rank  # this rank's local step time
    mx = bench.dist_max(dist, step, "cpu")
    inst = synth.make_instance(M=30, N=5, D=60, xmax=20.0, eta=0.8, shots=10**4, gamma=1e-3, eps=1e-6, seed=r)
    bench.dist_barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, mx, float(inst.P.sum()), inst.P.tobytes()))


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, m0, s0, b0), (r1, w1, m1, s1, b1) = out
    assert (r0, r1) == (0, 1) and w0 == w1 == 2
    assert m0 == m1 == 1.5  # max over ranks
    assert b0 != b1  # each rank solves its own instance
