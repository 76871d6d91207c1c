#!/usr/bin/env python3
"""Benchmark: time-to-solution of pqdts's two-metric projected truncated
Newton solve (mode 2, two stages, start Pi = 1/N) on one GB300.

Workload: the M=2000, N=200, D=4000 configuration (x_d linear 0.01..1800,
eta = 0.9, 1e7 shots, gamma = 1e-5), seeded synthetic data (pqdts_gb300.synth,
bit-identical on every platform), solved from Pi = 1/N.

One "step" = one full solve.
  FP64 (the drop-in, `value`): the reference's stopping rule conv < 1e-6.
    The trajectory is bitwise the CPU restatement's (checked in the same run:
    `config.parity`), so the CPU baseline does exactly the same iterations
    and reaches exactly the same objective L64.
  mixed (reported beside it): tensor-core (split-BF16x3) Hessian products /
    FP32 CG, gradient and objective checks in double-FP32 (~1e-13 relative),
    FP64 line-search decisions and projection, run until its objective is
    within 1e-8 relative of L64 (an extra stopping rule, off by default).
`value` = seconds per solve with the problem resident in HBM (CUDA events on
the library's stream); `e2e` = the same through the C ABI with host buffers
(problem upload, starting point upload, solve, result download inside the
timed region).  With one GPU the line also carries the metric's mixed /
batched comparisons as full time-to-solution: `config3` (M=10^4, N=10^3,
D=2*10^4) and `batch` (64 uneven instances), each with its clock record.

Several GPUs: one process per GPU, every rank solves the same instance
(replicas, no collective in the data path), the step time is the max over
ranks and the ranks' iteration counts are checked identical.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...   # the CPU restatement on host cores
"""
import argparse
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CONFIG = 2
EPS = 1e-6          # the reference's convergence threshold for this workload
OBJ_REL = 1e-8      # mixed precision: objective within 1e-8 relative of L64
MAXITER = 2000
# identical in both arms' lines (the same instance and stopping rule)
WORKLOAD = ("M=2000 N=200 D=4000 x_max=1800 eta=0.9 shots=1e7 gamma=1e-5 seed=0, mode-2 two-stage solve from "
            "Pi=1/N to the reference's stopping rule conv<1e-6 (FP64)")


def _passes(outer, cg, ls):
    """Banded-product passes (one pass = nnz*N FMAs) of a mode-2 solve:
    per outer iteration dL + dL after CG + L + dL + conv_test's dL (9 passes),
    2 per CG iteration (BF), 1 per line-search objective."""
    return 2.0 * cg + 9.0 * outer + ls


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------------------
# CPU restatement (oracle) runs, each in a clean subprocess so OpenMP sees
# the binding environment of pqdts.py (OMP_PROC_BIND, OMP_PLACES).
# --------------------------------------------------------------------------
def _oracle_subprocess(code, threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="true", OMP_PLACES="cores")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("oracle run failed: " + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_sample(config, seed, maxiter, eps, threads):
    """The first `maxiter` outer iterations of each stage (a bounded sample)."""
    code = (
        "import json,sys; sys.path.insert(0,%r)\n"
        "from pqdts_gb300 import synth\n"
        "from oracle.oracle import Oracle, set_threads\n"
        "set_threads(%d)\n"
        "inst=synth.make_config(%d, seed=%d)\n"
        "o=Oracle.from_instance(inst)\n"
        "X,st=o.solve(mode=2,maxiter=%d,eps=%r)\n"
        "print(json.dumps(st))\n" % (ROOT, threads, config, seed, maxiter, eps))
    return _oracle_subprocess(code, threads)


def cpu_full_solve(config, seed, eps, threads):
    """One full solve of the workload: the reference's `min` timer
    (pqdts.f90:1922, 2168) as `seconds`, the final objective's bits, the
    iteration counts and a SHA-256 of the final Pi (column-major bytes)."""
    code = (
        "import hashlib,json,sys; sys.path.insert(0,%r)\n"
        "from pqdts_gb300 import synth\n"
        "from oracle.oracle import Oracle, set_threads\n"
        "set_threads(%d)\n"
        "inst=synth.make_config(%d, seed=%d)\n"
        "o=Oracle.from_instance(inst)\n"
        "X,st=o.solve(mode=2,maxiter=%d,eps=%r)\n"
        "st['L_hex']=float(st['L']).hex()\n"
        "st['pi_sha256']=hashlib.sha256(X.tobytes(order='F')).hexdigest()\n"
        "print(json.dumps(st))\n" % (ROOT, threads, config, seed, MAXITER, eps))
    return _oracle_subprocess(code, threads)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# --------------------------------------------------------------------------
# distributed helpers (one process per GPU; replicas of one instance)
# --------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, use_cuda):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("nccl" if use_cuda else "gloo")
    return dist


def dist_max(dist, v, device):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def rank_workload(config=CONFIG):
    """The instance every rank solves: the same seed on every rank (replicas,
    so the max-over-ranks time measures the same work as one GPU does)."""
    from pqdts_gb300 import synth

    return synth.make_config(config, seed=0)


def replica_check(dist, stats, device):
    """Per-rank (outer, CG, line-search evaluations, objective) of the last
    solve, gathered on every rank; `identical` when all ranks did the same
    work (they solve the same instance, bit for bit)."""
    row = [float(stats["outer"]), float(stats["cg"]), float(stats.get("ls_evals", stats.get("ls", 0.0))),
           float(stats["L"])]
    if dist is None:
        rows = [row]
    else:
        import torch

        t = torch.tensor(row, dtype=torch.float64, device=device)
        out = [torch.zeros_like(t) for _ in range(dist.get_world_size())]
        dist.all_gather(out, t)
        rows = [x.cpu().tolist() for x in out]
    return replica_summary(rows)


def replica_summary(rows):
    """rows[r] = (outer, CG, line-search evaluations, objective) of rank r."""
    return {"identical": all(list(r) == list(rows[0]) for r in rows),
            "per_rank": [{"outer": r[0], "cg": r[1], "ls_evals": r[2], "L": r[3]} for r in rows]}


# --------------------------------------------------------------------------
# reference arm: the CPU restatement on the host cores
# --------------------------------------------------------------------------
def run_reference(args):
    """`value` = one full solve of the workload, timed (the `min` timer);
    each step = a bounded sample of the same solve (the first k outer
    iterations of each stage), so K + W steps end within minutes; the
    samples' seconds per banded-product pass times the full solve's passes
    is reported beside it as a cross-check."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    cores = host_cores()
    samples = []
    for k in range(args.warmup + args.steps):
        st = cpu_sample(CONFIG, 0, args.ref_sample_iters, EPS, cores)
        if k >= args.warmup:
            samples.append(st)
    t0 = time.perf_counter()
    full = cpu_full_solve(CONFIG, 0, EPS, cores)
    full_wall = time.perf_counter() - t0
    value = full["seconds"]
    per_pass = statistics.mean(s["seconds"] / _passes(s["outer"], s["cg"], s["ls"]) for s in samples)
    est = per_pass * _passes(full["outer"], full["cg"], full["ls"])
    unit = "s"
    line = {
        "impl": "reference", "metric": "time-to-solution at 1e-8 rel. objective (mode-2 solve, s)", "value": value,
        "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(s["seconds"] for s in samples) * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, pqdts_gb300.synth)",
        "config": {"workload": WORKLOAD, "threads": cores},
        "step": (f"one bounded sample of the same solve: the first {args.ref_sample_iters} outer iterations of each "
                 f"stage; `value` is the full solve below"),
        "full_solve": {"seconds": value, "wall_s": full_wall, "outer": full["outer"], "cg": full["cg"],
                       "L": full["L"], "L_hex": full["L_hex"], "pi_sha256": full["pi_sha256"]},
        "pass_scaled_estimate_s": est,
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                         "sample": "one full solve of the workload by the oracle (C++/OpenMP restatement of "
                                   "pqdts.f90), all host cores, OMP_PROC_BIND=true OMP_PLACES=cores"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def fp64_peak_tflops(device):
    """cuBLAS DGEMM (torch.matmul float64, n=4096) best of 5: the FP64
    denominator of the roofline (the banded products are FP64-ALU bound)."""
    import torch

    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=device)
    b = torch.randn(n, n, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = math.inf
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return 2.0 * n ** 3 / best / 1e12


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(path))
    except (OSError, ValueError):
        return {}


def profile_traffic(name):
    """dram bytes per launch from a committed ncu summary (profiles/<name>),
    line `traffic_bytes_per_launch: <int>`; None when absent."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def pi_sha256(X):
    return hashlib.sha256(X.tobytes(order="F")).hexdigest()


def timed_solve(solver, device, eps, target=0.0, maxiter=MAXITER):
    """One solve from Pi = 1/N timed with CUDA events on the library's stream."""
    import torch

    stream = torch.cuda.ExternalStream(solver.stream(), device=device)
    solver.set_objective_target(target)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.init_x()
    st = solver.solve(mode=2, maxiter=maxiter, eps=eps)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3, st


def north_star_config3(local, dev):
    """Full time-to-solution at M=10^4, N=10^3, D=2*10^4: the FP64 GPU solve to
    conv < 1e-6, then the mixed solver (tensor-core and CUDA-core Hessian
    products) to an objective within 1e-8 relative of the FP64 one; the error
    of the mixed Pi and objective against the FP64 result."""
    import numpy as np

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    t0 = time.perf_counter()
    inst = synth.make_config(3, seed=0)
    out = {"workload": "M=10000 N=1000 D=20000 x_max=9000 eta=0.75 shots=1e8 gamma=1e-6 seed=0, mode-2 solve "
                       "from Pi=1/N", "nnz_F": inst.nnz, "generation_s": time.perf_counter() - t0}
    clk = Clocks(local).start()
    with pq.Solver(local) as s:
        s.set_option("timers", 0)
        s.set_instance(inst, pq.FP64)
        timed_solve(s, dev, EPS, maxiter=2)  # warm-up: captures both stages' CG graphs
        t64, st64 = timed_solve(s, dev, EPS)
        X64 = s.get_x()
    L64 = st64["L"]
    out["fp64"] = {"seconds": t64, "stop": "conv < 1e-6", "L": L64, "outer": st64["outer"], "cg": st64["cg"]}
    flops_pair = 2 * 2.0 * inst.nnz * inst.N  # useful flops of one Hessian product (F.V, then F^T.(2 F.V))
    peaks = measured_peaks()
    for tc, key in ((-1, "mixed"), (0, "mixed_cuda_cores")):
        with pq.Solver(local) as s:
            s.set_option("tensor_cores", tc)
            s.set_instance(inst, pq.MIXED)
            b0 = s.timer("BF")
            timed_solve(s, dev, 1e-300, L64 * (1.0 + OBJ_REL))  # warm-up, region timers on
            b1 = s.timer("BF")
            s.set_option("timers", 0)
            timed_solve(s, dev, 1e-300, L64 * (1.0 + OBJ_REL))  # warm-up without them
            tm, sm = timed_solve(s, dev, 1e-300, L64 * (1.0 + OBJ_REL))
            Xm = s.get_x()
            bft, bfn = b1[0] - b0[0], b1[1] - b0[1]
            pair = {"calls": bfn, "us_per_call": bft / bfn * 1e6 if bfn else None,
                    "useful_tflops": flops_pair * bfn / bft / 1e12 if bft else None,
                    "note": "the CG's Hessian product (operand split, both products, row epilogue) per CG "
                            "iteration, GPU events in the solve"}
            if tc != 0 and bft and peaks.get("bf16_tflops"):
                # split-BF16x3: three bf16 MMA terms per useful product term (plus the zero fill of each
                # 128-row block's K window, not counted): a lower bound of the tensor pipe's work
                pair["issued_bf16_tflops_lower_bound"] = 3 * pair["useful_tflops"]
                pair["frac_of_bf16_peak_lower_bound"] = 3 * pair["useful_tflops"] / peaks["bf16_tflops"]
                pair["peak_source"] = "MEASURED_PEAKS.json bf16_tflops (burst, of measured)"

            out[key] = {"seconds": tm, "speedup_vs_fp64": t64 / tm, "stop": "objective <= L64*(1+1e-8)",
                        "L": sm["L"], "rel_obj_vs_fp64": (sm["L"] - L64) / L64, "reached": sm["L"] <= L64 * (1 + OBJ_REL),
                        "max_abs_pi_vs_fp64": float(np.max(np.abs(Xm - X64))), "min_pi": float(Xm.min()),
                        "max_row_sum_err": float(np.max(np.abs(Xm.sum(axis=1) - 1.0))),
                        "outer": sm["outer"], "cg": sm["cg"], "refine": sm["refine"],
                        "tensor_cores": bool(s.get_option("sched.tc")), "hessian_product": pair}
    out["clocks"] = clk.stop()
    return out


def north_star_batch(local, maxiter):
    """64 uneven instances (8 base detectors x 8 resampled P, gamma swept
    1e-7..1e-2) through pqdts_cuda_solve_batch, host buffers in and out:
    FP64 at conv < 1e-6, then mixed precision to within 1e-8 relative of each
    FP64 objective.  Wall time of each batched call."""
    import numpy as np

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    t0 = time.perf_counter()
    insts = synth.make_batch(seed=0)
    out = {"workload": "batch of %d instances: M log-uniform 500..5000, N 50..500, D=2M, 8 base detectors x 8 "
                       "resampled P (1e7 shots), gamma 1e-7..1e-2, seed=0" % len(insts),
           "generation_s": time.perf_counter() - t0, "nnz_F_total": int(sum(i.nnz for i in insts))}
    clk = Clocks(local).start()
    t0 = time.perf_counter()
    X64, st64 = pq.solve_batch(insts, precision=pq.FP64, maxiter=maxiter, eps=EPS, device=local)
    t64 = time.perf_counter() - t0
    L64 = np.array([x["L"] for x in st64])
    # the mixed solves stop at their targets; their iteration limit (twice
    # the FP64 one) only bounds an instance whose trajectory crawls
    t0 = time.perf_counter()
    Xm, stm = pq.solve_batch(insts, precision=pq.MIXED, maxiter=2 * maxiter, eps=1e-300,
                             targets=L64 * (1.0 + OBJ_REL), device=local)
    tmix = time.perf_counter() - t0
    out["clocks"] = clk.stop()
    Lm = np.array([x["L"] for x in stm])
    rel = (Lm - L64) / np.abs(L64)
    out["fp64"] = {"seconds": t64, "stop": "conv < 1e-6 per instance (maxiter %d)" % maxiter,
                   "outer_total": sum(x["outer"] for x in st64),
                   "cg_total": sum(x["cg"] for x in st64)}
    out["mixed"] = {"seconds": tmix, "speedup_vs_fp64": t64 / tmix,
                    "stop": "objective <= L64*(1+1e-8) per instance (maxiter %d)" % (2 * maxiter),
                    "outer_total": sum(x["outer"] for x in stm), "cg_total": sum(x["cg"] for x in stm),
                    "max_rel_objective_vs_fp64": float(rel.max()),
                    "instances_at_target": int((Lm <= L64 * (1.0 + OBJ_REL)).sum()), "instances": len(insts),
                    "min_pi": float(min(x.min() for x in Xm)),
                    "max_abs_pi_vs_fp64": float(max(np.max(np.abs(a - b)) for a, b in zip(Xm, X64)))}
    out["mixed"]["reached"] = out["mixed"]["instances_at_target"] == len(insts)
    return out


def run_ours(args):
    import numpy as np
    import torch

    import pqdts_gb300 as pq

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = dist_init(world, True)
    prec = pq.MIXED if args.precision == "mixed" else pq.FP64
    inst = rank_workload()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def timed_solves(solver, nsteps, eps, target=0.0):
        ts, sts = [], []
        for _ in range(nsteps):
            flush.fill_(1.0)  # L2 flush between steps (torch's stream, outside the events)
            t, st = timed_solve(solver, dev, eps, target)
            ts.append(t)
            sts.append(st)
        return ts, sts

    # FP64 reference solution of this instance (the drop-in's result): L64
    s64 = pq.Solver(local)
    s64.set_instance(inst, pq.FP64)
    _, st64 = timed_solves(s64, 1, EPS)
    L64 = st64[0]["L"]
    X64 = s64.get_x()
    target = L64 * (1.0 + OBJ_REL)

    if prec == pq.FP64:
        s, eps_run, tgt = s64, EPS, 0.0
    else:
        s = pq.Solver(local)
        s.set_instance(inst, pq.MIXED)
        eps_run, tgt = 1e-300, target
    # the region timers (CUDA events, ~4 us per span inside a captured CG
    # graph) are read from one solve; the warm-up and timed solves run
    # without them
    s.set_option("timers", 2)  # with the spans of the Hessian product's two products
    bf0, fw0, tr0 = s.timer("BF"), s.timer("BF.fwd"), s.timer("BF.trans")
    _, st_t = timed_solves(s, 1, eps_run, tgt)
    bf1, fw1, tr1 = s.timer("BF"), s.timer("BF.fwd"), s.timer("BF.trans")
    s.set_option("timers", 0)
    timed_solves(s, args.warmup, eps_run, tgt)
    launches0 = s.kernel_launches()
    clocks = Clocks(local)
    dist_barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    times, stats = timed_solves(s, args.steps, eps_run, tgt)
    torch.cuda.synchronize()
    dist_barrier(dist)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    launches = s.kernel_launches() - launches0
    step_s = dist_max(dist, statistics.mean(times), dev)
    rel_err = abs(stats[-1]["L"] - L64) / abs(L64)
    if prec == pq.FP64:
        assert all(x["L"] == L64 for x in stats), "FP64 solve is not deterministic"
    else:
        assert stats[-1]["L"] <= target, f"mixed solve ended at {stats[-1]['L']} above the target {target}"
    replicas = replica_check(dist, stats[-1], dev)
    assert replicas["identical"], f"ranks did different work on the same instance: {replicas}"

    # roofline of the dominant kernel: the transposed product of the CG's
    # Hessian product (k_trans_col's sums of F^T.(2 F.V) over each column's
    # non-zero rows, then k_trans's stencil, projection, mask and p.Hp
    # epilogue), FP64-ALU bound; its forward product (k_fwd_col) is reported
    # beside it
    nnz, N, M, D = inst.nnz, inst.N, inst.M, inst.D
    cg = st_t[0]["cg"]  # the CG iterations of the solve whose regions were timed
    bf_time = bf1[0] - bf0[0]
    tr_time, tr_n = tr1[0] - tr0[0], tr1[1] - tr0[1]
    fw_time, fw_n = fw1[0] - fw0[0], fw1[1] - fw0[1]
    flops_pair = 2 * 2.0 * nnz * N
    flops_one = flops_pair / 2
    achieved_tf = flops_one * tr_n / tr_time / 1e12 if tr_time > 0 else None
    peaks = measured_peaks()
    if prec == pq.FP64:
        peak_tf = fp64_peak_tflops(dev)
        peak_note = "cuBLAS DGEMM (n=4096) measured in this run; FP64 is the binding unit"
    else:
        peak_tf = None
        peak_note = "FP32 CUDA-core products; see profiles/"
    sval = 8 if prec == pq.FP64 else 4
    bytes_pass = nnz * (sval + 4) + (D + 1) * 8 + M * N * sval + D * N * sval
    traffic = profile_traffic("spmm_fp64_config2.txt" if prec == pq.FP64 else "spmm_fp32_config2.txt")
    hbm_gbs = bytes_pass * tr_n / tr_time / 1e9 if tr_time > 0 else None
    executed = None
    if prec == pq.FP64:
        # the FMAs the masked products execute, counted by the kernels, in
        # Hessian products at the solve's final (sparse) Pi with a direction
        # of the same zeros: the rate against the FP64 peak
        Xs = s.get_x()
        V = np.asfortranarray(np.where(Xs != 0.0, Xs - 1.0 / N, 0.0))
        s.set_option("timers", 2)
        s.set_option("count_fmas", 1)
        s.BF(V)
        a0, b0 = s.timer("BF.trans"), s.timer("BF.fwd")
        c0, d0 = s.get_option("fmas.transposed"), s.get_option("fmas.forward")
        for _ in range(5):
            s.BF(V)
        a1, b1 = s.timer("BF.trans"), s.timer("BF.fwd")
        c1, d1 = s.get_option("fmas.transposed"), s.get_option("fmas.forward")
        s.set_option("count_fmas", 0)
        s.set_option("timers", 0)
        ttr, tfw = a1[0] - a0[0], b1[0] - b0[0]
        executed = {
            "where": "5 Hessian products at the final Pi of the solve (V with Pi's zeros), GPU events, FMAs counted "
                     "by the kernels (option count_fmas)",
            "transposed": {"fmas_per_product": (c1 - c0) / 5, "dense_fmas_per_product": nnz * N,
                           "us_per_product": ttr / 5 * 1e6,
                           "executed_tflops": 2 * (c1 - c0) / ttr / 1e12 if ttr > 0 else None},
            "forward": {"fmas_per_product": (d1 - d0) / 5, "dense_fmas_per_product": nnz * N,
                        "us_per_product": tfw / 5 * 1e6,
                        "executed_tflops": 2 * (d1 - d0) / tfw / 1e12 if tfw > 0 else None}}
    roofline = {
        "kernel": "k_col_index + k_trans_col + k_trans (the Hessian product's F^T.(2 F.V): the occupied-row lists "
                  "of each column of 2 F.V, sums over them by (column, 32-row tile of F^T) warps, then the stencil, "
                  "projection, active-set mask epilogue)",
        "timed": "GPU events around each of the CG's transposed products in one solve of the workload "
                 "(region timers on)",
        "bound": "fp64" if prec == pq.FP64 else "fp32",
        "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
        "frac": (achieved_tf / peak_tf) if (achieved_tf and peak_tf) else None,
        "peak_source": peak_note,
        "traffic": traffic,
        "algorithmic_flops_per_launch": flops_one,
        "algorithmic_bytes_per_launch": bytes_pass,
        "us_per_launch": tr_time / tr_n * 1e6 if tr_n else None,
        "hbm_view": {"achieved": hbm_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": (hbm_gbs / peaks["hbm_gbs"]) if (hbm_gbs and peaks.get("hbm_gbs")) else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
        "executed": executed,
        "note": "achieved = algorithmic (dense) flops 2 nnz N per launch over the time; the masked products skip "
                "exact-zero terms and, in the CG, the outputs its active set masks, so this dense-equivalent rate "
                "exceeds the FP64 peak -- `executed` gives the rate of the FMAs the kernels do execute (through "
                "the BF entry point: no active set, no output skipped)",
        "forward_product": {
            "kernel": "k_col_index + k_fwd_col (F.V by (column of V, 32-row tile of F) warps visiting only the rows "
                      "where that column of V is non-zero; the same bits as the full chain)",
            "us_per_launch": fw_time / fw_n * 1e6 if fw_n else None,
            "dense_equivalent_tflops": flops_one * fw_n / fw_time / 1e12 if fw_time > 0 else None,
            "note": "dense-equivalent flops over the time: above the FP64 peak because the skipped terms are exact "
                    "zeros (the iterate and the CG direction are ~90 % zeros on this workload)"},
        "hessian_pair_us": bf_time / max(1, cg) * 1e6,
    }

    # e2e through the C ABI with host buffers
    e2e_times = []
    h2d = d2h = 0
    X0 = np.full((inst.M, inst.N), 1.0 / inst.N, order="F")
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        with pq.Solver(local) as se:
            se.set_option("timers", 0)
            se.set_objective_target(tgt)
            a0 = se.transfer_bytes()
            t0 = time.perf_counter()
            se.set_instance(inst, prec)
            se.set_x(X0)
            se.solve(mode=2, maxiter=MAXITER, eps=eps_run)
            se.get_x()
            e2e_times.append(time.perf_counter() - t0)
            a1 = se.transfer_bytes()
            h2d, d2h = a1[0] - a0[0], a1[1] - a0[1]
    e2e_s = dist_max(dist, statistics.mean(e2e_times), dev)

    # mixed precision on the same inputs (reported beside the FP64 drop-in):
    # time to an objective within 1e-8 relative of L64
    extra = {}
    if prec == pq.FP64 and args.with_mixed and world == 1:
        def mixed_run(tc):
            with pq.Solver(local) as sm:
                sm.set_option("tensor_cores", tc)
                sm.set_instance(inst, pq.MIXED)
                b0, l0, g0 = sm.timer("BF"), sm.timer("L"), sm.timer("dL")
                _, mst = timed_solves(sm, 1, 1e-300, target)  # the region timers' solve
                b1, l1, g1 = sm.timer("BF"), sm.timer("L"), sm.timer("dL")
                sm.set_option("timers", 0)
                timed_solves(sm, args.warmup, 1e-300, target)
                ck = Clocks(local).start()
                mt, ms = timed_solves(sm, args.steps, 1e-300, target)
                mclk = ck.stop()
                mval = statistics.mean(mt)
                cgs = mst[0]["cg"]
                bft = b1[0] - b0[0]
                Xm = sm.get_x()
                out = {"value": mval, "unit": "s", "speedup_vs_fp64": step_s / mval,
                       "stop": "objective <= L64*(1+1e-8)", "objective": ms[-1]["L"],
                       "rel_obj_vs_L64": (ms[-1]["L"] - L64) / L64, "reached": ms[-1]["L"] <= target,
                       "outer": ms[-1]["outer"], "cg": ms[-1]["cg"], "refine": ms[-1]["refine"],
                       "tensor_cores": bool(sm.get_option("sched.tc")),
                       "double_fp32_gradient_and_checks": bool(sm.get_option("sched.df_trans")),
                       # GPU time per solve in the objective (L: checks of the chosen
                       # steps) and gradient (dL) regions, double-FP32 products included
                       # (the region timers' solve)
                       "L_region_s_per_solve": l1[0] - l0[0],
                       "dL_region_s_per_solve": g1[0] - g0[0],
                       "max_abs_pi_vs_fp64": float(np.max(np.abs(Xm - X64))), "min_pi": float(Xm.min()),
                       "max_row_sum_err": float(np.max(np.abs(Xm.sum(axis=1) - 1.0))),
                       "hessian_product_pair": {"us_per_cg_iteration": bft / cgs * 1e6 if cgs else None,
                                                "algorithmic_tflops": flops_pair * cgs / bft / 1e12 if bft else None},
                       "clocks": mclk}
                return out
        extra["mixed"] = mixed_run(-1)
        if extra["mixed"]["tensor_cores"]:
            extra["mixed"]["cuda_core_variant"] = mixed_run(0)

    # parity and CPU baseline in one: the oracle's full solve of the same
    # instance on the host cores, compared with the FP64 GPU result bit for bit
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cores = host_cores()
            full = cpu_full_solve(CONFIG, 0, EPS, cores)
            cpu = {"value": full["seconds"], "unit": "s", "cores": cores, "kind": "port",
                   "sample": "one full solve of the same instance by the oracle (C++/OpenMP restatement of "
                             "pqdts.f90), all host cores, OMP_PROC_BIND=true OMP_PLACES=cores; the reference's "
                             "`min` timer"}
            gpu = {"L_hex": float(L64).hex(), "outer": st64[0]["outer"], "cg": st64[0]["cg"],
                   "pi_sha256": pi_sha256(X64)}
            parity = {"against": "oracle full solve, same instance",
                      "objective_bitwise": gpu["L_hex"] == full["L_hex"],
                      "counts_equal": gpu["outer"] == full["outer"] and gpu["cg"] == full["cg"],
                      "pi_bitwise": gpu["pi_sha256"] == full["pi_sha256"],
                      "gpu": gpu, "oracle": {k: full[k] for k in ("L_hex", "outer", "cg", "pi_sha256")}}
            parity["bitwise"] = parity["objective_bitwise"] and parity["counts_equal"] and parity["pi_bitwise"]
        except Exception as e:  # reported, never silently replaced
            cpu = {"value": None, "error": str(e)[:300]}

    # the metric's mixed / batched comparisons at full time-to-solution
    if prec == pq.FP64 and world == 1 and args.north_star:
        extra["config3"] = north_star_config3(local, dev)
        extra["batch"] = north_star_batch(local, args.batch_maxiter)

    if rank == 0:
        line = {
            "metric": "time-to-solution at 1e-8 rel. objective (mode-2 solve, s)",
            "value": step_s, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == pq.FP64 else "f32+f64",
            "data": "synthetic (seeded, pqdts_gb300.synth; every rank solves the seed-0 instance)",
            "config": {"workload": WORKLOAD,
                       "nnz_F": nnz, "precision": args.precision, "l2": "flushed between steps (256 MiB write)",
                       "objective": stats[-1]["L"], "objective_fp64": L64,
                       "rel_obj_vs_fp64": rel_err, "outer": stats[-1]["outer"], "cg": stats[-1]["cg"],
                       "ls_evals": stats[-1]["ls_evals"], "parallelism": f"{world} replica(s) of one instance",
                       "parity": parity},
            "replicas": replicas,
            "solves_per_s": world / step_s,
            "wall_s_timed_region": t_wall,
            "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        line.update(extra)
        print(json.dumps(line))
    s.close()
    s64.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_profile_case(case):
    """Launches for ncu on the benchmark workload.
      fp64 / mixed: the Hessian product (3x BF resp. BF32), then 3x dL and
        3x L at a random feasible X -- real banded-product launches only
        (fp64: row-flattened products, no autotuning launches);
      solve64 / solvemix: one full benchmark solve (the launch list);
      fp64sp: the FP64 Hessian product (3x BF), 3x dL and 3x L at the
        FP64 solution of the workload (a sparse Pi, as the solve's iterates
        are once in stage 2: the column lists of the products see the
        zeros they skip in the solve; the solve itself runs without the
        zero skipping, so the masked kernels' first launches are these); V =
        that Pi minus 1/N on its non-zeros, so it has the same zeros;
      solvemix3: the mixed solve of M=10000 N=1000 D=20000 to its own
        stopping rule conv < 1e-6 (no FP64 solve first: the launch list of
        the mixed solver alone)."""
    import numpy as np

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    if case in ("tc3", "tcdense", "tc3p", "tcdensep"):
        # the tensor-core Hessian product pair (3 BF32 calls, no autotuning
        # launches) at M=10000 N=1000 D=20000, or on the dense-F variant;
        # ...p: the persistent kernel
        inst = synth.make_config(3 if case.startswith("tc3") else 6, seed=0)
        with pq.Solver(0) as s:
            s.set_option("autotune", 0)
            s.set_option("tc_persistent", 1 if case.endswith("p") else 0)
            s.set_instance(inst, pq.MIXED)
            assert s.get_option("sched.tc") == 1
            rng = np.random.default_rng(0)
            V = rng.standard_normal((inst.M, inst.N))
            for _ in range(3):
                s.BF32(V)
            print(json.dumps({"profile_case": case, "launches": s.kernel_launches(), "nnz": inst.nnz}))
        return 0
    if case == "solvemix3":
        inst = synth.make_config(3, seed=0)
        with pq.Solver(0) as s:
            s.set_option("timers", 0)
            s.set_instance(inst, pq.MIXED)
            st = s.solve(mode=2, maxiter=MAXITER, eps=EPS)
            print(json.dumps({"profile_case": case, "stats": st, "launches": s.kernel_launches(),
                              "schedule": s.schedule()}))
        return 0
    inst = synth.make_config(CONFIG, seed=0)
    prec = pq.MIXED if case in ("mixed", "solvemix") else pq.FP64
    with pq.Solver(0) as s:
        if case == "solve64":
            s.set_option("rows_kernels", 1)  # the form the autotuner picks on this workload
        if case == "fp64":
            # no autotuning launches before the captured ones; the
            # row-flattened products, the form the autotuner picks here
            s.set_option("autotune", 0)
            s.set_option("rows_kernels", 1)
        s.set_instance(inst, prec)
        if case == "fp64sp":
            with pq.Solver(0) as s64:
                s64.set_option("row_masks", 0)  # (no masked-product launches before the profiled ones)
                s64.set_instance(inst, pq.FP64)
                s64.solve(mode=2, maxiter=MAXITER, eps=EPS)
                Xs = s64.get_x()
            s.set_option("autotune", 0)
            V = np.where(Xs != 0.0, Xs - 1.0 / inst.N, 0.0)
            for _ in range(3):
                s.BF(np.asfortranarray(V))
            for _ in range(3):
                s.set_x(Xs)
                s.dL()
            for _ in range(3):
                s.set_x(Xs)
                s.L()
            print(json.dumps({"profile_case": case, "zero_frac": float(np.mean(Xs == 0.0)),
                              "launches": s.kernel_launches()}))
            return 0
        if case.startswith("solve"):
            L64 = None
            if prec == pq.MIXED:
                with pq.Solver(0) as s64:
                    s64.set_instance(inst, pq.FP64)
                    L64 = s64.solve(mode=2, maxiter=MAXITER, eps=EPS)["L"]
                s.set_objective_target(L64 * (1 + OBJ_REL))
            s.init_x()
            st = s.solve(mode=2, maxiter=MAXITER, eps=EPS if prec == pq.FP64 else 1e-300)
            print(json.dumps({"profile_case": case, "stats": st, "launches": s.kernel_launches()}))
            return 0
        rng = np.random.default_rng(0)
        X = rng.random((inst.M, inst.N))
        X /= X.sum(1, keepdims=True)
        s.set_x(X)
        V = rng.standard_normal((inst.M, inst.N))
        for _ in range(3):
            (s.BF32 if prec == pq.MIXED else s.BF)(V)
        for _ in range(3):
            s.set_x(X)
            s.dL()
        for _ in range(3):
            s.set_x(X)
            s.L()
        print(json.dumps({"profile_case": case, "launches": s.kernel_launches()}))
    return 0


def run_workload(name, args):
    """Secondary measurements (one JSON line each, not the bench line):
      batch   -- 64 uneven instances (8 base detectors x 8 resampled P with a
                 gamma sweep) through pqdts_cuda_solve_batch: FP64 at the
                 reference's stopping rule conv < 1e-6, then mixed precision
                 to within 1e-8 relative of each FP64 objective (optionally
                 the FP64 solves one after another for comparison);
      config3 -- M=10000, N=1000, D=20000: FP64 vs mixed (tensor-core and
                 CUDA-core Hessian products) over the first outer iterations;
      dense   -- the same on the dense-F variant M=D=8192, N=256;
      config5 -- the same at M=50000, N=5000, D=100000 (one outer
                 iteration per stage by default)."""
    import numpy as np

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    if name == "batch":
        insts = synth.make_batch(seed=0)
        out = {"workload": "batch of %d instances (8 base detectors x 8 resampled P, gamma 1e-7..1e-2)" % len(insts),
               "sizes": {"M": [i.M for i in insts[::8]], "N": [i.N for i in insts[::8]],
                         "D": [i.D for i in insts[::8]]}}
        # FP64 batch at the reference's stopping rule: each instance's
        # objective L64 is the target of the mixed batch (within 1e-8 rel.)
        t0 = time.perf_counter()
        _, st64 = pq.solve_batch(insts, precision=pq.FP64, maxiter=args.batch_maxiter, eps=EPS)
        t64 = time.perf_counter() - t0
        L64 = np.array([x["L"] for x in st64])
        t0 = time.perf_counter()
        _, stm = pq.solve_batch(insts, precision=pq.MIXED, maxiter=args.batch_maxiter, eps=1e-300,
                                targets=L64 * (1.0 + OBJ_REL))
        tmix = time.perf_counter() - t0
        Lm = np.array([x["L"] for x in stm])
        rel = (Lm - L64) / np.abs(L64)
        out["fp64"] = {"batched_s": t64, "outer_total": sum(x["outer"] for x in st64),
                       "cg_total": sum(x["cg"] for x in st64)}
        out["mixed"] = {"batched_s": tmix, "outer_total": sum(x["outer"] for x in stm),
                        "cg_total": sum(x["cg"] for x in stm), "max_rel_objective_vs_fp64": float(rel.max()),
                        "instances_at_target": int((Lm <= L64 * (1.0 + OBJ_REL)).sum())}
        out["mixed_speedup_vs_fp64"] = t64 / tmix
        out["workers"] = int(os.environ.get("PQDTS_BATCH_WORKERS", "0")) or min(16, os.cpu_count() or 1)
        if args.batch_sequential:
            # the same FP64 solves one after another through one context
            t0 = time.perf_counter()
            with pq.Solver(0) as s:
                Ls = []
                for inst in insts:
                    s.set_instance(inst, pq.FP64)
                    Ls.append(s.solve(mode=2, maxiter=args.batch_maxiter, eps=EPS)["L"])
            out["fp64"]["sequential_s"] = time.perf_counter() - t0
            out["fp64"]["identical_objectives"] = bool(np.array_equal(np.array(Ls), L64))
        print(json.dumps(out))
        return 0
    if name in ("config3", "dense", "config5"):
        cfg = {"config3": 3, "dense": 6, "config5": 5}[name]
        iters = args.config5_iters if cfg == 5 else args.config3_iters
        t0 = time.perf_counter()
        inst = synth.make_config(cfg, seed=0)
        gen_s = time.perf_counter() - t0
        out = {"workload": {3: "M=10000 N=1000 D=20000 (banded F)",
                            6: "M=8192 N=256 D=8192 (dense F, every entry kept)",
                            5: "M=50000 N=5000 D=100000 (banded F)"}[cfg], "nnz_F": inst.nnz,
               "iterations_per_stage": iters, "generation_s": gen_s}
        flops_pair = 2 * 2.0 * inst.nnz * inst.N
        for prec, tc, tag in ((pq.FP64, 0, "fp64"), (pq.MIXED, -1, "mixed_tc"), (pq.MIXED, 0, "mixed_cuda_cores")):
            with pq.Solver(0) as s:
                s.set_option("tensor_cores", tc)
                s.set_instance(inst, prec)
                s.init_x()
                t0 = time.perf_counter()
                st = s.solve(mode=2, maxiter=iters, eps=EPS)
                el = time.perf_counter() - t0
                bf = s.timer("BF")
                tl, tg = s.timer("L"), s.timer("dL")
                out[tag] = {"seconds": el, "outer": st["outer"], "cg": st["cg"],
                            "L_seconds": tl[0], "L_calls": tl[1], "dL_seconds": tg[0], "dL_calls": tg[1],
                            "double_fp32": bool(s.get_option("sched.df_fwd")) if prec == pq.MIXED else False,
                            "s_per_outer": el / max(1, st["outer"]), "L": st["L"],
                            "tensor_cores": bool(s.get_option("sched.tc")) if prec == pq.MIXED else False,
                            "bf_seconds": bf[0], "bf_calls": bf[1],
                            "bf_us_per_call": bf[0] / bf[1] * 1e6 if bf[1] else None,
                            "bf_tflops_algorithmic": flops_pair * st["cg"] / bf[0] / 1e12 if bf[0] else None}
        print(json.dumps(out))
        return 0
    raise SystemExit("unknown workload " + name)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--with-mixed", dest="with_mixed", action="store_true", default=True)
    ap.add_argument("--no-mixed", dest="with_mixed", action="store_false")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-sample-iters", type=int, default=3)
    ap.add_argument("--profile-case", choices=["fp64", "fp64sp", "mixed", "solve64", "solvemix", "solvemix3", "tc3",
                                               "tcdense", "tc3p", "tcdensep"], default=None,
                    help="launches of the workload for ncu (see run_profile_case)")
    ap.add_argument("--workload", choices=["batch", "config3", "dense", "config5"], default=None,
                    help="secondary measurement instead of the bench line")
    ap.add_argument("--batch-maxiter", type=int, default=200)
    ap.add_argument("--no-north-star", dest="north_star", action="store_false", default=True,
                    help="skip the config3 / batch time-to-solution keys of the bench line")
    ap.add_argument("--batch-sequential", action="store_true",
                    help="batch workload: also time the FP64 solves one after another")
    ap.add_argument("--config3-iters", type=int, default=3)
    ap.add_argument("--config5-iters", type=int, default=1)
    args = ap.parse_args()
    if args.workload:
        return run_workload(args.workload, args)
    if args.profile_case:
        return run_profile_case(args.profile_case)
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
