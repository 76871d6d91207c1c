"""Generate tests/golden/oracle_golden.json: the oracle's results on seeded
inputs, to pin the restatement across machines and rebuilds.

  python tests/golden/make_golden.py

Cases
  config1      M=200 N=20 D=400 (benchmark configuration 1), file F, mode 2
  small_mode1  M=80 N=12 D=160, mode 1
  internal_F   D=21, M=(D-1)^2=400, N=20, F computed internally (nnzF < 0)
               and P from the seeded stream (nnzP < 0)

Recorded: sha256 of the inputs (F band values, P), the final objective as
float.hex, iteration counts, sha256 of the final X (float64, column-major),
and L / sha256(dL) at a fixed feasible point.  Everything is bit-exact: the
generator uses IEEE basic operations only and the oracle fixed-order
arithmetic (the internal-F case also depends on the C library's lgamma/exp).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def point(M, N, seed):
    rng = np.random.default_rng(seed)
    X = rng.random((M, N))
    return np.asfortranarray(X / X.sum(1, keepdims=True))


def case_results(o, mode, maxiter, eps, M, N):
    X, st = o.solve(mode=mode, maxiter=maxiter, eps=eps)
    Xp = point(M, N, 99)
    Lp, _ = o.L(Xp)
    G, _ = o.dL(Xp)
    return {"L": float(st["L"]).hex(), "outer": int(st["outer"]), "cg": int(st["cg"]), "ls": int(st["ls"]),
            "X_sha": sha(np.asfortranarray(X).ravel(order="F")), "L_point": float(Lp).hex(),
            "dL_point_sha": sha(np.asfortranarray(G).ravel(order="F"))}


def build_cases():
    from oracle.oracle import Oracle
    from pqdts_gb300 import synth

    out = {}
    inst = synth.make_config(1, seed=0)
    out["config1"] = {"inputs": {"F_sha": sha(inst.band_val), "P_sha": sha(inst.P), "nnz": inst.nnz},
                      **case_results(Oracle.from_instance(inst), 2, 200, 1e-6, inst.M, inst.N)}
    small = synth.make_instance(M=80, N=12, D=160, xmax=60.0, eta=0.85, shots=10**5, gamma=1e-3, eps=1e-6, seed=7)
    out["small_mode1"] = {"inputs": {"F_sha": sha(small.band_val), "P_sha": sha(small.P), "nnz": small.nnz},
                          **case_results(Oracle.from_instance(small), 1, 40, 1e-6, small.M, small.N)}
    M, N, D = 400, 20, 21
    o = Oracle(M, N, D, 1e-4, None, None)
    lo, hi, off, val = o.bands()
    out["internal_F"] = {"inputs": {"F_sha": sha(val), "P_sha": sha(o.P()), "nnz": int(val.size)},
                         **case_results(o, 2, 200, 1e-6, M, N)}
    return out


if __name__ == "__main__":
    res = build_cases()
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res, indent=1))
