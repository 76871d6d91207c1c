"""The reference's own wrapper script (pqdts.py) drives a CLI with
pqdts_omp.x's interface end to end: it writes data/{P,F}_*.bin, runs the
executable with the 14 positional arguments, parses its `iter` lines and the
status file, and reads rank_     0_final.dat back.  Run here against the
oracle's CLI, whose output files the GPU CLI reproduces byte for byte
(tests/test_gpu_cli.py); skipped where the reference tree is absent.  The
wrapper's plots go to a no-op matplotlib (tests/stubs)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _wrapper():
    sys.path.insert(0, ROOT)
    from oracle import build as obuild

    path = os.path.join(obuild.REFERENCE_TREE, "pqdts.py")
    if not os.path.exists(path):
        pytest.skip("reference wrapper not present")
    return path


def test_reference_wrapper_drives_the_cli(built, tmp_path):
    from oracle.oracle import Oracle
    from pqdts_gb300 import synth

    wrapper = _wrapper()
    inst = synth.make_instance(M=80, N=12, D=160, xmax=60.0, eta=0.85, shots=10**5, gamma=1e-3, eps=1e-6, seed=7)
    F = np.zeros((inst.D, inst.M))
    off = 0
    for d in range(inst.D):
        if inst.band_lo[d] >= 0:
            w = inst.band_hi[d] - inst.band_lo[d] + 1
            F[d, inst.band_lo[d] : inst.band_hi[d] + 1] = inst.band_val[off : off + w]
            off += w
    np.save(tmp_path / "P.npy", inst.P)
    np.save(tmp_path / "F.npy", F)
    cli = os.path.join(ROOT, "oracle", "pqdts_oracle.x")
    env = dict(os.environ, PYTHONPATH=os.path.join(ROOT, "tests", "stubs"))
    r = subprocess.run([sys.executable, wrapper, "-P", "P.npy", "-F", "F.npy", "-p", cli, "-e", "1e-6", "-g", "1e-3",
                        "-m", "200", "-o", "povm.npy"], cwd=tmp_path, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    povm = np.load(tmp_path / "povm.npy")
    X, st = Oracle.from_instance(inst).solve(mode=2, maxiter=200, eps=1e-6)
    assert povm.shape == (inst.M, inst.N)
    assert np.array_equal(povm, X)  # the same solve, read back through the wrapper
    assert "objective value=" in r.stdout
