"""pqdts_cuda.x as a drop-in for pqdts_omp.x: same arguments, same data/
inputs, same output files and stdout lines as the oracle's CLI (which
restates pqdts_omp.x), on the same working-directory layout that pqdts.py
prepares (pqdts.py:15-73)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _read_state(path):
    from scipy.io import FortranFile

    f = FortranFile(path, "r")
    M = f.read_ints(np.int64)[0]
    N = f.read_ints(np.int64)[0]
    D = f.read_ints(np.int64)[0]
    ML = f.read_ints(np.int64)[0]
    rank = f.read_ints(np.int32)[0]
    X = f.read_reals(float).reshape((ML, N), order="F")
    return M, N, D, ML, rank, X


def _run(exe, cwd, args):
    r = subprocess.run([exe, *map(str, args)], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _iter_lines(out):
    # what pqdts.py parses: lines starting with " iter   ", token 4 = objective
    return [ln.split() for ln in out.splitlines() if ln.startswith(" iter   ")]


@pytest.mark.parametrize("output", [1, 2])
def test_cli_matches_oracle_cli(built, tmp_path, small, output):
    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    dirs = {}
    for name in ("gpu", "oracle"):
        d = tmp_path / name
        d.mkdir()
        nF, nP = synth.write_data_dir(small, str(d))
        dirs[name] = d
    args = [small.M, small.N, small.D, nF, nP, 2, 100, output, small.gamma, small.eps, 1, 0, 0, 0]
    out_g = _run(pq.CLI_PATH, dirs["gpu"], args)
    out_o = _run(os.path.join(os.path.dirname(pq.__file__), "..", "oracle", "pqdts_oracle.x"), dirs["oracle"], args)
    it_g, it_o = _iter_lines(out_g), _iter_lines(out_o)
    assert len(it_g) == len(it_o) and len(it_g) > 2
    for a, b in zip(it_g, it_o):
        assert a[:5] == b[:5]  # stage, iteration, "L=", objective -- identical text
        assert float(a[4]) == float(b[4])
    fin_g = _read_state(str(dirs["gpu"] / "rank_     0_final.dat"))
    fin_o = _read_state(str(dirs["oracle"] / "rank_     0_final.dat"))
    assert fin_g[:5] == fin_o[:5] == (small.M, small.N, small.D, small.M, 0)
    assert np.array_equal(fin_g[5], fin_o[5])
    # byte-identical files
    assert (dirs["gpu"] / "rank_     0_final.dat").read_bytes() == (dirs["oracle"] / "rank_     0_final.dat").read_bytes()
    for stage in (1, 2):
        name = f"rank_     0_oiter     {stage}.dat"
        assert (dirs["gpu"] / name).exists() == (output >= 2)
        if output >= 2:
            assert (dirs["gpu"] / name).read_bytes() == (dirs["oracle"] / name).read_bytes()
    status = (dirs["gpu"] / "status_           0 .out").read_text()
    assert any(ln.startswith(" VmHWM:") for ln in status.splitlines())
    assert (dirs["gpu"] / "timing_           0 .out").exists()


def test_cli_restart_and_smoothing(built, tmp_path, small):
    """read_input = 1 reads data/initial_     0.dat as pqdts.py writes it
    (pqdts.py:42-58, scipy FortranFile with int64 header records)."""
    from scipy.io import FortranFile

    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    rng = np.random.default_rng(0)
    X0 = rng.random((small.M, small.N))
    X0 /= X0.sum(1, keepdims=True)
    outs = {}
    for name, exe in (("gpu", pq.CLI_PATH),
                      ("oracle", os.path.join(os.path.dirname(pq.__file__), "..", "oracle", "pqdts_oracle.x"))):
        d = tmp_path / name
        d.mkdir()
        nF, nP = synth.write_data_dir(small, str(d))
        fi = FortranFile(str(d / "data" / "initial_     0.dat"), "w")
        for v in (small.M, small.N, small.D, small.M, 0):
            fi.write_record(np.array([v], dtype=np.int64))
        fi.write_record(X0.reshape(small.M * small.N, order="F"))
        fi.close()
        # smoothing factor 2 (arg 13): rows beyond 100 only, so M=80 keeps X0
        _run(exe, d, [small.M, small.N, small.D, nF, nP, 2, 60, 1, small.gamma, small.eps, 2, 1, 2.0, 0])
        outs[name] = (d / "rank_     0_final.dat").read_bytes()
    assert outs["gpu"] == outs["oracle"]


def test_cli_internal_F(built, tmp_path):
    """nnzF = -1: F computed internally with M = (D-1)^2."""
    import pqdts_gb300 as pq
    from pqdts_gb300 import synth

    D, N = 16, 10
    M = (D - 1) ** 2
    inst = synth.make_instance(M=M, N=N, D=D, xmax=200.0, eta=0.8, shots=10**5, gamma=1e-4, eps=1e-6, seed=5)
    outs = {}
    for name, exe in (("gpu", pq.CLI_PATH),
                      ("oracle", os.path.join(os.path.dirname(pq.__file__), "..", "oracle", "pqdts_oracle.x"))):
        d = tmp_path / name
        d.mkdir()
        _, nP = synth.write_data_dir(inst, str(d), with_F=False)
        _run(exe, d, [M, N, D, -1, nP, 2, 50, 1, 1e-4, 1e-6, 1, 0, 0, 0])
        outs[name] = (d / "rank_     0_final.dat").read_bytes()
    assert outs["gpu"] == outs["oracle"]
