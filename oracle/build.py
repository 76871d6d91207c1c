"""Build recipe for the CPU oracle (test infrastructure only).

Outputs (all git-ignored):
  oracle/liboracle.so      ctypes library used by tests/ and bench.py's CPU leg
  oracle/pqdts_oracle.x    CLI with pqdts_omp.x's 14 positional arguments
  oracle/_ref/libcondat_ref.so
                           the reference's own condat_simplexproj.c, compiled
                           where it lies in the reference tree, only when that
                           tree is present (it is absent on the GPU machine)

Floating point: -ffp-contract=off so that only the explicit std::fma calls in
the restatement fuse; -mfma on x86-64 turns them into single instructions
(aarch64 has FMA in its base ISA).  No -march=native: results must be the
same on the x86 build machine and the aarch64 GPU host.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: PQDTS_REFERENCE_TREE, else a checkout named
# `reference` beside this repository; absent (the GPU machine) -> skipped.
REFERENCE_TREE = os.environ.get("PQDTS_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                         "reference")


def _flags():
    f = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function"]
    if platform.machine() in ("x86_64", "AMD64"):
        f.append("-mfma")
    return f


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed: " + " ".join(cmd))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False):
    src = os.path.join(HERE, "pqdts_oracle.cpp")
    lib = os.path.join(HERE, "liboracle.so")
    exe = os.path.join(HERE, "pqdts_oracle.x")
    if force or _stale(lib, [src, __file__]):
        _run(["g++", *_flags(), "-shared", src, "-o", lib])
    if force or _stale(exe, [src, __file__]):
        _run(["g++", *_flags(), "-DORACLE_MAIN", src, "-o", exe])
    ref_c = os.path.join(REFERENCE_TREE, "condat_simplexproj.c")
    if os.path.exists(ref_c):
        out_dir = os.path.join(HERE, "_ref")
        os.makedirs(out_dir, exist_ok=True)
        ref_so = os.path.join(out_dir, "libcondat_ref.so")
        if force or _stale(ref_so, [ref_c, __file__]):
            # The reference compiles this file with g++ (Makefile:2,19-20).
            _run(["g++", "-O3", "-fPIC", "-shared", "-ffp-contract=off", ref_c, "-o", ref_so])
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("oracle built")
