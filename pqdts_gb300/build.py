"""In-tree build of the CUDA library and the CLI drop-in.

  pqdts_gb300/libpqdts_cuda.so   nvcc, sm_103a only, -lineinfo
  pqdts_gb300/pqdts_cuda.x       g++ host CLI linked against the library

No cmake; one translation unit per artefact so a fresh machine builds in
well under a minute.  Outputs are git-ignored.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libpqdts_cuda.so")
CLI = os.path.join(HERE, "pqdts_cuda.x")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [os.path.join(ROOT, "include", "pqdts_cuda.h")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return r.stdout + r.stderr


def build(force=False, verbose_ptxas=False):
    deps = _sources() + [__file__]
    if force or _stale(LIB, deps):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
               "-o", LIB, os.path.join(CSRC, "pqdts_cuda.cu")]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        out = _run(cmd)
        if verbose_ptxas:
            sys.stderr.write(out)
    if force or _stale(CLI, deps + [LIB]):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
        _run(["g++", "-O2", "-std=c++17", "-o", CLI, os.path.join(CSRC, "pqdts_cuda_main.cpp"), "-L" + HERE,
              "-lpqdts_cuda", "-Wl,-rpath,$ORIGIN", "-L" + cuda_lib, "-lcudart"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print("built", LIB, CLI)
