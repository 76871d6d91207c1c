"""The C-ABI library loads on a machine without a GPU and exports every
symbol that include/pqdts_cuda.h declares; without a device the entry points
return error codes instead of crashing or falling back to the CPU."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*int\s+(pqdts_cuda_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared()
    for must in ("pqdts_cuda_create", "pqdts_cuda_set_problem", "pqdts_cuda_solve", "pqdts_cuda_L", "pqdts_cuda_dL",
                 "pqdts_cuda_BF", "pqdts_cuda_simplexproj", "pqdts_cuda_solve_batch"):
        assert must in names


def test_library_exports_all_declared_symbols(built):
    import pqdts_gb300 as pq

    L = C.CDLL(pq.LIB_PATH)
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_library_exports_the_reference_condat_symbol(built):
    """simplexproj_condat_ (condat_simplexproj.c:60) with its C prototype in
    the header, exported under that exact name, so pqdts.f90's call at
    :1133 links against the library unchanged."""
    import pqdts_gb300 as pq

    src = open(os.path.join(ROOT, "include", "pqdts_cuda.h")).read()
    assert re.search(r"^void simplexproj_condat_\(double\* y, double\* x, int\* plength\);", src, flags=re.M)
    assert hasattr(C.CDLL(pq.LIB_PATH), "simplexproj_condat_")


def test_no_device_is_an_error_code(built):
    import torch

    if torch.cuda.is_available():
        import pytest

        pytest.skip("a GPU is present")
    import pqdts_gb300 as pq

    h = C.c_void_p()
    rc = pq.lib().pqdts_cuda_create(0, C.byref(h))
    assert rc < 0 and not h.value


def test_cli_usage_without_args(built):
    import subprocess

    import pqdts_gb300 as pq

    r = subprocess.run([pq.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr


def test_fortran_module_binds_every_entry_point():
    """pqdts_gb300/fortran/pqdts_cuda_mod.f90 declares an iso_c_binding
    interface for each function of the C header (no Fortran compiler here:
    checked by name)."""
    src = open(os.path.join(ROOT, "pqdts_gb300", "fortran", "pqdts_cuda_mod.f90")).read()
    bound = set(re.findall(r'bind\(C,\s*name="(pqdts_cuda_\w+)"\)', src))
    assert bound == set(_declared()), (set(_declared()) - bound, bound - set(_declared()))
