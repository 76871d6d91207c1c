import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library, the CLI and the oracle once per session."""
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def cfg1():
    from pqdts_gb300 import synth

    return synth.make_config(1, seed=0)


@pytest.fixture(scope="session")
def small():
    """A small banded instance with a nontrivial active set and gamma."""
    from pqdts_gb300 import synth

    return synth.make_instance(M=80, N=12, D=160, xmax=60.0, eta=0.85, shots=10**5, gamma=1e-3, eps=1e-6, seed=7)


@pytest.fixture(scope="session")
def empty_rows():
    """Probe rows 117..399 have no band inside M (x_d beyond the last
    photon number): empty F rows and whole empty 128-row blocks; gamma = 0."""
    from pqdts_gb300 import synth

    return synth.make_instance(M=60, N=10, D=400, xmax=500.0, eta=0.85, shots=10**5, gamma=0.0, eps=1e-6, seed=9)


@pytest.fixture(scope="session")
def mid():
    """N = 40 (not a multiple of 32, >= 32): the row-flattened FP64 products
    apply (4 rows x 40 columns = 5 full warps per block)."""
    from pqdts_gb300 import synth

    return synth.make_instance(M=300, N=40, D=600, xmax=250.0, eta=0.85, shots=10**6, gamma=1e-4, eps=1e-6, seed=11)
