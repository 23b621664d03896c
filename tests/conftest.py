import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    lib = os.path.join(ROOT, "kaminogpu_gb300", "lib", "libkamino_gb300.so")
    orc = os.path.join(ROOT, "oracle", "_build", "libkamino_oracle.so")
    if not (os.path.exists(lib) and os.path.exists(orc)):
        import __graft_entry__
        __graft_entry__.build()


_ensure_built()


@pytest.fixture(scope="session")
def kg():
    import kaminogpu_gb300
    return kaminogpu_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle
