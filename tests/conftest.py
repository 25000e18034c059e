import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as G

    mod = G.load_package()
    lib = mod.native.LIB_PATH
    if not os.path.exists(lib):
        G._load_build_module().build()
    return mod


@pytest.fixture(scope="session")
def oracle():
    from oracle import tnmmap_oracle

    return tnmmap_oracle


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture
def emulated(pkg, monkeypatch):
    """``native.Program`` replaced by the numpy emulator of the compiled
    program, so the decoder classes run on the CPU (the product itself has
    no CPU path: this stand-in exists only in the tests)."""
    import tensorqec_gb300.native as native
    from plan_emulator import EmulatedProgram

    EmulatedProgram.instances = []
    monkeypatch.setattr(native, "Program", EmulatedProgram)
    return EmulatedProgram
