from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "vectorized-join_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _import(path: Path, name: str):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def oracle():
    mod = _import(ROOT / "oracle" / "oracle.py", "vj_oracle")
    mod.build()
    return mod


@pytest.fixture(scope="session")
def vjlib():
    """The ctypes binding of the built library (built on demand, never a fallback)."""
    builder = _import(PKG / "build.py", "vj_build")
    builder.build()
    return _import(PKG / "vj.py", "vj")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ctx(vjlib, cuda):
    c = vjlib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def hash_kat():
    import numpy as np

    return np.load(GOLDEN / "hash_kat.npz")


@pytest.fixture(scope="session")
def join_cases():
    import numpy as np

    return np.load(GOLDEN / "join_cases.npz")
