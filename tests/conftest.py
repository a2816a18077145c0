"""Shared fixtures: the package is imported from `qxtools.jl_gb300/` as `qxtools_gb300`."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as _entry  # noqa: E402

_entry.load()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libqxgpu.so")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def q():
    return _entry.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_lib(q):
    """libqxgpu built for this machine (the GPU tests build it once if missing)."""
    lib = ROOT / "qxtools.jl_gb300" / "_build" / "libqxgpu.so"
    if not lib.exists():
        _entry._load_build_module().build()
    return q.load_library()
