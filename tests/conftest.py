"""Shared test setup: the `gpu` marker, import paths, and the oracle/reference handles.

Tests marked `gpu` need a CUDA device and go through libntg.so's C ABI; everything else runs on
the CPU (oracle pins, fixtures, host tables, ABI exports)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "nvidia-texture-tools_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build_oracle()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference library built from its own sources; skipped where the source tree is absent."""
    import pyoracle
    path = pyoracle.build_reference()
    if path is None:
        pytest.skip("reference source tree not available on this machine")
    return pyoracle.Reference(path)


@pytest.fixture(scope="session")
def ntg_lib():
    import ntg
    ntg.build()
    return ntg.lib()


@pytest.fixture(scope="session")
def ctx(ntg_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntg
    c = ntg.Context(0)
    yield c
    c.close()
