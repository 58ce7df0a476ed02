"""Test configuration: import paths, the `gpu` marker, and the oracle build.

`-m "not gpu"` tests run on any machine (oracle against known answers, host logic, the
C ABI's exports); `-m gpu` tests call the CUDA path through the C ABI on a GB300 and
compare it with the oracle.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "rust-sloth_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsloth_gpu.so")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The oracle and the GPU-free loader tool (`sloth_meshdump`) are built for every run,
    so the loader tests never depend on an earlier build step."""
    from oracle.build import build_oracle
    import build as pkg_build   # rust-sloth_gb300/build.py
    build_oracle()
    pkg_build.build_meshdump()
