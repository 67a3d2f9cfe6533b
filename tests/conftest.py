"""Test configuration: the ``gpu`` marker and import paths.

``-m gpu`` tests need a CUDA device and the built library; ``-m "not gpu"`` tests run anywhere
(the oracle against the golden fixtures, the host logic, the library's exported symbols).
"""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "tests" / "golden", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine library")
    config.addinivalue_line("markers", "slow: long CPU run")
