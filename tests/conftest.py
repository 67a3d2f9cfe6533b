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


def pytest_collection_modifyitems(config: pytest.Config, items: list[pytest.Item]) -> None:
    """GPU tests need the built library and a device; without them they are skipped loudly."""
    gpu_items = [i for i in items if i.get_closest_marker("gpu")]
    if not gpu_items:
        return
    reason = None
    try:
        from open_analysis_gb300 import native

        if native.load().oafdtd_device_count() == 0:
            reason = "no CUDA device visible"
    except Exception as exc:  # library not built
        reason = f"engine library unavailable: {exc}"
    if reason:
        for item in gpu_items:
            item.add_marker(pytest.mark.skip(reason=reason))
