"""Structured errors, shaped like the reference's ``oa_accel`` errors.

Mirrors ``packages/oa-accel/src/oa_accel/errors.py:17-34`` (``ErrorInfo``, ``AccelError``) so that
callers which classify failures by ``code`` (the worker's error line, the adapter's ``collect``)
see the same shape from this engine.
"""

from __future__ import annotations

from dataclasses import asdict, dataclass


@dataclass(frozen=True)
class ErrorInfo:
    """Machine-readable failure: stable code, one sentence, optional path and hint."""

    code: str
    message: str
    path: str | None = None
    hint: str | None = None

    def to_dict(self) -> dict[str, str | None]:
        return asdict(self)


class AccelError(Exception):
    """Raised when the device path fails; always carries an :class:`ErrorInfo`."""

    def __init__(self, info: ErrorInfo) -> None:
        super().__init__(f"{info.code}: {info.message}")
        self.info = info
