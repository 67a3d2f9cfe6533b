"""The C ABI library: builds, loads, exports exactly what include/oafdtd.h declares, and the ctypes
descriptor has the C struct's layout. No device calls (runs without a GPU)."""

from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from open_analysis_gb300 import native

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "oafdtd.h"


def declared() -> set[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(oafdtd_[a-z_0-9]+)\s*\(", text))


@pytest.fixture(scope="module")
def lib() -> C.CDLL:
    if not native.library_path().exists():
        if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
            pytest.skip("engine library not built and nvcc unavailable")
        from open_analysis_gb300 import build

        build.build()
    return native.load()


def test_library_exports_every_declared_symbol(lib: C.CDLL) -> None:
    names = declared()
    assert names, "no declarations parsed"
    for name in names:
        assert hasattr(lib, name), name
    assert names == set(native.SIGNATURES), names ^ set(native.SIGNATURES)


def test_abi_version_and_no_device_path(lib: C.CDLL) -> None:
    assert lib.oafdtd_abi_version() == native.ABI_VERSION
    assert lib.oafdtd_device_count() >= 0
    # a null descriptor is rejected before any device work
    h = C.c_void_p()
    assert lib.oafdtd_create(None, C.byref(h)) == native.E_INVALID
    assert lib.oafdtd_last_error()


def _c_layout() -> dict[str, int]:
    fields = [name for name, _ in native.Problem._fields_]
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    src.append('printf("size %zu\\n", sizeof(oafdtd_problem));')
    for f in fields:
        src.append(f'printf("{f} %zu\\n", offsetof(oafdtd_problem, {f}));')
    src.append('printf("corr_size %zu\\n", sizeof(oafdtd_correction));')
    src.append("return 0; }")
    return {"src": "\n".join(src)}  # type: ignore[dict-item]


def test_ctypes_struct_matches_c_layout(tmp_path: Path) -> None:
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    c_file = tmp_path / "layout.c"
    c_file.write_text(_c_layout()["src"])  # type: ignore[index]
    exe = tmp_path / "layout"
    subprocess.run([gcc, str(c_file), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    assert int(out["size"]) == C.sizeof(native.Problem)
    assert int(out["corr_size"]) == C.sizeof(native.Correction)
    for name, _ in native.Problem._fields_:
        assert int(out[name]) == getattr(native.Problem, name).offset, name
