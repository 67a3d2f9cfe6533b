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


def test_other_structs_match_c_layout(tmp_path: Path) -> None:
    """``oafdtd_material_desc`` and ``oafdtd_energy_view`` as C lays them out."""
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    structs = {"oafdtd_material_desc": native.MaterialDesc, "oafdtd_energy_view": native.EnergyView}
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for cname, py in structs.items():
        src.append(f'printf("{cname}.size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            src.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src.append("return 0; }")
    c_file = tmp_path / "layout2.c"
    c_file.write_text("\n".join(src))
    exe = tmp_path / "layout2"
    subprocess.run([gcc, str(c_file), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(out[f"{cname}.size"]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)


def test_native_compiler_from_plain_c(tmp_path: Path) -> None:
    """A C program linked against the library builds the materials of a small vacuum box with one
    dielectric region (no GPU involved): the table holds vacuum and the region, every non-PEC
    edge is indexed, the PEC edges are 0."""
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib_path = native.library_path()
    prog = r'''
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include "HEADER"
int main(void) {
  enum { NX = 6, NY = 5, NZ = 4 };
  double w[3][NX + 2], c[3][NX];
  const int n[3] = {NX, NY, NZ};
  for (int a = 0; a < 3; ++a) {
    for (int i = 0; i < n[a] + 2; ++i) w[a][i] = (i >= 1 && i <= n[a]) ? 1e-3 : 0.0;
    for (int i = 0; i < n[a]; ++i) c[a][i] = (i + 0.5) * 1e-3;
  }
  const long lat = (long)(NX + 1) * (NY + 1) * (NZ + 1);
  uint8_t* pec[3];
  for (int a = 0; a < 3; ++a) pec[a] = calloc(lat, 1);
  pec[2][0] = 1; /* one PEC edge */
  double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {1.0, 1.0, 2.0e-3}, eps = 4.0, sig = 0.0;
  oafdtd_material_desc d = {0};
  d.nx = NX; d.ny = NY; d.nz = NZ;
  for (int a = 0; a < 3; ++a) { d.cell_w[a] = w[a]; d.centres[a] = c[a]; d.pec[a] = pec[a]; }
  d.n_regions = 1; d.reg_lo = lo; d.reg_hi = hi; d.reg_eps = &eps; d.reg_sig = &sig;
  d.n_poles = 0; d.threads = 2; d.dt = 1e-12; d.eps0 = 8.854e-12;
  oafdtd_materials* m = NULL;
  if (oafdtd_materials_build(&d, &m) != 0) { printf("build failed %s\n", oafdtd_last_error()); return 1; }
  int32_t nmat; int64_t ade[3];
  oafdtd_materials_sizes(m, &nmat, ade);
  const int pitch = (NX + 2 + 31) / 32 * 32;
  const long st = (long)(NZ + 2) * (NY + 2) * pitch;
  uint16_t* idx[3];
  for (int a = 0; a < 3; ++a) idx[a] = calloc(st, 2);
  double et[16], stab[16];
  oafdtd_materials_fetch(m, idx[0], idx[1], idx[2], et, stab, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL);
  oafdtd_materials_free(m);
  long zeros = 0, max_id = 0;
  for (int k = 1; k <= NZ + 1; ++k)
    for (int j = 1; j <= NY + 1; ++j)
      for (int i = 1; i <= NX + 1; ++i) {
        const uint16_t v = idx[2][((long)k * (NY + 2) + j) * pitch + i];
        if (v == 0) ++zeros;
        if (v > max_id) max_id = v;
      }
  printf("nmat %d ade %ld eps1 %.17g eps2 %.17g eps3 %.17g zeros %ld max_id %ld\n", nmat,
         (long)(ade[0] + ade[1] + ade[2]), et[1], et[2], et[3], zeros, max_id);
  return 0;
}
'''.replace("HEADER", str(HEADER))
    c_file = tmp_path / "use.c"
    c_file.write_text(prog)
    exe = tmp_path / "use"
    subprocess.run([gcc, str(c_file), "-o", str(exe), str(lib_path), f"-Wl,-rpath,{lib_path.parent}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2], strict=False))
    # PEC entry 0, then the sorted keys: vacuum, the interface average (4 + 1) / 2, the region
    assert int(vals["nmat"]) == 4 and vals["ade"] == "0"
    assert [float(vals[k]) for k in ("eps1", "eps2", "eps3")] == [1.0, 2.5, 4.0]
    assert int(vals["zeros"]) == 1  # exactly the one PEC edge
    assert int(vals["max_id"]) == 3
