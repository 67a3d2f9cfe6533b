"""ctypes binding of the engine's C ABI (``include/oafdtd.h``).

The library is loaded from the package's own ``lib`` directory. There is no fallback: when the
library or a CUDA device is missing every engine entry point raises, so a CPU path can never stand
in for the GPU engine unnoticed.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Any

from open_analysis_gb300.errors import AccelError, ErrorInfo

ABI_VERSION = 1
OK, E_INVALID, E_OOM, E_CUDA, E_RANGE, E_TABLE, E_NODEVICE, E_TIMEOUT = 0, -1, -2, -3, -4, -5, -6, -7
CODES = {
    E_INVALID: "FDTD_BAD_INPUT",
    E_OOM: "ACCEL_OUT_OF_MEMORY",
    E_CUDA: "ACCEL_DEVICE_ERROR",
    E_RANGE: "FDTD_STEP_RANGE",
    E_TABLE: "FDTD_TOO_MANY_MATERIALS",
    E_NODEVICE: "ACCEL_NO_DEVICE",
    E_TIMEOUT: "ACCEL_TIMEOUT",
}

_d = C.c_double
_i32 = C.c_int32
_i64 = C.c_int64
_pd = C.POINTER(C.c_double)
_pi32 = C.POINTER(C.c_int32)
_pi64 = C.POINTER(C.c_int64)
_pu16 = C.POINTER(C.c_uint16)


class Correction(C.Structure):
    _fields_ = [
        ("kind", _i32),
        ("c", _i32),
        ("a", _i32),
        ("b", _i32),
        ("sign", _d),
        ("lo", _i32 * 3),
        ("hi", _i32 * 3),
    ]


class Problem(C.Structure):
    _fields_ = [
        ("abi_version", _i32),
        ("real_bytes", _i32),
        ("nx", _i32),
        ("ny", _i32),
        ("nz", _i32),
        ("pitch", _i32),
        ("batch", _i32),
        ("dt", _d),
        ("dtmu", _d),
        ("idx", _pu16 * 3),
        ("n_mat", _i32),
        ("ca_tab", _pd),
        ("cb_tab", _pd),
        ("eps_tab", _pd),
        ("inv_primal", _pd * 3),
        ("inv_dual", _pd * 3),
        ("node_w", _pd * 3),
        ("cell_w", _pd * 3),
        ("pmc_mask", _i32),
        ("n_corr", _i32),
        ("corr", C.POINTER(Correction)),
        ("pml", (_pd * 6) * 3),
        ("n_chan", _i32),
        ("max_steps", _i32),
        ("wave", _pd),
        ("drive", _pd),
        ("n_inj", _i64),
        ("inj_comp", _pi32),
        ("inj_flat", _pi64),
        ("inj_amp", _pd),
        ("inj_chan", _pi32),
        ("n_probe", _i32),
        ("probe_kind", _pi32),
        ("probe_comp", _pi32),
        ("probe_off", _pi64),
        ("probe_flat", _pi64),
        ("probe_w", _pd),
        ("n_freq", _i32),
        ("omega", _pd),
        ("record_series", _i32),
        ("ade_poles", _i32),
        ("ade_kp", _pd),
        ("ade_n", _i64 * 3),
        ("ade_flat", _pi64 * 3),
        ("ade_beta", _pd * 3),
        ("ade_cbe", _pd * 3),
        ("sibc_n", _i64),
        ("sibc_poles", _i32),
        ("sibc_nmat", _i32),
        ("sibc_comp", _pi32),
        ("sibc_flat", _pi64),
        ("sibc_hcomp", _pi32),
        ("sibc_hflat", _pi64),
        ("sibc_hsign", _pd),
        ("sibc_mat", _pi32),
        ("sibc_r0", _pd),
        ("sibc_rp", _pd),
        ("sibc_cp", _pd),
        ("sibc_gp", _pd),
    ]


class EnergyView(C.Structure):
    """``oafdtd_energy_view``: device pointers of resident fields for the no-allocation energy."""

    _fields_ = [
        ("real_bytes", _i32),
        ("nx", _i32),
        ("ny", _i32),
        ("nz", _i32),
        ("pitch", _i32),
        ("batch", _i32),
        ("field", C.c_void_p * 6),
        ("idx", C.c_void_p * 3),
        ("eps_tab", C.c_void_p),
        ("node_w", C.c_void_p * 3),
        ("cell_w", C.c_void_p * 3),
        ("stream", C.c_void_p),
    ]


class MaterialDesc(C.Structure):
    """``oafdtd_material_desc``: the native model compiler's input (host pointers)."""

    _fields_ = [
        ("nx", _i32),
        ("ny", _i32),
        ("nz", _i32),
        ("cell_w", _pd * 3),
        ("centres", _pd * 3),
        ("n_regions", _i32),
        ("reg_lo", _pd),
        ("reg_hi", _pd),
        ("reg_eps", _pd),
        ("reg_sig", _pd),
        ("n_poles", _i32),
        ("reg_strength", _pd),
        ("static_fac", _pd),
        ("pec", C.POINTER(C.c_uint8) * 3),
        ("n_loads", _i64),
        ("load_comp", _pi32),
        ("load_lattice", _pi64),
        ("load_sig", _pd),
        ("threads", _i32),
        ("dt", _d),
        ("eps0", _d),
        ("taus", _pd),
    ]


# every exported symbol with its argument types; tests check the library exports exactly these
SIGNATURES: dict[str, tuple[Any, list[Any]]] = {
    "oafdtd_abi_version": (_i32, []),
    "oafdtd_last_error": (C.c_char_p, []),
    "oafdtd_device_count": (_i32, []),
    "oafdtd_set_device": (C.c_int, [_i32]),
    "oafdtd_device_info": (C.c_int, [C.c_char_p, _i32, _pi32, _pi32, _pi64, _pi64, _pi32]),
    "oafdtd_create": (C.c_int, [C.POINTER(Problem), C.POINTER(C.c_void_p)]),
    "oafdtd_destroy": (C.c_int, [C.c_void_p]),
    "oafdtd_step": (C.c_int, [C.c_void_p, _i64]),
    "oafdtd_step_timed": (C.c_int, [C.c_void_p, _i64, _pd]),
    "oafdtd_step_count": (C.c_int, [C.c_void_p, _pi64]),
    "oafdtd_energy": (C.c_int, [C.c_void_p, _pd]),
    "oafdtd_dft": (C.c_int, [C.c_void_p, _pd]),
    "oafdtd_series": (C.c_int, [C.c_void_p, _pd]),
    "oafdtd_fields": (C.c_int, [C.c_void_p, _i32, _pd]),
    "oafdtd_set_field": (C.c_int, [C.c_void_p, _i32, _pd]),
    "oafdtd_step_half": (C.c_int, [C.c_void_p, _i32]),
    "oafdtd_step_async": (C.c_int, [C.c_void_p, _i64]),
    "oafdtd_snapshot_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "oafdtd_snapshot": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oafdtd_restore": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oafdtd_wait": (C.c_int, [C.c_void_p]),
    "oafdtd_plane": (C.c_int, [C.c_void_p, _i32, _i32, _pd]),
    "oafdtd_set_plane": (C.c_int, [C.c_void_p, _i32, _i32, _pd]),
    "oafdtd_plane_device": (C.c_int, [C.c_void_p, _i32, _i32, C.c_void_p]),
    "oafdtd_set_plane_device": (C.c_int, [C.c_void_p, _i32, _i32, C.c_void_p]),
    "oafdtd_peak_bytes": (C.c_int, [C.c_void_p, _pi64]),
    "oafdtd_set_graph": (C.c_int, [C.c_void_p, _i32]),
    "oafdtd_set_tuning": (C.c_int, [C.c_void_p, _i32, _i32]),
    "oafdtd_get_tuning": (C.c_int, [C.c_void_p, _pi32, _pi32]),
    "oafdtd_batch_create": (C.c_int, [C.POINTER(C.c_void_p), _i32, C.POINTER(C.c_void_p)]),
    "oafdtd_batch_step_async": (C.c_int, [C.c_void_p, _i64]),
    "oafdtd_batch_wait": (C.c_int, [C.c_void_p]),
    "oafdtd_batch_graph_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "oafdtd_batch_destroy": (C.c_int, [C.c_void_p]),
    "oafdtd_set_profiling": (C.c_int, [C.c_void_p, _i32]),
    "oafdtd_kernel_times": (C.c_int, [C.c_void_p, _pd, _i32]),
    "oafdtd_model_bytes": (C.c_int, [C.c_void_p, _pd]),
    "oafdtd_graph_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "oafdtd_kernel_bytes": (C.c_int, [C.c_void_p, _pd, _i32]),
    "oafdtd_energy_noalloc": (C.c_int, [C.POINTER(EnergyView), _pd]),
    # native model compiler (host pointers)
    "oafdtd_materials_build": (C.c_int, [C.POINTER(MaterialDesc), C.POINTER(C.c_void_p)]),
    "oafdtd_materials_sizes": (C.c_int, [C.c_void_p, _pi32, _pi64]),
    "oafdtd_materials_fetch": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_uint16)] * 3 + [_pd, _pd] + [_pi64] * 3 + [_pd] * 6),
    "oafdtd_materials_free": (C.c_int, [C.c_void_p]),
    # surrogate kernels (device pointers as void*)
    "oafdtd_mlp_gemm": (
        C.c_int,
        [C.c_void_p] * 6 + [_i32] * 9 + [C.c_float, C.c_void_p],
    ),
    "oafdtd_mlp_colsum": (C.c_int, [C.c_void_p, _i32, _i32, _i32, C.c_void_p, _i32, _i64, _i64, C.c_void_p]),
    "oafdtd_mlp_mse_grad": (C.c_int, [C.c_void_p, C.c_void_p, _i32, _i32] + [C.c_void_p] * 3 + [_i32, C.c_void_p]),
    "oafdtd_mlp_adam": (
        C.c_int,
        [C.c_void_p] * 5 + [_i64, C.c_void_p] + [C.c_float] * 3 + [C.c_void_p, C.c_void_p],
    ),
    "oafdtd_mlp_count": (C.c_int, [C.c_void_p, C.c_void_p]),
    "oafdtd_mlp_gather": (C.c_int, [C.c_void_p, _i32, C.c_void_p, _i32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "oafdtd_mlp_gemm_tn": (
        C.c_int,
        [C.c_void_p] * 7 + [_i32] * 8 + [C.c_float, _i32] + [_i64] * 5 + [C.c_void_p, C.c_void_p],
    ),
    "oafdtd_mlp_transpose": (C.c_int, [C.c_void_p, _i32, _i32, _i32, C.c_void_p, _i32, _i32, _i64, _i64, C.c_void_p]),
}

_lock = threading.Lock()
_lib: C.CDLL | None = None


def library_path() -> Path:
    return Path(__file__).resolve().parent / "lib" / "liboafdtd.so"


def load() -> C.CDLL:
    """Load the engine library once; raise :class:`AccelError` when it was never built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists():
            raise AccelError(
                ErrorInfo(
                    "ACCEL_NATIVE_MISSING",
                    f"the engine library {path.name} is not built",
                    str(path),
                    "Run `python -m open_analysis_gb300.build` (needs nvcc).",
                )
            )
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.oafdtd_abi_version() != ABI_VERSION:
            raise AccelError(ErrorInfo("ACCEL_NATIVE_MISMATCH", "engine library ABI version mismatch", str(path)))
        _lib = lib
        return lib


def check(rc: int, what: str) -> None:
    """Raise for a non-zero status; ``E_RANGE`` becomes ``ValueError`` as in the reference."""
    if rc == OK:
        return
    msg = load().oafdtd_last_error().decode(errors="replace")
    if rc == E_RANGE:
        raise ValueError(msg or "step count exceeds max_steps (wave table length)")
    if rc == E_INVALID:
        from open_analysis_gb300.model import ModelError

        raise ModelError("FDTD_BAD_INPUT", f"{what}: {msg}")
    code = CODES.get(rc, "ACCEL_DEVICE_ERROR")
    raise AccelError(ErrorInfo(code, f"{what}: {msg}", what))


def set_device(device: int) -> None:
    """Select the CUDA device that engines created on this thread use."""
    check(load().oafdtd_set_device(int(device)), "set_device")


def device_info() -> dict[str, Any]:
    """Current-device facts for the AccelReport-shaped report."""
    lib = load()
    name = C.create_string_buffer(256)
    major, minor, rv = _i32(), _i32(), _i32()
    free, total = _i64(), _i64()
    check(
        lib.oafdtd_device_info(name, 256, C.byref(major), C.byref(minor), C.byref(free), C.byref(total), C.byref(rv)),
        "device_info",
    )
    return {
        "device_name": name.value.decode(),
        "compute_capability": f"{major.value}.{minor.value}",
        "free_bytes": int(free.value),
        "total_bytes": int(total.value),
        "runtime_version": f"{rv.value // 1000}.{(rv.value % 1000) // 10}",
    }
