"""ctypes binding of libsimplemoc_gb300.so (the C ABI in include/simplemoc_gb300.h).

The library is loaded from the package directory.  There is no fallback: if the
shared library is missing or was built for another machine, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libsimplemoc_gb300.so"

MOC_OK = 0
MOC_ERR_ARG = 1
MOC_ERR_CUDA = 2
MOC_ERR_OOM = 3
MOC_ERR_STATE = 4
MOC_ERR_TIMEOUT = 5
MOC_ERR_UNSUPPORTED = 6
MOC_ERR_NO_DEVICE = 7

MOC_MODE_PLAIN = 0
MOC_MODE_MIXED = 1
MOC_MODE_FP64 = 2
MOC_FLAG_COMPENSATED = 0x1
MOC_FLAG_SIMT_UPDATE = 0x2
MOC_FLAG_DETERMINISTIC = 0x4
MOC_FLAG_FP32_STATE = 0x8
MOC_FAULT_CUDA = 0
MOC_FAULT_DEVICE_INPUT = 1
MOC_FAULT_DEVICE_TIMEOUT = 2
# phases of the reference's results summary (src/main.c:103-113)
PHASE_NAMES = ("Transport Sweep", "Domain Flux Exchange", "Flux Renormalization",
               "Update Source", "K-Effective Calc")

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)


class MocDims(C.Structure):
    _fields_ = [
        ("n_groups", C.c_int32), ("fai", C.c_int32), ("cai", C.c_int32),
        ("decomp_ax", C.c_int32), ("height", C.c_float), ("axial_exp", C.c_int32),
        ("n_sources", C.c_int64), ("n_sigt", C.c_int32), ("n_xs", C.c_int32),
        ("n_tracks_2d", C.c_int64), ("n_polar", C.c_int32), ("z_stacked", C.c_int32),
        ("n_seg", C.c_int32), ("table_n", C.c_int32), ("table_dx", C.c_float),
        ("table_maxval", C.c_float),
    ]


class MocHost(C.Structure):
    _fields_ = [
        ("seg_len", f32p), ("seg_src", i32p), ("az_weight", f32p), ("p_weight", f32p),
        ("z0", f32p), ("polar_angles", f32p), ("src_sigt", i32p), ("src_xs", i32p),
        ("vol", f32p), ("sigt", f32p), ("xs", f32p), ("scatter", f32p),
        ("fine_source", f32p), ("fine_flux", f32p), ("psi_f", f32p), ("psi_b", f32p),
        ("table", f32p),
    ]


class MocGenParams(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("n_materials", C.c_int32), ("n_fuel", C.c_int32),
        ("len_lo", C.c_float), ("len_hi", C.c_float), ("sigt_lo", C.c_float),
        ("sigt_hi", C.c_float), ("scatter_ratio", C.c_float), ("nusf_hi", C.c_float),
        ("siga_ratio", C.c_float), ("vol_lo", C.c_float), ("vol_hi", C.c_float),
        ("axial_z_sep", C.c_float),
    ]


class MocError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _lib().moc_status_string(status).decode() if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


# (name, restype, argtypes) for every exported symbol of the ABI
SIGNATURES = {
    "moc_exp_table_size": (C.c_int32, [C.c_float, C.c_float]),
    "moc_build_exp_table": (C.c_int, [C.c_float, C.c_float, f32p, C.c_int32, f32p, f32p]),
    "moc_generate": (C.c_int, [C.POINTER(MocDims), C.POINTER(MocGenParams), f32p, i32p, f32p,
                               f32p, f32p, f32p, i32p, i32p, f32p, f32p, f32p, f32p, f32p]),
    "moc_create": (C.c_int, [C.POINTER(MocDims), C.POINTER(MocHost), C.c_int,
                             C.POINTER(C.c_void_p)]),
    "moc_destroy": (C.c_int, [C.c_void_p]),
    "moc_upload": (C.c_int, [C.c_void_p, C.POINTER(MocHost)]),
    "moc_download": (C.c_int, [C.c_void_p, f32p, f32p, f32p, f32p]),
    "moc_download64": (C.c_int, [C.c_void_p, f64p, f64p, f64p, f64p]),
    "moc_status": (C.c_int, [C.c_void_p]),
    "moc_status_string": (C.c_char_p, [C.c_int]),
    "moc_device_bytes": (C.c_int64, [C.c_void_p]),
    "moc_set_mode": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "moc_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "moc_get_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "moc_autotune": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_int),
                               f64p]),
    "moc_transport_sweep": (C.c_int, [C.c_void_p, i64p]),
    "moc_renormalize_flux": (C.c_int, [C.c_void_p]),
    "moc_update_sources": (C.c_int, [C.c_void_p, C.c_double, f64p]),
    "moc_compute_keff": (C.c_int, [C.c_void_p, C.c_double, f64p]),
    "moc_power_iteration": (C.c_int, [C.c_void_p, C.c_double, f64p, f64p]),
    "moc_synchronize": (C.c_int, [C.c_void_p]),
    "moc_time_sweep": (C.c_int, [C.c_void_p, C.c_int, f64p]),
    "moc_launch_count": (C.c_int64, [C.c_void_p]),
    "moc_time_power_iterations": (C.c_int, [C.c_void_p, C.c_int, f64p, f64p, f64p, f64p]),
    "moc_set_fine_source_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_set_fine_source64_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_set_sigma_t": (C.c_int, [C.c_void_p, f32p]),
    "moc_zero_state": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "moc_get_fine_flux_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_time_phases": (C.c_int, [C.c_void_p, C.c_int, f64p, f64p, f64p]),
    "moc_fine_flux_storage": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int32)]),
    "moc_get_fine_flux64_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_adjoint_forward": (C.c_int, [C.c_void_p, C.c_int]),
    "moc_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "moc_set_adjoint_width": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "moc_time_adjoint": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, f64p, f64p]),
    "moc_update_sources_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                             C.c_void_p, C.c_void_p, C.c_void_p]),
    "moc_set_cross_sections": (C.c_int, [C.c_void_p, f32p, f32p]),
    "moc_set_fine_flux_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_get_fine_source_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "moc_set_memory_limit": (C.c_int, [C.c_int64]),
    "moc_inject_fault": (C.c_int, [C.c_void_p, C.c_int]),
    "moc_selftest_wait": (C.c_int, [C.c_void_p, C.c_int64]),
    "moc_adjoint_backward_fit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]),
    "moc_set_pipeline": (C.c_int, [C.c_void_p, C.c_int]),
    "moc_get_pipeline": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "moc_openmoc_probe": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64)]),
    "moc_openmoc_read": (C.c_int, [C.c_char_p, C.c_int, C.c_int64, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "moc_batch_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "moc_batch_destroy": (C.c_int, [C.c_void_p]),
    "moc_batch_autotune": (C.c_int, [C.c_void_p]),
    "moc_batch_set_width": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "moc_batch_widths": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "moc_batch_sweep": (C.c_int, [C.c_void_p]),
    "moc_batch_power_iterations": (C.c_int, [C.c_void_p, C.c_int, C.c_int, f64p]),
    "moc_batch_results": (C.c_int, [C.c_void_p, f64p, f64p]),
    "moc_batch_launch_count": (C.c_int64, [C.c_void_p]),
    "moc_renormalize_flux_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_int64, C.c_int32,
                                               C.c_int32, C.c_int64, C.c_void_p, C.c_void_p]),
}

_LIB: C.CDLL | None = None


def _lib() -> C.CDLL:
    """Loads the library once; raises if it is absent (no CPU fallback exists)."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("SIMPLEMOC_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise ImportError(
                f"{path} is not built; run `python -m simplemoc_gb300.build` "
                "(the transport sweep has no CPU fallback)")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def check(status: int, what: str = "") -> None:
    if status != MOC_OK:
        raise MocError(status, what)


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (None stays NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the library must be contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))
