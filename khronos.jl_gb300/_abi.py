"""ctypes binding of libkhronos_gb300.so (the C ABI in include/khronos_gb300.h).

The library is loaded from the package directory; if it is missing the import
fails loudly — there is no CPU fallback for the step loop.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libkhronos_gb300.so"

KH_OK, KH_ERR_INVALID, KH_ERR_OOM, KH_ERR_CUDA, KH_ERR_TIMEOUT, KH_ERR_NAN, KH_ERR_UNSUPPORTED = range(7)
KH_F32, KH_F64 = 0, 1
KH_MAT_EPS_INV, KH_MAT_MU_INV, KH_MAT_SIGMA_D, KH_MAT_SIGMA_B, KH_MAT_CHI3 = range(5)
KH_TIME_GAUSSIAN, KH_TIME_CW, KH_TIME_TABLE = range(3)
KH_SHAPE_BALL, KH_SHAPE_CUBOID, KH_SHAPE_CYLINDER = range(3)
KH_SMOOTH_NONE, KH_SMOOTH_VOLUME, KH_SMOOTH_ANISOTROPIC = range(3)
KH_SEM_REFERENCE_CPU, KH_SEM_CPML = 0, 1
KH_REQ_QUEUED, KH_REQ_ADMITTED, KH_REQ_RUNNING, KH_REQ_DONE, KH_REQ_FAILED, KH_REQ_RELEASED = range(6)

STATUS_NAMES = {
    0: "KH_OK", 1: "KH_ERR_INVALID", 2: "KH_ERR_OOM", 3: "KH_ERR_CUDA",
    4: "KH_ERR_TIMEOUT", 5: "KH_ERR_NAN", 6: "KH_ERR_UNSUPPORTED",
}

D3 = C.c_double * 3
I3 = C.c_int32 * 3
P3 = C.POINTER(C.c_double) * 3


class SimDesc(C.Structure):
    _fields_ = [
        ("n", I3),
        ("dtype", C.c_int32),
        ("delta", D3),
        ("dt", C.c_double),
        ("pml_lo", I3),
        ("pml_hi", I3),
        ("sigma_b", P3),
        ("sigma_d", P3),
        ("eps_inv", C.c_double),
        ("mu_inv", C.c_double),
        ("semantics", C.c_int32),
        ("periodic", C.c_int32),
    ]


class PoleCoeffs(C.Structure):
    _fields_ = [
        ("gamma1_inv", C.c_double),
        ("gamma1", C.c_double),
        ("omega0_dt_sq", C.c_double),
        ("sigma_omega0_dt_sq", C.c_double),
        ("drude_coeff", C.c_double),
        ("is_drude", C.c_int32),
    ]


class SourceDesc(C.Structure):
    _fields_ = [
        ("component", C.c_int32),
        ("start", I3),
        ("dims", I3),
        ("amp", C.POINTER(C.c_double)),
        ("time_kind", C.c_int32),
        ("fcen", C.c_double),
        ("width", C.c_double),
        ("peak_time", C.c_double),
        ("cutoff", C.c_double),
        ("table_len", C.c_int64),
        ("table", C.POINTER(C.c_double)),
    ]


class GeomObject(C.Structure):
    _fields_ = [
        ("shape", C.c_int32),
        ("axis", C.c_int32),
        ("center", D3),
        ("size", D3),
        ("eps", C.c_double),
    ]


class FieldView(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("dtype", C.c_int32),
        ("dims", C.c_int32 * 3),
        ("strides", C.c_int64 * 3),
    ]


class ServerDesc(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_int64),
        ("max_resident", C.c_int32),
        ("quantum_steps", C.c_int32),
    ]


class RequestInfo(C.Structure):
    _fields_ = [
        ("state", C.c_int32),
        ("status", C.c_int32),
        ("steps", C.c_int64),
        ("bytes", C.c_int64),
        ("t_submit", C.c_double),
        ("t_admit", C.c_double),
        ("t_start", C.c_double),
        ("t_done", C.c_double),
    ]


# Every exported symbol with its ctypes signature: (restype, argtypes).
SIGNATURES = {
    "kh_version": (C.c_char_p, []),
    "kh_device_info": (C.c_int32, [C.POINTER(C.c_int32)] * 3),
    "kh_sim_create": (C.c_int32, [C.POINTER(SimDesc), C.POINTER(C.c_void_p)]),
    "kh_sim_destroy": (None, [C.c_void_p]),
    "kh_last_error": (C.c_char_p, [C.c_void_p]),
    "kh_sim_set_material": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "kh_sim_attach_material": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32]),
    "kh_device_alloc_count": (C.c_int32, [C.POINTER(C.c_int64)]),
    "kh_sim_add_pole": (C.c_int32, [C.c_void_p, C.POINTER(PoleCoeffs), C.POINTER(C.c_double)]),
    "kh_sim_add_source": (C.c_int32, [C.c_void_p, C.POINTER(SourceDesc)]),
    "kh_sim_add_dft_monitor": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.c_int32, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32)]),
    "kh_sim_prepare": (C.c_int32, [C.c_void_p]),
    "kh_sim_step": (C.c_int32, [C.c_void_p, C.c_int64, C.c_void_p]),
    "kh_sim_synchronize": (C.c_int32, [C.c_void_p]),
    "kh_sim_timestep": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "kh_sim_sources_active": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32)]),
    "kh_sim_launch_count": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "kh_sim_set_geometry": (C.c_int32, [C.c_void_p, C.POINTER(GeomObject), C.c_int32, C.c_double,
                                        C.POINTER(C.c_double), C.c_int32]),
    "kh_sim_read_material": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "kh_sim_graph_replays": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "kh_sim_get_field": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "kh_sim_read_dft": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "kh_sim_monitor_info": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "kh_sim_flux": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_double, C.POINTER(C.c_double)]),
    "kh_sim_flux_static": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_double,
                                       C.POINTER(C.c_double)]),
    "kh_sim_reset": (C.c_int32, [C.c_void_p]),
    "kh_sim_state_bytes": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "kh_sim_export_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64]),
    "kh_sim_import_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64]),
    "kh_sim_model_bytes_per_step": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double)]),
    "kh_sim_model_bytes_split": (C.c_int32, [C.c_void_p] + [C.POINTER(C.c_double)] * 3),
    "kh_sim_step_timed": (C.c_int32, [C.c_void_p, C.c_int64, C.c_void_p] + [C.POINTER(C.c_double)] * 3),
    "kh_sim_memory_bytes": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "kh_sim_update_material_box": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                               C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "kh_sim_update_source": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64,
                                         C.POINTER(C.c_double), C.c_double]),
    "kh_sim_dft_overlap": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "kh_adjoint_accumulate": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_void_p,
                                          C.POINTER(C.c_int32), C.c_int32, C.c_double, C.c_double,
                                          C.POINTER(C.c_double)]),
    "kh_sim_add_history_monitor": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                               C.c_int64, C.POINTER(C.c_int32)]),
    "kh_sim_read_history": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)]),
    "kh_history_correlate": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32),
                                         C.c_int64, C.c_double, C.POINTER(C.c_double)]),
    "kh_sim_field_sq_norms": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double)]),
    "kh_sim_check_finite": (C.c_int32, [C.c_void_p]),
    "kh_debug_bounds": (C.c_int32, [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "kh_sim_dft_norms": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double)]),
    "kh_sim_field_view": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(FieldView)]),
    "kh_server_create": (C.c_int32, [C.POINTER(ServerDesc), C.POINTER(C.c_void_p)]),
    "kh_server_submit": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "kh_server_wait": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double]),
    "kh_server_wait_any": (C.c_int32, [C.c_void_p, C.c_double, C.POINTER(C.c_int64)]),
    "kh_server_info": (C.c_int32, [C.c_void_p, C.c_int64, C.POINTER(RequestInfo)]),
    "kh_server_release": (C.c_int32, [C.c_void_p, C.c_int64]),
    "kh_server_stats": (C.c_int32, [C.c_void_p] + [C.POINTER(C.c_int64)] * 3),
    "kh_server_last_error": (C.c_char_p, [C.c_void_p]),
    "kh_server_destroy": (None, [C.c_void_p]),
}

_lib = None


def load(path: Path | None = None):
    """Load the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()'). "
            "The FDTD step loop has no CPU fallback."
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class KhError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int, lib, handle) -> None:
    if status != KH_OK:
        msg = lib.kh_last_error(handle).decode() if handle else ""
        raise KhError(status, msg)
