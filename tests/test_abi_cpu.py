"""The C-ABI library builds, loads without a GPU and exports every symbol the
header declares; argument validation needs no device."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "khronos_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kh_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("kh_sim_create", "kh_sim_step", "kh_sim_get_field", "kh_sim_read_dft", "kh_sim_flux",
                     "kh_sim_destroy", "kh_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(gpu_lib):
    from khronos_gb300 import _abi

    for name in declared_functions():
        assert hasattr(gpu_lib, name), name
        assert name in _abi.SIGNATURES, name
    assert gpu_lib.kh_version().decode().startswith("khronos_gb300")


def test_invalid_arguments_without_a_gpu(gpu_lib):
    from khronos_gb300 import _abi

    d = _abi.SimDesc()
    h = C.c_void_p()
    assert gpu_lib.kh_sim_create(C.byref(d), C.byref(h)) == _abi.KH_ERR_INVALID  # zero-size grid
    assert gpu_lib.kh_sim_create(None, C.byref(h)) == _abi.KH_ERR_INVALID
    d.n[0], d.n[1], d.n[2] = 8, 8, 8
    d.dtype = 7
    d.delta[0] = d.delta[1] = d.delta[2] = 0.1
    d.dt = 0.05
    assert gpu_lib.kh_sim_create(C.byref(d), C.byref(h)) == _abi.KH_ERR_INVALID  # bad dtype
    d.dtype = _abi.KH_F32
    assert gpu_lib.kh_sim_create(C.byref(d), C.byref(h)) == _abi.KH_OK
    try:
        # set-up calls are host-only
        vals = (C.c_double * 512)(*([1.0] * 512))
        assert gpu_lib.kh_sim_set_material(h, 99, 0, vals) == _abi.KH_ERR_INVALID
        assert gpu_lib.kh_sim_set_material(h, _abi.KH_MAT_EPS_INV, 5, vals) == _abi.KH_ERR_INVALID
        assert gpu_lib.kh_sim_set_material(h, _abi.KH_MAT_EPS_INV, 0, vals) == _abi.KH_OK
        st = (C.c_int32 * 3)(0, 0, 0)
        dm = (C.c_int32 * 3)(20, 1, 1)  # beyond the grid
        fr = (C.c_double * 1)(1.0)
        mid = C.c_int32()
        assert gpu_lib.kh_sim_add_dft_monitor(h, 0, st, dm, 1, fr, 1, C.byref(mid)) == _abi.KH_ERR_INVALID
        assert b"outside" in gpu_lib.kh_last_error(h)
        assert gpu_lib.kh_sim_step(h, 1, None) == _abi.KH_ERR_INVALID  # before prepare
        ts = C.c_int64(-1)
        assert gpu_lib.kh_sim_timestep(h, C.byref(ts)) == _abi.KH_OK and ts.value == 0
    finally:
        gpu_lib.kh_sim_destroy(h)


def test_missing_library_fails_loudly(tmp_path):
    from khronos_gb300 import _abi

    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _abi.load(tmp_path / "libkhronos_gb300.so")


def test_regular_build_has_no_bounds_record(gpu_lib):
    """kh_debug_bounds answers KH_ERR_UNSUPPORTED outside the bounds-checked
    build (no device work)."""
    import ctypes as C

    from khronos_gb300 import _abi

    c, i, s = C.c_int64(7), C.c_int64(7), C.c_int32(7)
    assert gpu_lib.kh_debug_bounds(C.byref(c), C.byref(i), C.byref(s)) == _abi.KH_ERR_UNSUPPORTED
    assert (c.value, i.value, s.value) == (0, 0, 0)
