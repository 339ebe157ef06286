"""ORACLE — test infrastructure, not product code.

ctypes driver of oracle/libkhronos_oracle.so, the C++ CPU restatement of the
reference's CPU step loop (oracle/khronos_oracle.cpp).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker.
It consumes the same SimSpec as the CUDA library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "libkhronos_oracle.so"
# The same restatement built with FMA contraction: the timed CPU baseline only
# (its last-bit rounding differs, so parity checks use LIB).
LIB_TIMED = HERE / "libkhronos_oracle_timed.so"

COMPONENT_EXTRA = {0: (0, 1, 1), 1: (1, 0, 1), 2: (1, 1, 0), 3: (1, 0, 0), 4: (0, 1, 0), 5: (0, 0, 1)}


def build(force: bool = False) -> Path:
    src = HERE / "khronos_oracle.cpp"
    stale = any(not p.exists() or p.stat().st_mtime < src.stat().st_mtime for p in (LIB, LIB_TIMED))
    if force or stale:
        r = subprocess.run(["make", "-C", str(HERE), "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


_lib = None
_lib_timed = None


def load(timed: bool = False):
    """The parity build, or (timed=True) the FMA-contracted build used only
    for the timed CPU baseline."""
    global _lib, _lib_timed
    if timed:
        if _lib_timed is None:
            build()
            _lib_timed = _declare(C.CDLL(str(LIB_TIMED)))
        return _lib_timed
    if _lib is None:
        build()
        _lib = _declare(C.CDLL(str(LIB)))
    return _lib


def _declare(lib):
    vp = C.c_void_p
    pd = C.POINTER(C.c_double)
    pi = C.POINTER(C.c_int32)
    lib.khref_create.restype = vp
    lib.khref_create.argtypes = [vp]
    lib.khref_destroy.argtypes = [vp]
    lib.khref_last_error.restype = C.c_char_p
    lib.khref_last_error.argtypes = [vp]
    lib.khref_set_material.argtypes = [vp, C.c_int, C.c_int, pd]
    lib.khref_add_pole.argtypes = [vp, vp, pd]
    lib.khref_add_source.argtypes = [vp, vp]
    lib.khref_add_dft_monitor.argtypes = [vp, C.c_int, pi, pi, C.c_int, pd, C.c_int, pi]
    lib.khref_prepare.argtypes = [vp]
    lib.khref_step.argtypes = [vp, C.c_int64]
    lib.khref_timestep.restype = C.c_int64
    lib.khref_timestep.argtypes = [vp]
    lib.khref_sources_active.argtypes = [vp]
    lib.khref_get_field.argtypes = [vp, C.c_int, pd]
    lib.khref_read_dft.argtypes = [vp, C.c_int, pd]
    lib.khref_num_threads.restype = C.c_int
    return lib


def num_threads() -> int:
    return load().khref_num_threads()


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleSim:
    """CPU oracle run of one SimSpec."""

    def __init__(self, spec, timed: bool = False):
        import importlib

        abi = importlib.import_module("khronos_gb300._abi")
        from khronos_gb300.spec import flat_complex, flat_f

        self.spec = spec
        self.lib = load(timed)
        keep = []
        d = abi.SimDesc()
        for a in range(3):
            d.n[a] = int(spec.n[a])
            d.delta[a] = float(spec.delta[a])
            d.pml_lo[a] = int(spec.pml_lo[a])
            d.pml_hi[a] = int(spec.pml_hi[a])
            for name in ("sigma_b", "sigma_d"):
                arr = getattr(spec, name)[a]
                if arr is not None:
                    h = np.ascontiguousarray(arr, dtype=np.float64)
                    keep.append(h)
                    getattr(d, name)[a] = _dptr(h)
        d.dtype = int(spec.dtype)
        d.dt = float(spec.dt)
        d.eps_inv = float(spec.eps_inv)
        d.mu_inv = float(spec.mu_inv)
        d.semantics = int(spec.semantics)
        d.periodic = int(spec.periodic)
        self.h = C.c_void_p(self.lib.khref_create(C.byref(d)))
        if not self.h:
            raise RuntimeError("oracle create failed")
        mats = list(spec.materials)
        if getattr(spec, "geometry", None) is not None:  # the device rasterises these; restated here
            from .geometry import eps_inv_arrays

            T = np.float32 if spec.dtype == 0 else np.float64
            for c, arr in enumerate(eps_inv_arrays(spec.geometry, spec.n, spec.delta, T)):
                mats.append((0, c, arr.astype(np.float64)))
        for kind, comp, arr in mats:
            h = flat_f(arr)
            self._check(self.lib.khref_set_material(self.h, kind, comp, _dptr(h)))
        for p in spec.poles:
            pc = abi.PoleCoeffs(**p.coeffs)
            h = flat_f(p.sigma)
            self._check(self.lib.khref_add_pole(self.h, C.byref(pc), _dptr(h)))
        for s in spec.sources:
            sd = abi.SourceDesc()
            sd.component = s.component
            for a in range(3):
                sd.start[a] = int(s.start[a])
                sd.dims[a] = int(s.dims[a])
            amp = flat_complex(s.amp)
            sd.amp = _dptr(amp)
            sd.time_kind = s.time_kind
            sd.fcen, sd.width, sd.peak_time, sd.cutoff = s.fcen, s.width, s.peak_time, s.cutoff
            tab = None
            if s.table is not None:
                tab = flat_complex(np.asarray(s.table).reshape(-1))
                sd.table_len = int(np.asarray(s.table).shape[0])
                sd.table = _dptr(tab)
            self._check(self.lib.khref_add_source(self.h, C.byref(sd)))
        self.monitor_ids = []
        for m in spec.monitors:
            st = (C.c_int32 * 3)(*m.start)
            dm = (C.c_int32 * 3)(*m.dims)
            fr = np.ascontiguousarray(m.freqs, dtype=np.float64)
            mid = C.c_int32()
            self._check(self.lib.khref_add_dft_monitor(self.h, m.component, st, dm, len(fr), _dptr(fr),
                                                       int(m.decimation), C.byref(mid)))
            self.monitor_ids.append(mid.value)
        self._check(self.lib.khref_prepare(self.h))

    def _check(self, st):
        if st != 0:
            raise RuntimeError(f"oracle status {st}: {self.lib.khref_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            self.lib.khref_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1):
        self._check(self.lib.khref_step(self.h, int(n)))

    @property
    def timestep(self) -> int:
        return self.lib.khref_timestep(self.h)

    @property
    def sources_active(self) -> bool:
        return bool(self.lib.khref_sources_active(self.h))

    def field(self, comp: int) -> np.ndarray:
        dims = tuple(self.spec.n[a] + COMPONENT_EXTRA[comp][a] for a in range(3))
        out = np.zeros(int(np.prod(dims)), dtype=np.float64)
        self._check(self.lib.khref_get_field(self.h, comp, _dptr(out)))
        return out.reshape(dims, order="F")

    def dft(self, monitor_index: int) -> np.ndarray:
        m = self.spec.monitors[monitor_index]
        cnt = int(np.prod(m.dims)) * len(m.freqs)
        out = np.zeros(2 * cnt, dtype=np.float64)
        self._check(self.lib.khref_read_dft(self.h, self.monitor_ids[monitor_index], _dptr(out)))
        z = out[0::2] + 1j * out[1::2]
        return z.reshape(tuple(m.dims) + (len(m.freqs),), order="F")
