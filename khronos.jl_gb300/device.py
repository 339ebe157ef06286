"""GpuSim: one SimSpec realised as a kh_sim handle of libkhronos_gb300.so."""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _abi
from .grid import COMPONENT_EXTRA
from .spec import SimSpec, flat_complex, flat_f


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _material_array(a: np.ndarray):
    """A cell-indexed material array as the library reads it: x fastest,
    contiguous, float32 or float64 kept as given (no copy when it already is,
    e.g. a Fortran-ordered float32 array in pinned memory), with its KH_F* tag."""
    a = np.asarray(a)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    flat = a.ravel(order="F")
    return flat, (_abi.KH_F32 if flat.dtype == np.float32 else _abi.KH_F64)


class GpuSim:
    """Device-resident simulation driven through the C ABI."""

    def __init__(self, spec: SimSpec, lib=None, prepare: bool = True):
        self.spec = spec
        self.lib = lib or _abi.load()
        self.handle = C.c_void_p()
        self._keep = []  # host arrays referenced by the descriptor during creation
        d = _abi.SimDesc()
        for a in range(3):
            d.n[a] = int(spec.n[a])
            d.delta[a] = float(spec.delta[a])
            d.pml_lo[a] = int(spec.pml_lo[a])
            d.pml_hi[a] = int(spec.pml_hi[a])
            for name in ("sigma_b", "sigma_d"):
                arr = getattr(spec, name)[a]
                if arr is not None:
                    h = np.ascontiguousarray(arr, dtype=np.float64)
                    self._keep.append(h)
                    getattr(d, name)[a] = _dptr(h)
        d.dtype = int(spec.dtype)
        d.dt = float(spec.dt)
        d.eps_inv = float(spec.eps_inv)
        d.mu_inv = float(spec.mu_inv)
        d.semantics = int(spec.semantics)
        d.periodic = int(spec.periodic)
        self._check(self.lib.kh_sim_create(C.byref(d), C.byref(self.handle)))
        # material arrays the library reads at prepare (kh_sim_attach_material);
        # held until then (for a request server, until the simulation is released)
        self._materials = []
        try:
            for kind, comp, arr in spec.materials:
                h, dt = _material_array(arr)
                self._materials.append(h)
                self._check(self.lib.kh_sim_attach_material(self.handle, kind, comp, h.ctypes.data, dt))
            for p in spec.poles:
                pc = _abi.PoleCoeffs(**p.coeffs)
                h = flat_f(p.sigma)
                self._check(self.lib.kh_sim_add_pole(self.handle, C.byref(pc), _dptr(h)))
            for s in spec.sources:
                sd = _abi.SourceDesc()
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
                self._check(self.lib.kh_sim_add_source(self.handle, C.byref(sd)))
            self.monitor_ids: List[int] = []
            for m in spec.monitors:
                st = (C.c_int32 * 3)(*m.start)
                dm = (C.c_int32 * 3)(*m.dims)
                fr = np.ascontiguousarray(m.freqs, dtype=np.float64)
                mid = C.c_int32()
                self._check(self.lib.kh_sim_add_dft_monitor(self.handle, m.component, st, dm, len(fr),
                                                            _dptr(fr), int(m.decimation), C.byref(mid)))
                self.monitor_ids.append(mid.value)
            if spec.geometry is not None:
                g = spec.geometry
                objs = (_abi.GeomObject * max(1, len(g.objects)))()
                for q, (shape, axis, c, sz, eps) in enumerate(g.objects):
                    objs[q].shape, objs[q].axis, objs[q].eps = shape, axis, eps
                    for a in range(3):
                        objs[q].center[a] = c[a]
                        objs[q].size[a] = sz[a]
                org = (C.c_double * 3)(*g.origin)
                self._check(self.lib.kh_sim_set_geometry(self.handle, objs, len(g.objects), float(g.background),
                                                         org, int(g.smoothing)))
            self.history_ids: List[int] = []
            for h in spec.histories:
                st = (C.c_int32 * 3)(*h.start)
                dm = (C.c_int32 * 3)(*h.dims)
                hid = C.c_int32()
                self._check(self.lib.kh_sim_add_history_monitor(self.handle, h.component, st, dm,
                                                                int(h.capacity), C.byref(hid)))
                self.history_ids.append(hid.value)
            if prepare:
                self._check(self.lib.kh_sim_prepare(self.handle))
                self._materials = []
        except Exception:
            self.close()
            raise
        self._keep.clear()

    def _check(self, st):
        _abi.check(st, self.lib, self.handle)

    def close(self):
        if self.handle:
            if not getattr(self, "_detached", False):
                self.lib.kh_sim_destroy(self.handle)
            self.handle = C.c_void_p()

    def detach(self):
        """Hand the handle's ownership to another owner (a request server):
        close() no longer destroys it."""
        self._detached = True

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping ---------------------------------------------------------
    def step(self, nsteps: int = 1, stream: Optional[int] = None):
        self._check(self.lib.kh_sim_step(self.handle, int(nsteps), C.c_void_p(stream) if stream else None))

    def synchronize(self):
        self._check(self.lib.kh_sim_synchronize(self.handle))

    @property
    def timestep(self) -> int:
        v = C.c_int64()
        self._check(self.lib.kh_sim_timestep(self.handle, C.byref(v)))
        return v.value

    @property
    def sources_active(self) -> bool:
        v = C.c_int32()
        self._check(self.lib.kh_sim_sources_active(self.handle, C.byref(v)))
        return bool(v.value)

    @property
    def launches(self) -> int:
        v = C.c_int64()
        self._check(self.lib.kh_sim_launch_count(self.handle, C.byref(v)))
        return v.value

    @property
    def graph_replays(self) -> int:
        v = C.c_int64()
        self._check(self.lib.kh_sim_graph_replays(self.handle, C.byref(v)))
        return v.value

    # -- results ------------------------------------------------------------
    def field(self, comp: int) -> np.ndarray:
        """Component array in the reference's component dimensions, indexed [i, j, k]."""
        dims = tuple(self.spec.n[a] + COMPONENT_EXTRA[comp][a] for a in range(3))
        out = np.zeros(int(np.prod(dims)), dtype=np.float64)
        self._check(self.lib.kh_sim_get_field(self.handle, comp, _dptr(out)))
        return out.reshape(dims, order="F")

    def field_view(self, comp: int, ghosted: bool = False):
        """Component `comp` in place on the device as a torch tensor indexed
        [i, j, k] (no copy; strided over the padded layout).  Its values are
        current after synchronize(); it keeps this simulation from being
        garbage-collected, and is invalid after close().

        ``ghosted=True`` starts the view at the (−1, −1, −1) ghost cell, one
        more cell per axis: the reference's raw field layout with the ghost at
        index 0 and the interior at 1..N (Fields.jl:130-141; readers take
        2:N+1 in Julia's 1-based indexing, Visualization.jl:296-302)."""
        import torch

        v = _abi.FieldView()
        self._check(self.lib.kh_sim_field_view(self.handle, comp, C.byref(v)))
        item = 4 if v.dtype == _abi.KH_F32 else 8
        if ghosted:
            v.data = int(v.data) - item * int(v.strides[0] + v.strides[1] + v.strides[2])
            for a in range(3):
                v.dims[a] += 1

        class _Holder:
            pass

        h = _Holder()
        h.sim = self
        h.__cuda_array_interface__ = {
            "shape": tuple(int(d) for d in v.dims),
            "typestr": "<f4" if item == 4 else "<f8",
            "strides": tuple(int(s) * item for s in v.strides),
            "data": (int(v.data), False),
            "version": 2,
        }
        return torch.as_tensor(h, device=torch.device("cuda", torch.cuda.current_device()))

    def dft(self, monitor_index: int) -> np.ndarray:
        """DFT accumulator of a monitor, shape (Nx, Ny, Nz, Nf), complex128."""
        m = self.spec.monitors[monitor_index]
        cnt = int(np.prod(m.dims)) * len(m.freqs)
        z = np.empty(cnt, dtype=np.complex128)  # interleaved (re, im) doubles
        self._check(self.lib.kh_sim_read_dft(self.handle, self.monitor_ids[monitor_index],
                                             z.ctypes.data_as(C.POINTER(C.c_double))))
        return z.reshape(tuple(m.dims) + (len(m.freqs),), order="F")

    def flux(self, monitor_indices: Sequence[int], normal_axis: int, dA: float) -> np.ndarray:
        ids = (C.c_int32 * 4)(*[self.monitor_ids[i] for i in monitor_indices])
        nf = len(self.spec.monitors[monitor_indices[0]].freqs)
        out = np.zeros(nf, dtype=np.float64)
        self._check(self.lib.kh_sim_flux(self.handle, ids, int(normal_axis), float(dA), _dptr(out)))
        return out

    def model_bytes_per_step(self) -> float:
        v = C.c_double()
        self._check(self.lib.kh_sim_model_bytes_per_step(self.handle, C.byref(v)))
        return v.value

    def model_bytes_split(self):
        """(H half-step, E half-step, DFT) model bytes of one step."""
        h, e, d = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.kh_sim_model_bytes_split(self.handle, C.byref(h), C.byref(e), C.byref(d)))
        return h.value, e.value, d.value

    def step_timed(self, nsteps: int, stream: Optional[int] = None):
        """Step with CUDA events around every launch; returns (H ms, E ms, DFT ms) summed."""
        h, e, d = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.kh_sim_step_timed(self.handle, int(nsteps), C.c_void_p(stream) if stream else None,
                                               C.byref(h), C.byref(e), C.byref(d)))
        return h.value, e.value, d.value

    def material(self, kind: int, comp: int) -> np.ndarray:
        """A per-voxel material array (Center range), indexed [i, j, k]."""
        out = np.zeros(int(np.prod(self.spec.n)))
        self._check(self.lib.kh_sim_read_material(self.handle, int(kind), int(comp), _dptr(out)))
        return out.reshape(tuple(self.spec.n), order="F")

    def field_sq_norms(self) -> np.ndarray:
        """Σ E_c², Σ H_c² over the grid (6 values, FP64 on the device)."""
        out = np.zeros(6)
        self._check(self.lib.kh_sim_field_sq_norms(self.handle, _dptr(out)))
        return out

    def dft_norms(self) -> np.ndarray:
        """sqrt(Σ|F|²) of every DFT monitor of the spec (in spec order), FP64 on the device."""
        out = np.zeros(max(1, max(self.monitor_ids, default=0) + 1))
        self._check(self.lib.kh_sim_dft_norms(self.handle, _dptr(out)))
        return np.array([out[m] for m in self.monitor_ids])

    def check_finite(self) -> None:
        """Raise KhronosError(KH_ERR_NAN) once any field value is non-finite."""
        self._check(self.lib.kh_sim_check_finite(self.handle))

    # -- adjoint support -------------------------------------------------------
    def update_material_box(self, kind: int, comp: int, start, values: np.ndarray):
        """Overwrite per-voxel ε⁻¹/μ⁻¹ of one component over the cell box
        start..start+values.shape-1 (values indexed [i, j, k])."""
        v = flat_f(values)
        st = (C.c_int32 * 3)(*[int(s) for s in start])
        dm = (C.c_int32 * 3)(*[int(d) for d in np.shape(values)])
        self._check(self.lib.kh_sim_update_material_box(self.handle, int(kind), int(comp), st, dm, _dptr(v)))

    def update_source(self, index: int, amp: Optional[np.ndarray] = None, table: Optional[np.ndarray] = None,
                      cutoff: float = 0.0):
        """Replace source ``index``'s amplitude array (same footprint) and/or
        its time table ((steps, 2) complex: f(nΔt), f(nΔt + Δt/2))."""
        a = flat_complex(amp) if amp is not None else None
        t = flat_complex(np.asarray(table).reshape(-1)) if table is not None else None
        n = int(np.asarray(table).shape[0]) if table is not None else 0
        self._check(self.lib.kh_sim_update_source(self.handle, int(index), _dptr(a) if a is not None else None,
                                                  n, _dptr(t) if t is not None else None, float(cutoff)))

    def dft_overlap(self, monitor_index: int, weights: np.ndarray) -> np.ndarray:
        """Σ_cells weights·F per frequency, FP64 on the device; weights has the
        monitor's DFT shape (Nx, Ny, Nz, Nf)."""
        m = self.spec.monitors[monitor_index]
        shape = tuple(m.dims) + (len(m.freqs),)
        w = np.asarray(weights, dtype=np.complex128)
        if w.shape != shape:
            raise ValueError(f"weights shape {w.shape} != monitor shape {shape}")
        wf = flat_complex(w)
        out = np.zeros(2 * len(m.freqs))
        self._check(self.lib.kh_sim_dft_overlap(self.handle, self.monitor_ids[monitor_index], _dptr(wf), _dptr(out)))
        return out[0::2] + 1j * out[1::2]

    def adjoint_accumulate(self, fwd_monitors, fwd_freq: int, adj: "GpuSim", adj_monitors, adj_freq: int,
                           coef: complex, grad: np.ndarray):
        """grad += Re(coef·Σ_c F_c·A_c) per design voxel (FP64 on the device);
        grad is a float64 array over the design box, indexed [i, j, k]."""
        fi = (C.c_int32 * 3)(*[self.monitor_ids[i] for i in fwd_monitors])
        ai = (C.c_int32 * 3)(*[adj.monitor_ids[i] for i in adj_monitors])
        flat = np.ascontiguousarray(grad.ravel(order="F"))
        self._check(self.lib.kh_adjoint_accumulate(self.handle, fi, int(fwd_freq), adj.handle, ai, int(adj_freq),
                                                   float(np.real(coef)), float(np.imag(coef)), _dptr(flat)))
        grad[...] = flat.reshape(grad.shape, order="F")

    def history(self, index: int, step: int) -> np.ndarray:
        """Recorded values of history monitor ``index`` at ``step``, indexed [i, j, k]."""
        h = self.spec.histories[index]
        out = np.zeros(int(np.prod(h.dims)))
        self._check(self.lib.kh_sim_read_history(self.handle, self.history_ids[index], int(step), _dptr(out)))
        return out.reshape(tuple(h.dims), order="F")

    def history_correlate(self, fwd_histories, adj: "GpuSim", adj_histories, nsteps: int, coef: float,
                          grad: np.ndarray):
        """grad += coef·Σ_c Σ_m F_c[m]·A_c[N−1−m] per box cell (FP64 on the device)."""
        fi = (C.c_int32 * 3)(*[self.history_ids[i] for i in fwd_histories])
        ai = (C.c_int32 * 3)(*[adj.history_ids[i] for i in adj_histories])
        flat = np.ascontiguousarray(grad.ravel(order="F"))
        self._check(self.lib.kh_history_correlate(self.handle, fi, adj.handle, ai, int(nsteps), float(coef),
                                                  _dptr(flat)))
        grad[...] = flat.reshape(grad.shape, order="F")

    # -- state ----------------------------------------------------------------
    def reset(self):
        self._check(self.lib.kh_sim_reset(self.handle))

    def export_state(self) -> bytes:
        n = C.c_int64()
        self._check(self.lib.kh_sim_state_bytes(self.handle, C.byref(n)))
        buf = (C.c_char * n.value)()
        self._check(self.lib.kh_sim_export_state(self.handle, buf, n.value))
        return bytes(buf)

    def import_state(self, data: bytes):
        buf = (C.c_char * len(data)).from_buffer_copy(data)
        self._check(self.lib.kh_sim_import_state(self.handle, buf, len(data)))
