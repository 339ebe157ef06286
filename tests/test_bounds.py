"""The bounds-checked build (KH_DEBUG_BOUNDS) as a stand-in for a memory
sanitizer: every global and shared-memory index of the step kernels is tested
against its array's extent, and a violating access is recorded and skipped.
Small odd-sized grids through every kernel variant (TMA and register-pipelined
half-steps, LEAN and FULL, both CPML semantics, FP32 and FP64, sources in
and out of CPML, χ3, poles, z tilings, DFT decimation, history recording)
must record no violation and give the regular build's results: bit for bit
on the TMA path, within rounding where the compiler may contract a different
set of multiply-adds in the checked code (FP32 ≤ 1e-5, FP64 ≤ 1e-12 relative
L2)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import _odd_sim


@pytest.fixture(scope="module")
def bounds_lib():
    from khronos_gb300 import _abi, build

    return _abi.load(build.build(bounds=True))


def _violations(lib):
    c, i, s = C.c_int64(), C.c_int64(), C.c_int32()
    assert lib.kh_debug_bounds(C.byref(c), C.byref(i), C.byref(s)) == 0
    return c.value, i.value, s.value


def _run(spec, lib, chunks):
    from khronos_gb300.device import GpuSim

    g = GpuSim(spec, lib=lib)
    for n in chunks:
        g.step(n)
    out = [g.field(c) for c in range(6)] + [g.dft(m) for m in range(len(spec.monitors))]
    for h, hs in enumerate(spec.histories):
        out += [g.history(h, s) for s in (0, min(hs.capacity, sum(chunks)) - 1)]
    g.close()
    return out


def _same(spec, gpu_lib, bounds_lib, chunks=(7, 40, 13), exact=True):
    _violations(bounds_lib)  # clear
    ref = _run(spec, gpu_lib, chunks)
    got = _run(spec, bounds_lib, chunks)
    count, index, site = _violations(bounds_lib)
    assert count == 0, f"{count} out-of-range accesses, first at site {site} index {index}"
    tol = 1e-5 if spec.dtype == 0 else 1e-12
    for a, b in zip(ref, got):
        if exact:
            assert np.array_equal(a, b)
        else:
            assert rel_l2(a, b) <= tol


pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["tma", "simt"])
@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_odd_grid_all_paths(kh, gpu_lib, bounds_lib, monkeypatch, kernel, semantics, dtype):
    if kernel == "simt":
        monkeypatch.setenv("KHRONOS_GB300_KERNEL", "simt")
    from khronos_gb300.spec import HistorySpec

    sp = _odd_sim(kh, semantics, dtype).spec()
    sp.histories.append(HistorySpec(component=kh.EY, start=(3, 0, 5), dims=(35, 23, 1), capacity=50))
    sp.histories.append(HistorySpec(component=kh.HZ, start=(0, 2, 0), dims=(5, 3, 20), capacity=9))
    _same(sp, gpu_lib, bounds_lib, chunks=(7, 25, 8) if semantics == "reference_cpu" else (7, 40, 13),
          exact=kernel == "tma")


@pytest.mark.parametrize("boundaries", [None, ((0.5, 0.5), (0, 0), (0, 0)), ((0, 0), (0, 0), (0.3, 0.0))])
def test_partial_or_no_pml(kh, gpu_lib, bounds_lib, boundaries):
    _same(_odd_sim(kh, "cpml", "f64", boundaries=boundaries).spec(), gpu_lib, bounds_lib)


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_source_in_cpml_full_kernel(kh, gpu_lib, bounds_lib, semantics):
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3), component=kh.EX,
                           center=(-1.05, 0.1, 0.0), size=(0, 0.8, 0.6))
    mon = kh.DFTMonitor(component=kh.EY, center=(0.3, 0, 0), size=(0, 1.0, 1.0), frequencies=[0.8])
    sim = kh.Simulation(cell_size=(2.7, 2.1, 1.7), resolution=10, sources=[src], monitors=[mon],
                        boundaries=[[0.4, 0.4]] * 3, dtype="f64", semantics=semantics)
    _same(sim.spec(), gpu_lib, bounds_lib, chunks=(9, 20))


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_dispersive_and_kerr(kh, gpu_lib, bounds_lib, dtype):
    from khronos_gb300 import configs

    _same(configs.dispersive(dtype=dtype, scale=0.25).sim.spec(), gpu_lib, bounds_lib, chunks=(5, 30))


@pytest.mark.parametrize("zplanes", ["1", "7", "64"])
def test_z_tilings(kh, gpu_lib, bounds_lib, monkeypatch, zplanes):
    from khronos_gb300 import configs

    monkeypatch.setenv("KHRONOS_GB300_ZPLANES", zplanes)
    sp = configs.waveguide(dtype="f32", scale=0.25).sim.spec()
    _same(sp, gpu_lib, bounds_lib, chunks=(3, 31))
