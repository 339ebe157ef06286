"""FP32 production path (bulk FP32, Kahan-compensated DFT, FP64 flux
reduction) against full-FP64 runs of the same inputs: flux spectra within
1e-4 relative L2.

The FP64 run is the FP32 run's spec promoted (`SimSpec.promoted`): the same
cell indices, monitor boxes and FP32-rounded input values, computed in FP64.
(Specs built directly in FP64 place grid volumes with FP64 index arithmetic,
which can move a flux plane by one cell, so they measure a different plane.)

* point dipole 64³, 1000 steps: FP32 GPU against the FP64 oracle;
* Si-strip waveguide at half resolution (160×96×64), the full physical run
  (2000 steps): FP32 GPU against the FP64 oracle;
* the same waveguide at full size (320×192×128, 4000 steps): FP32 GPU
  against the FP64 oracle (about 3·10¹⁰ cell-updates on the host cores).
"""
import pytest

pytestmark = pytest.mark.gpu

FLUX_TOL = 1e-4


def _gpu_fluxes(w, steps, gpu_lib, promote=False):
    from khronos_gb300.device import GpuSim

    sp = w.sim.spec()
    if promote:
        sp = sp.promoted()
    g = GpuSim(sp, lib=gpu_lib)
    g.step(steps)
    out, base = [], 0
    for fm in w.flux_monitors:
        out.append(g.flux(list(range(base, base + 4)), fm.normal_axis, fm.dA))
        base += 4
    g.close()
    return out


def _oracle_fluxes(w, steps, oracle):
    from khronos_gb300.monitors import flux_from_dft

    sp = w.sim.spec().promoted()
    r = oracle.OracleSim(sp)
    r.step(steps)
    out, base = [], 0
    for fm in w.flux_monitors:
        out.append(flux_from_dft(fm.normal_axis, *[r.dft(i) for i in range(base, base + 4)], fm.dA))
        base += 4
    r.close()
    return out


def _check(test, ref):
    from khronos_gb300.monitors import flux_error

    errs = [flux_error(a, b) for a, b in zip(test, ref)]
    worst = max(e["rel_l2"] for e in errs)
    assert worst <= FLUX_TOL, errs
    return errs


def test_dipole_fp32_flux_vs_fp64_oracle(kh, oracle, gpu_lib):
    from khronos_gb300 import configs

    w32 = configs.dipole(dtype="f32")
    assert tuple(w32.sim.spec().n) == (64, 64, 64)
    _check(_gpu_fluxes(w32, 1000, gpu_lib), _oracle_fluxes(w32, 1000, oracle))


def test_waveguide_half_resolution_fp32_flux_vs_fp64_oracle(kh, oracle, gpu_lib):
    from khronos_gb300 import configs

    w32 = configs.waveguide(dtype="f32", scale=0.5)
    _check(_gpu_fluxes(w32, 2000, gpu_lib), _oracle_fluxes(w32, 2000, oracle))


def test_waveguide_full_size_fp32_flux_vs_fp64_oracle(kh, oracle, gpu_lib):
    from khronos_gb300 import configs

    w32 = configs.waveguide(dtype="f32")
    assert tuple(w32.sim.spec().n) == (320, 192, 128)
    _check(_gpu_fluxes(w32, 4000, gpu_lib), _oracle_fluxes(w32, 4000, oracle))
