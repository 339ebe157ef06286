"""CUDA step loop against the CPU oracle at the benchmark configurations as
stated (not scaled down), through the C ABI.

* 3-D point dipole in vacuum, 64×64×64 with a 10-cell CPML, 1000 steps: FP64
  fields (six components) and all twelve DFT arrays of the x-normal flux plane
  (Ey, Ez, Hy, Hz × 3 frequencies) within 1e-10 relative L2, in both CPML
  semantics.  With the reference CPU path's stage dispatch the fields grow by
  ~10²⁹ per 100 steps from step ~70 on (the dropped σ_prev stage,
  Helpers.jl:208-223) but stay finite in FP64 through step 1000, so that
  semantics is compared over the whole run too, on rescaled norms.  FP32
  within 2e-4 (CUDA-path semantics; FP32 overflows on the growing CPU path).
* heterogeneous waveguide, 320×192×128 with a 12-cell CPML, FP64, 200 steps
  (source active, six DFT updates; 100 steps with the CPU-path stages):
  fields and DFT arrays within 1e-10.
* dispersive + Kerr grid, 256×256×256 with a 12-cell CPML (χ3 slab, Lorentz
  and Drude spheres), FP64, 200 steps: fields and DFT arrays within 1e-10.

Errors are normalised as in test_gpu_parity (whole E or H field; largest
monitor norm).
"""
import numpy as np
import pytest

from conftest import dft_errors, field_errors

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-10, "f32": 2e-4}


def _compare(spec, steps, oracle, gpu_lib, tol):
    from khronos_gb300.device import GpuSim

    gpu = GpuSim(spec, lib=gpu_lib)
    gpu.step(steps)
    fa = [gpu.field(c) for c in range(6)]
    da = [gpu.dft(m) for m in range(len(spec.monitors))]
    ts, sa = gpu.timestep, gpu.sources_active
    gpu.close()
    ref = oracle.OracleSim(spec)
    ref.step(steps)
    fb = [ref.field(c) for c in range(6)]
    db = [ref.dft(m) for m in range(len(spec.monitors))]
    assert (ts, sa) == (ref.timestep, ref.sources_active)
    ref.close()
    for c in range(6):
        assert np.all(np.isfinite(fb[c]))
    worst = {f"field{c}": e for c, e in enumerate(field_errors(fa, fb))}
    worst.update({f"dft{m}": e for m, e in enumerate(dft_errors(da, db))})
    bad = {k: v for k, v in worst.items() if not v <= tol}
    assert not bad, f"relative L2 above {tol}: {bad}"
    return worst


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_dipole_64_cubed_fp64_1000_steps(kh, oracle, gpu_lib, semantics):
    from khronos_gb300 import configs

    w = configs.dipole(dtype="f64", steps=1000)
    w.sim.semantics = semantics
    spec = w.sim.spec()
    assert tuple(spec.n) == (64, 64, 64) and len(spec.monitors) == 4
    assert sum(len(m.freqs) for m in spec.monitors) == 12
    _compare(spec, 1000, oracle, gpu_lib, TOL["f64"])


def test_dipole_64_cubed_fp32_1000_steps(kh, oracle, gpu_lib):
    from khronos_gb300 import configs

    w = configs.dipole(dtype="f32", steps=1000)
    _compare(w.sim.spec(), 1000, oracle, gpu_lib, TOL["f32"])


# The CPU-path semantics is compared over 100 steps: its CPML grows from step
# ~70 on, and by step 200 the growth has amplified last-bit differences (FMA
# contraction on the device, none in the oracle) to 2.4e-10 on Ey and Hx.
@pytest.mark.parametrize("semantics,steps", [("cpml", 200), ("reference_cpu", 100)])
def test_waveguide_full_size_fp64(kh, oracle, gpu_lib, semantics, steps):
    from khronos_gb300 import configs

    w = configs.waveguide(dtype="f64")
    w.sim.semantics = semantics
    spec = w.sim.spec()
    assert tuple(spec.n) == (320, 192, 128)
    _compare(spec, steps, oracle, gpu_lib, TOL["f64"])


def test_dispersive_full_size_fp64_200_steps(kh, oracle, gpu_lib):
    from khronos_gb300 import configs

    w = configs.dispersive(dtype="f64")
    spec = w.sim.spec()
    assert tuple(spec.n) == (256, 256, 256) and spec.poles and any(k == 4 for k, _, _ in spec.materials)
    _compare(spec, 200, oracle, gpu_lib, TOL["f64"])
