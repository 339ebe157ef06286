"""Divergence detection: kh_sim_check_finite reports KH_ERR_NAN once a run
has blown up.  The blow-up is made by the physics, never by a fault: the
time step is doubled past the Courant limit dt ≤ Δ/(c√3), so the Yee
recurrence has eigenvalues outside the unit circle and grows each step until
it overflows (FP32 by step ~50, FP64 by step ~320 on the 32³ dipole)."""
import dataclasses

import numpy as np
import pytest


def _unstable_spec(dtype):
    from khronos_gb300 import configs

    w = configs.dipole(dtype=dtype, resolution=10)
    sp = w.sim.spec()
    return sp, dataclasses.replace(sp, dt=2.0 * sp.dt)


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_oracle_diverges_above_courant_limit(kh, oracle, dtype):
    """The premise of the GPU test, on the CPU: the stable spec stays finite
    and the doubled step overflows within 400 steps."""
    stable, unstable = _unstable_spec(dtype)
    a = oracle.OracleSim(stable)
    b = oracle.OracleSim(unstable)
    a.step(400)
    b.step(400)
    assert all(np.all(np.isfinite(a.field(c))) for c in range(6))
    assert not all(np.all(np.isfinite(b.field(c))) for c in range(6))
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_check_finite_reports_divergence(kh, gpu_lib, dtype):
    from khronos_gb300 import _abi
    from khronos_gb300.device import GpuSim

    stable, unstable = _unstable_spec(dtype)
    ok = GpuSim(stable, lib=gpu_lib)
    ok.step(400)
    ok.check_finite()
    ok.close()

    bad = GpuSim(unstable, lib=gpu_lib)
    bad.step(5)
    bad.check_finite()  # still growing, not yet overflowed
    bad.step(395)
    with pytest.raises(_abi.KhError) as e:
        bad.check_finite()
    assert e.value.status == _abi.KH_ERR_NAN
    assert "non-finite values in" in str(e.value)
    # the simulation stays usable: reset clears the fields, and a sticky
    # error is not left behind
    bad.reset()
    bad.check_finite()
    bad.close()
