"""Failure detection without a GPU fault: every shared-memory ring wait of the
TMA half-step kernels is bounded, and a kernel that gives up records
KH_ERR_TIMEOUT for the host instead of hanging.  The test makes the wait run
out through a test hook (KHRONOS_GB300_TEST_STALL=1: the first ring stage of
each CTA expects 16 bytes, no copy is issued into it, and the limit drops to
4096 polls); the status reaches kh_sim_synchronize, the kernels return, and the
context stays usable for the next simulation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives(kh, gpu_lib, monkeypatch):
    from khronos_gb300 import _abi, configs
    from khronos_gb300.device import GpuSim

    spec = configs.dipole(dtype="f32", resolution=10).sim.spec()
    monkeypatch.setenv("KHRONOS_GB300_GRAPHS", "0")
    monkeypatch.setenv("KHRONOS_GB300_TEST_STALL", "1")
    g = GpuSim(spec, lib=gpu_lib)
    monkeypatch.delenv("KHRONOS_GB300_TEST_STALL")
    with pytest.raises(_abi.KhError) as e:
        g.step(2)
        g.synchronize()
    assert e.value.status == _abi.KH_ERR_TIMEOUT
    assert "gave up" in str(e.value)
    g.close()

    ok = GpuSim(spec, lib=gpu_lib)
    ok.step(30)
    ok.synchronize()
    ok.check_finite()
    assert np.any(ok.field(kh.EZ) != 0)
    ok.close()
