"""Request server (kh_server_*): continuous batching of independent
simulations.  Results must be the same alone and in the mix: each request's
kernels do the same arithmetic on its own arrays whatever runs beside it, so
the bar is bit-for-bit equality of the DFT arrays (tolerance 0)."""
import ctypes as C

import numpy as np
import pytest


def _small_stream(n, seed=7):
    from khronos_gb300 import configs

    rng = np.random.default_rng(seed)
    grids = [(64, 64, 64), (96, 96, 96), (64, 64, 64), (128, 128, 128)]
    return [configs.serving_request(i, grids[i % len(grids)], int(rng.integers(150, 400)),
                                    int(rng.integers(0, 2 ** 31 - 1))) for i in range(n)]


def test_server_rejects_bad_descriptor(kh, gpu_lib):
    from khronos_gb300 import _abi

    h = C.c_void_p()
    assert gpu_lib.kh_server_create(None, C.byref(h)) == _abi.KH_ERR_INVALID
    d = _abi.ServerDesc(0, 4, 64)  # zero budget
    assert gpu_lib.kh_server_create(C.byref(d), C.byref(h)) == _abi.KH_ERR_INVALID
    d = _abi.ServerDesc(1 << 30, -1, 64)
    assert gpu_lib.kh_server_create(C.byref(d), C.byref(h)) == _abi.KH_ERR_INVALID
    assert gpu_lib.kh_server_submit(None, None, 10, None) == _abi.KH_ERR_INVALID


def test_memory_estimate_and_plan(kh, gpu_lib):
    from khronos_gb300 import configs
    from khronos_gb300.serve import estimate_bytes, plan_batch

    small = configs.serving_request(0, (64, 64, 64), 100, 1).sim.spec()
    big = configs.serving_request(1, (128, 128, 128), 100, 1).sim.spec()
    es, eb = estimate_bytes(small, gpu_lib), estimate_bytes(big, gpu_lib)
    # E, H, B, D, U, W (6 components each with CPML on every axis) + ε⁻¹ (3):
    # 27 FP32 arrays in the padded layout (row pitch 96 for 64 cells, one
    # ghost plane each side), + cell classes, DFT and small tables
    padded = 96 * 66 * 66 * 4
    assert 27 * padded < es < 29 * padded
    assert 6 < eb / es < 7  # padded volumes 160·130·130 / 96·66·66 = 6.47
    p = plan_batch(small, 10, 3 * es, gpu_lib)
    assert p["max_batch"] == 3 and p["n_waves"] == 4


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(kh, gpu_lib):
    from khronos_gb300.device import GpuSim
    from khronos_gb300.serve import Server

    ws = _small_stream(6)
    solo = []
    for w in ws:
        g = GpuSim(w.sim.spec(), lib=gpu_lib)
        g.step(w.steps)
        solo.append([g.dft(i) for i in range(4)])
        g.close()
    with Server(budget_bytes=8 << 30, max_resident=4, quantum_steps=32, lib=gpu_lib) as srv:
        reqs = [srv.submit(w.sim.spec(), w.steps) for w in ws]
        seen = 0
        while seen < len(reqs):
            r = srv.next_done(timeout=120)
            assert r is not None
            assert r.wait()
            i = reqs.index(r)
            info = r.info()
            assert info.status == 0 and info.t_submit <= info.t_admit <= info.t_start <= info.t_done
            for m in range(4):
                np.testing.assert_array_equal(r.sim.dft(m), solo[i][m])
            assert r.sim.timestep == ws[i].steps
            r.release()
            seen += 1


@pytest.mark.gpu
def test_budget_bounds_residency(kh, gpu_lib):
    import time

    from khronos_gb300 import configs
    from khronos_gb300.serve import Server, estimate_bytes

    ws = [configs.serving_request(i, (96, 96, 96), 300, 100 + i) for i in range(5)]
    per = estimate_bytes(ws[0].sim.spec(), gpu_lib)
    budget = int(2.5 * per)
    with Server(budget_bytes=budget, max_resident=8, quantum_steps=32, lib=gpu_lib) as srv:
        reqs = [srv.submit(w.sim.spec(), w.steps) for w in ws]
        done = 0
        peak = 0
        while done < len(reqs):
            st = srv.stats()
            assert st["budget_used"] <= budget * 1.05
            peak = max(peak, st["resident"])
            r = srv.next_done(timeout=0.005)
            if r is not None:
                r.wait()
                r.release()
                done += 1
            time.sleep(0.001)
        assert 1 <= peak <= 2


@pytest.mark.gpu
def test_oversize_and_early_release_rejected(kh, gpu_lib):
    from khronos_gb300 import _abi, configs
    from khronos_gb300.serve import Server, estimate_bytes

    w = configs.serving_request(0, (64, 64, 64), 2000, 3)
    per = estimate_bytes(w.sim.spec(), gpu_lib)
    with Server(budget_bytes=per // 2, lib=gpu_lib) as srv:
        with pytest.raises(_abi.KhError) as ei:
            srv.submit(w.sim.spec(), w.steps)
        assert ei.value.status == _abi.KH_ERR_OOM
    with Server(budget_bytes=4 * per, lib=gpu_lib) as srv:
        r = srv.submit(w.sim.spec(), w.steps)
        with pytest.raises(_abi.KhError):
            r.release()  # still queued or running
        assert r.wait(timeout=120)
        r.release()


@pytest.mark.gpu
def test_run_batch_concurrent_matches_run_batch(kh, gpu_lib):
    from khronos_gb300.serve import run_batch, run_batch_concurrent

    ws = _small_stream(5, seed=11)
    specs = [w.sim.spec() for w in ws]
    steps = [w.steps for w in ws]
    a = run_batch(specs, steps, lib=gpu_lib)
    b = run_batch_concurrent(specs, steps, budget_bytes=8 << 30, max_concurrent=3, lib=gpu_lib)
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)
