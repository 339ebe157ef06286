"""run(sim; until = f) and stop_when_dft_decayed (Simulation.jl:295-485):
the stop function's logic on scripted norm sequences (host), and on the
device that the batched run stops at the same step as a call-per-step replay
that reads every monitor norm afresh."""
import math
import warnings

import numpy as np
import pytest


class _Scripted:
    """A stand-in simulation: round_time = timestep·dt, norms from a script."""

    def __init__(self, norms, dt=1.0):
        self.norms = norms
        self.timestep = 0
        self.dt = dt

    def round_time(self, ts=None):
        return (self.timestep if ts is None else ts) * self.dt

    def dft_fields_norms(self):
        return np.asarray(self.norms[self.timestep], dtype=float)


def _decisions(stop, sim, n):
    out = []
    for _ in range(n):
        out.append(stop(sim))
        sim.timestep += 1
    return out


def test_stop_when_dft_decayed_logic(kh):
    # two monitors; monitor 1 never sees signal (norm 0 throughout)
    norms = [[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [2.5, 0.0], [2.5 + 1e-9, 0.0], [2.5 + 1e-9, 0.0]]
    stop = kh.stop_when_dft_decayed(tolerance=1e-6)
    # t0: no signal; t1: first record; t2: change 1 = max → not converged;
    # t3: change 0.5 / 1; t4: 1e-9 / 1 ≤ 1e-6 → converged
    assert _decisions(stop, _Scripted(norms), 5) == [False, False, False, False, True]
    assert 1 not in stop.state


def test_stop_when_dft_decayed_decimation_quirk(kh):
    """A decimated monitor's norm is flat between updates, so the step after
    its first change reports convergence (change 0 ≤ tol·maxchange)."""
    norms = [[1.0], [1.0], [1.0], [3.0], [3.0], [3.0]]
    stop = kh.stop_when_dft_decayed(tolerance=1e-6)
    assert _decisions(stop, _Scripted(norms), 5) == [False, False, False, False, True]


def test_stop_when_dft_decayed_runtime_bounds(kh):
    norms = [[1.0 + t] for t in range(20)]
    stop = kh.stop_when_dft_decayed(tolerance=1e-6, minimum_runtime=5.0, maximum_runtime=8.0)
    sim = _Scripted(norms)
    assert stop.steps_before_decision(sim) == 5
    d = _decisions(stop, sim, 5)
    assert d == [False] * 5 and stop.state == {}
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        d = _decisions(stop, sim, 5)
    assert d == [False, False, False, False, True]  # t = 5..8 run, t = 9 > 8 stops
    assert any("Maximum runtime" in str(x.message) for x in w)
    with pytest.raises(ValueError):
        kh.stop_when_dft_decayed(minimum_runtime=2.0, maximum_runtime=1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_run_until_stop_function_matches_per_step_replay(kh, gpu_lib, dtype, caplog):
    import logging

    from khronos_gb300 import configs

    def fresh():
        return configs.dipole(dtype=dtype, resolution=10).sim

    sim = fresh()
    stop = kh.stop_when_dft_decayed(tolerance=1e-6, minimum_runtime=2.0)
    with caplog.at_level(logging.INFO, logger="khronos_gb300"):
        sim.run(until_after_sources=stop)
    msgs = [r.getMessage() for r in caplog.records]
    assert "All sources have terminated..." in msgs
    assert any(m.startswith(f"Simulation complete: {sim.timestep} steps") for m in msgs)
    t_stop = sim.timestep
    norms_at_stop = sim.dft_fields_norms()
    sim.close()

    # replay: one step at a time, every norm read from the device
    ref = fresh()
    ref.prepare()
    last = ref.last_source_time()
    while ref.round_time() <= last:
        ref.step(1)

    class _Fresh:
        timestep = property(lambda self: ref.timestep)
        round_time = staticmethod(ref.round_time)
        dft_fields_norms = staticmethod(lambda: ref._dev.dft_norms())

    stop2 = kh.stop_when_dft_decayed(tolerance=1e-6, minimum_runtime=2.0)
    w = _Fresh()
    while not stop2(w):
        ref.step(1)
    assert ref.timestep == t_stop
    assert np.array_equal(ref._dev.dft_norms(), norms_at_stop)
    # the norms are those of the DFT arrays
    for i in range(len(ref._dft_monitors)):
        d = ref._dev.dft(i)
        assert math.isclose(float(np.sqrt(np.sum(np.abs(d) ** 2))), norms_at_stop[i], rel_tol=1e-12)
    ref.close()
