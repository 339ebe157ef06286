"""Boundary conditions (DataStructures.jl:157-162, Boundaries.jl:99-164): a
PEC or PMC side keeps the PML region its ``boundaries`` thickness gives but
with zero conductivity; so does a Periodic or Bloch side, whose halo wrap
(tests/test_periodic.py) needs both sides of the axis; a Bloch phase k ≠ 0
is refused (complex fields)."""
import numpy as np
import pytest


def _sim(kh, semantics="cpml", bcs=None):
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3), component=kh.EZ,
                           center=(0.13, -0.07, 0.05), size=(0.3, 0, 0))
    mon = kh.DFTMonitor(component=kh.EZ, center=(0.2, 0, 0), size=(0, 0.6, 0.5), frequencies=[0.7, 0.8])
    return kh.Simulation(cell_size=(2.1, 1.7, 1.5), resolution=10, sources=[src], monitors=[mon],
                         boundaries=[[0.4, 0.3], [0.3, 0.4], [0.3, 0.3]], dtype="f64", semantics=semantics,
                         boundary_conditions=bcs)


def _bcs(kh):
    return [[kh.PECBoundary(), None], [None, kh.PMCBoundary()], [None, None]]


def test_pec_pmc_sides_zero_sigma_keep_regions(kh):
    plain = _sim(kh).spec()
    sp = _sim(kh, bcs=_bcs(kh)).spec()
    assert sp.pml_lo == plain.pml_lo and sp.pml_hi == plain.pml_hi
    n0, nl = sp.n[0], sp.pml_lo[0]
    assert np.all(sp.sigma_b[0][:nl] == 0) and np.any(plain.sigma_b[0][:nl] > 0)
    assert np.array_equal(sp.sigma_b[0][n0 // 2:], plain.sigma_b[0][n0 // 2:])  # x high side untouched
    n1, nh = sp.n[1], sp.pml_hi[1]
    assert np.all(sp.sigma_d[1][n1 - nh:] == 0) and np.any(plain.sigma_d[1][n1 - nh:] > 0)
    assert np.array_equal(sp.sigma_b[2], plain.sigma_b[2])


@pytest.mark.parametrize("bc", ["Periodic", "Bloch"])
def test_periodic_and_bloch_sides(kh, bc):
    cond = getattr(kh, bc)()
    sp = _sim(kh, bcs=[[cond, cond], [None, None], [None, None]]).spec()
    assert sp.periodic == 1 and np.all(sp.sigma_b[0] == 0) and sp.pml_lo[0] > 0
    one = _sim(kh, bcs=[[cond, None], [None, None], [None, None]]).spec()
    assert one.periodic == 0 and np.all(one.sigma_b[0][:one.pml_lo[0]] == 0)
    with pytest.raises(NotImplementedError):
        _sim(kh, bcs=[[kh.Bloch(k=0.5), kh.Bloch(k=0.5)], [None, None], [None, None]])


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_pec_pmc_sides_match_oracle(kh, oracle, gpu_lib, semantics):
    from test_gpu_parity import TOL, compare

    compare(_sim(kh, semantics, _bcs(kh)).spec(), 100 if semantics == "cpml" else 40, oracle, gpu_lib,
            TOL["f64"])
