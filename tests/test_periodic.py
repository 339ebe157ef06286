"""Periodic boundaries (Periodic, or Bloch with k = 0, on both sides of an
axis): after each half-step the updated field's last interior layer wraps
into the ghost layer below the first and the first into the layer above the
last (_add_periodic_connections! single-chunk branch, Chunking.jl:1751-1768;
_exchange_halos_local!, Chunking.jl:2138-2172).  The E wrap is taken before
the χ3 correction (exchange_halos!(:E) ends step_E_fused!, Kernels.jl:452).

CPU: the axis mask, and the oracle's wrap pinned by two exact properties of
a periodic axis without PML — a source uniform along it gives fields uniform
along it, and moving a source by whole cells rolls the fields by as many.
GPU: the device against the oracle on periodic grids (both CPML semantics,
FP64 and FP32, sources and monitors on the wrap faces, χ3 on the faces, ADE
poles, the register-pipelined kernel) and the bounds-checked build."""
import math

import numpy as np
import pytest

TOL = {"f64": 1e-10, "f32": 2e-4}


def _pulse(kh, fcen=0.8):
    return kh.GaussianPulseSource(fcen=fcen, fwidth=0.3)


def _slab_sim(kh, semantics="cpml", dtype="f64", src_center_x=0.0, src_size_x=math.inf, periodic=(0, 1),
              res=10, **kw):
    """Periodic along `periodic` axes with no PML there, PML along the others:
    the reference's periodic-slab set-up (periodic x, y; PML z)."""
    bnd = [[0.0, 0.0] if a in periodic else [0.3, 0.4] for a in range(3)]
    bcs = [[kh.Periodic(), kh.Periodic()] if a in periodic else [None, None] for a in range(3)]
    src = kh.UniformSource(time_profile=_pulse(kh), component=kh.EX,
                           center=(src_center_x, 0.11, -0.3), size=(src_size_x, 0.5, 0))
    # monitors on the wrap faces: the first reaches layer n along x in FP32
    # (a full-span box there reads one layer past the component in FP32 and is
    # refused by the device)
    mons = [kh.DFTMonitor(component=kh.EX, center=(0.15, 0.1, 0.35), size=(1.0, 0.9, 0),
                          frequencies=[0.7, 0.8]),
            kh.DFTMonitor(component=kh.HY, center=(-0.15, 0, 0.2), size=(1.0, 0.6, 0), frequencies=[0.8],
                          decimation=2)]
    return kh.Simulation(cell_size=(1.3, 1.1, 2.3), resolution=res, sources=[src], monitors=mons,
                         boundaries=bnd, boundary_conditions=bcs, dtype=dtype, semantics=semantics, **kw)


# ---------------------------------------------------------------- host logic


def test_periodic_mask(kh):
    from khronos_gb300.boundaries import periodic_mask

    P, B = kh.Periodic, kh.Bloch
    assert periodic_mask(None) == 0
    assert periodic_mask([[P(), P()], [None, None], [P(), B(k=0.0)]]) == 0b101
    assert periodic_mask([[P(), None], [B(), B()], [None, None]]) == 0b010  # one side only: no wrap
    with pytest.raises(NotImplementedError):
        periodic_mask([[B(k=0.4), B(k=0.4)], [None, None], [None, None]])


def test_periodic_sides_zero_sigma(kh):
    sp = _slab_sim(kh).spec()
    assert sp.periodic == 0b011
    assert sp.pml_lo[:2] == (0, 0) and sp.pml_hi[:2] == (0, 0)
    sim = kh.Simulation(cell_size=(1.3, 1.1, 2.3), resolution=10, boundaries=[[0.3, 0.3]] * 3,
                        boundary_conditions=[[kh.Periodic(), kh.Periodic()], [None, None], [None, None]])
    s = sim.spec()
    assert s.periodic == 1 and s.pml_lo[0] > 0 and np.all(s.sigma_b[0] == 0)


# ------------------------------------------------------- oracle properties


def _oracle_fields(oracle, spec, steps):
    o = oracle.OracleSim(spec)
    o.step(steps)
    out = [o.field(c) for c in range(6)]
    o.close()
    return out


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_oracle_uniform_along_periodic_axis(kh, oracle, semantics):
    """A source covering the whole periodic x axis: every x layer of every
    component stays bit-identical; with zero walls instead it does not."""
    sp = _slab_sim(kh, semantics, periodic=(0,)).spec()
    f = _oracle_fields(oracle, sp, 60)
    nx = sp.n[0]
    assert np.abs(f[kh.EX]).max() > 0 and np.abs(f[kh.HZ]).max() > 0
    for c in range(6):
        a = f[c]
        for i in range(1, a.shape[0]):
            assert np.array_equal(a[i], a[0]), (c, i)
    sp.periodic = 0
    g = _oracle_fields(oracle, sp, 60)
    assert not np.array_equal(g[kh.EX][nx - 1], g[kh.EX][nx // 2])


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_oracle_shift_rolls_fields(kh, oracle, semantics):
    """Moving a point-like source by s whole cells along the periodic axes rolls
    every field by s cells (the staggered layer n, a copy of layer 0, follows)."""
    s = (3, -2)  # the moved source stays inside the cell (sources do not wrap)
    d = 0.1
    a = _slab_sim(kh, semantics, src_center_x=0.02, src_size_x=0.0).spec()
    b_sim = _slab_sim(kh, semantics, src_center_x=0.02 + s[0] * d, src_size_x=0.0)
    b_sim.sources[0].center = (0.02 + s[0] * d, 0.11 + s[1] * d, -0.3)
    b = b_sim.spec()
    fa = _oracle_fields(oracle, a, 50)
    fb = _oracle_fields(oracle, b, 50)
    n = a.n
    scale = max(np.abs(f).max() for f in fb)
    for c in range(6):
        x = fa[c][:n[0], :n[1]]
        y = fb[c][:n[0], :n[1]]
        r = np.roll(x, s, axis=(0, 1))
        assert np.abs(r - y).max() <= 1e-12 * scale, c
        # the staggered wall layer of a periodic axis holds layer 0 over the
        # Center range of the other axes (edges where two walls meet are not
        # copied: _component_send_range, Chunking.jl:2184-2200)
        if fb[c].shape[0] == n[0] + 1:
            assert np.array_equal(fb[c][n[0], :n[1], :n[2]], fb[c][0, :n[1], :n[2]])
        if fb[c].shape[1] == n[1] + 1:
            assert np.array_equal(fb[c][:n[0], n[1], :n[2]], fb[c][:n[0], 0, :n[2]])


# ------------------------------------------------------------------- device


def _kerr_sim(kh, dtype="f64", semantics="reference_cpu"):
    """Fully periodic in x and y with a χ3 slab filling them: the wrap faces
    carry χ3, so the ghost layers must hold E before the Kerr correction."""
    sim = _slab_sim(kh, semantics, dtype=dtype, periodic=(0, 1))
    n = sim.n
    chi3 = np.zeros(n)
    chi3[:, :, n[2] // 2 - 4:n[2] // 2 + 3] = 2.0
    sim.chi3 = chi3
    sim.sources[0].amplitude = 3.0
    return sim


def _pole_sim(kh, dtype="f64"):
    sim = _slab_sim(kh, "reference_cpu", dtype=dtype, periodic=(0,))
    n = sim.n
    sigma = np.zeros(n)
    sigma[:, 3:n[1] - 3, n[2] // 2 - 3:n[2] // 2 + 3] = 1.0
    sim.poles = [(kh.LorentzianSusceptibility(1.0, 0.05, 1.0), sigma)]
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("periodic", [(0, 1), (0,), (1, 2), (0, 1, 2)])
def test_periodic_matches_oracle(kh, oracle, gpu_lib, semantics, dtype, periodic):
    from test_gpu_parity import compare

    sim = _slab_sim(kh, semantics, dtype, periodic=periodic, src_center_x=0.07, src_size_x=0.6)
    compare(sim.spec(), 80 if semantics == "cpml" else 40, oracle, gpu_lib, TOL[dtype], chunks=2)


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_periodic_uniform_source_on_wrap_faces(kh, oracle, gpu_lib, semantics):
    from test_gpu_parity import compare

    compare(_slab_sim(kh, semantics, periodic=(0,)).spec(), 60, oracle, gpu_lib, TOL["f64"])


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_periodic_kerr_on_wrap_faces(kh, oracle, gpu_lib, dtype):
    from test_gpu_parity import compare

    compare(_kerr_sim(kh, dtype).spec(), 40, oracle, gpu_lib, TOL[dtype])


def test_kerr_case_is_nonlinear(kh, oracle):
    """The Kerr case above runs where χ3 changes the fields well above the
    parity bar, on the wrap faces too."""
    sp = _kerr_sim(kh).spec()
    lin = _kerr_sim(kh)
    lin.chi3 = None
    a = _oracle_fields(oracle, sp, 40)[kh.EX]
    b = _oracle_fields(oracle, lin.spec(), 40)[kh.EX]
    face = np.s_[0, :, :]
    assert np.linalg.norm(a[face] - b[face]) > 1e-3 * np.linalg.norm(b[face])


@pytest.mark.gpu
def test_periodic_poles(kh, oracle, gpu_lib):
    from test_gpu_parity import compare

    compare(_pole_sim(kh).spec(), 40, oracle, gpu_lib, TOL["f64"])


@pytest.mark.gpu
def test_periodic_register_kernel(kh, oracle, gpu_lib, monkeypatch):
    from test_gpu_parity import compare

    monkeypatch.setenv("KHRONOS_GB300_KERNEL", "simt")
    compare(_kerr_sim(kh, "f64").spec(), 30, oracle, gpu_lib, TOL["f64"])
    compare(_slab_sim(kh, "cpml", "f32", periodic=(0, 2)).spec(), 60, oracle, gpu_lib, TOL["f32"])


@pytest.mark.gpu
def test_periodic_bounds_checked(kh, gpu_lib):
    from test_bounds import _same
    from khronos_gb300 import _abi, build

    blib = _abi.load(build.build(bounds=True))
    _same(_kerr_sim(kh, "f64").spec(), gpu_lib, blib, chunks=(5, 17))
    _same(_slab_sim(kh, "cpml", "f32", periodic=(0, 1, 2)).spec(), gpu_lib, blib, chunks=(5, 17))


@pytest.mark.gpu
def test_periodic_requests_in_server_mix(kh, gpu_lib):
    """Periodic and zero-wall requests served together: each matches its solo
    run bit for bit (the wrap launches ride in each request's own step loop)."""
    from khronos_gb300.device import GpuSim
    from khronos_gb300.serve import Server

    specs = [_slab_sim(kh, "cpml", "f32", periodic=p, src_center_x=0.07, src_size_x=0.6).spec()
             for p in ((0, 1), (), (0, 1, 2), (2,))]
    specs.append(_kerr_sim(kh, "f32", "cpml").spec())
    steps = [90, 70, 110, 50, 60]
    solo = []
    for sp, n in zip(specs, steps):
        g = GpuSim(sp, lib=gpu_lib)
        g.step(n)
        solo.append([g.dft(m) for m in range(len(sp.monitors))] + [g.field(c) for c in range(6)])
        g.close()
    with Server(budget_bytes=4 << 30, max_resident=3, quantum_steps=16, lib=gpu_lib) as srv:
        reqs = [srv.submit(sp, n) for sp, n in zip(specs, steps)]
        for _ in reqs:
            r = srv.next_done(timeout=120)
            assert r is not None and r.wait()
            i = reqs.index(r)
            got = [r.sim.dft(m) for m in range(len(specs[i].monitors))] + [r.sim.field(c) for c in range(6)]
            for a, b in zip(got, solo[i]):
                np.testing.assert_array_equal(a, b)
            r.release()
