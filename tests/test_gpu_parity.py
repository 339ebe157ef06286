"""CUDA step loop vs the CPU oracle, through the C ABI, on seeded inputs.

Bar: FP64 fields and DFT values within 1e-10 relative L2 of the oracle (both
CPML semantics); FP32 within 2e-4 relative L2 of the FP32 oracle (different
rounding: FMA contraction and the B/D-free update of plain cells).
"""
import math

import numpy as np
import pytest

from conftest import dft_errors, field_errors, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-10, "f32": 2e-4}


def safe_rel(a, b):
    s = max(float(np.max(np.abs(b))), 1e-300)
    return rel_l2(a / s, b / s)


def compare(spec, steps, oracle, gpu_lib, tol, check_dft=True, chunks=1):
    from khronos_gb300.device import GpuSim

    gpu = GpuSim(spec, lib=gpu_lib)
    ref = oracle.OracleSim(spec)
    per = steps // chunks
    for _ in range(chunks):
        gpu.step(per)
        ref.step(per)
    assert gpu.timestep == ref.timestep
    assert gpu.sources_active == ref.sources_active
    worst = {}
    fa = [gpu.field(c) for c in range(6)]
    fb = [ref.field(c) for c in range(6)]
    for c in range(6):
        assert np.all(np.isfinite(fa[c])) == np.all(np.isfinite(fb[c]))
    for c, e in enumerate(field_errors(fa, fb)):
        worst[f"field{c}"] = e
    if check_dft and spec.monitors:
        da = [gpu.dft(m) for m in range(len(spec.monitors))]
        db = [ref.dft(m) for m in range(len(spec.monitors))]
        for m, e in enumerate(dft_errors(da, db)):
            worst[f"dft{m}"] = e
    gpu.close()
    ref.close()
    bad = {k: v for k, v in worst.items() if not v <= tol}
    assert not bad, f"relative L2 above {tol}: {bad}"
    return worst


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dipole_small(kh, oracle, gpu_lib, semantics, dtype):
    from khronos_gb300 import configs

    w = configs.dipole(dtype=dtype, steps=160, resolution=10)
    w.sim.semantics = semantics
    # the CPU-path semantics grow without bound: keep those runs short
    steps = 160 if semantics == "cpml" else 60
    compare(w.sim.spec(), steps, oracle, gpu_lib, TOL[dtype])


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_waveguide_scaled(kh, oracle, gpu_lib, semantics, dtype):
    from khronos_gb300 import configs

    w = configs.waveguide(dtype=dtype, scale=0.25)
    w.sim.semantics = semantics
    steps = 120 if semantics == "cpml" else 50
    compare(w.sim.spec(), steps, oracle, gpu_lib, TOL[dtype], chunks=2)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dispersive_scaled(kh, oracle, gpu_lib, dtype):
    from khronos_gb300 import configs

    w = configs.dispersive(dtype=dtype, scale=0.25)
    compare(w.sim.spec(), 150, oracle, gpu_lib, TOL[dtype])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_photonic_slab_scaled(kh, oracle, gpu_lib, dtype):
    """The periodic benchmark workload (x and y wrapped, CPML along z) at a
    quarter of its resolution: 64×64×32."""
    from khronos_gb300 import configs

    w = configs.photonic_slab(dtype=dtype, scale=0.25)
    assert tuple(w.sim.spec().n) == (64, 64, 32) and w.sim.spec().periodic == 3
    compare(w.sim.spec(), 150, oracle, gpu_lib, TOL[dtype])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dispersive_cells_pass_matches_full_launch(kh, oracle, gpu_lib, dtype, monkeypatch):
    """χ3 and pole cells updated by the LEAN E launch plus the dispersive-cell
    pass agree with the FULL launch (KHRONOS_GB300_DISP_FIX=0), which does
    them in the cell loop, across the source cutoff; both match the oracle."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.dispersive(dtype=dtype, scale=0.25)
    spec = w.sim.spec()
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("KHRONOS_GB300_DISP_FIX", mode)
        g = GpuSim(spec, lib=gpu_lib)
        g.step(400)
        out[mode] = ([g.field(c) for c in range(6)], [g.dft(m) for m in range(len(spec.monitors))])
        g.close()
    tol = 1e-13 if dtype == "f64" else 1e-6
    for a, b in zip(field_errors(out["1"][0], out["0"][0]), [0] * 6):
        assert a <= tol
    assert max(dft_errors(out["1"][1], out["0"][1])) <= tol
    monkeypatch.setenv("KHRONOS_GB300_DISP_FIX", "1")
    compare(spec, 150, oracle, gpu_lib, TOL[dtype])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dispersive_cells_pass_on_an_odd_grid(kh, oracle, gpu_lib, dtype, monkeypatch):
    """The dispersive-cell pass on a grid whose x extent is odd (the last lane
    of a row has one cell), with χ3-only row segments, pole segments and a
    12%-filled χ3 mix inside and outside the CPML: same as the FULL launch and
    the oracle."""
    from khronos_gb300 import grid as G
    from khronos_gb300.device import GpuSim
    from khronos_gb300.simulation import apply_chi1_correction
    from khronos_gb300.spec import DrudeSusceptibility, LorentzianSusceptibility

    rng = np.random.default_rng(11)
    n = (37, 22, 18)
    chi3 = np.where(rng.uniform(size=n) > 0.88, 0.04, 0.0)
    chi3[:, :, 8:11] = 0.02  # whole χ3 planes: segments without pole cells
    lor, dru = LorentzianSusceptibility(1.0, 0.05, 1.0), DrudeSusceptibility(0.1, 40.0)
    sl = np.zeros(n)
    sl[25:37, 3:9, 4:12] = lor.sigma
    sd = np.zeros(n)
    sd[2:7, 12:20, 6:14] = dru.sigma
    poles = [(lor, sl), (dru, sd)]
    dt = G.Grid.build((3.7, 2.2, 1.8), (0, 0, 0), 10, dtype).dt
    eps = apply_chi1_correction([1.0 / rng.uniform(1.0, 3.0, size=n) for _ in range(3)], poles, dt, T=np.float64)
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EZ,
                           center=(0.2, 0, 0), size=(0.4, 0.6, 0.5), amplitude=3.0)
    # sources on Lorentz cells: their term enters the pass's E = ε⁻¹(D + S − ΣP),
    # the second (Ex) on cells in the x-CPML, where E also goes through the W stage
    src2 = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EY,
                            center=(1.2, -0.55, -0.1), size=(0.4, 0.2, 0.2), amplitude=2.0)
    src3 = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EX,
                            center=(1.7, -0.55, -0.1), size=(0.2, 0.2, 0.2), amplitude=2.0)
    mon = kh.DFTMonitor(component=kh.EX, center=(0, 0, 0), size=(3.7, 2.2, 0), frequencies=[0.7, 0.9])
    sim = kh.Simulation(cell_size=(3.7, 2.2, 1.8), resolution=10, sources=[src, src2, src3], monitors=[mon],
                        boundaries=[[0.3, 0.3]] * 3, dtype=dtype, eps_inv=eps, chi3=chi3, poles=poles)
    spec = sim.spec()
    assert tuple(spec.n) == n
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("KHRONOS_GB300_DISP_FIX", mode)
        g = GpuSim(spec, lib=gpu_lib)
        g.step(160)
        out[mode] = ([g.field(c) for c in range(6)], [g.dft(0)])
        g.close()
    # FP32: the pass applies the W stage of x-CPML pole cells as a correction
    # of the LEAN launch's result (E' + op·ΔW), the FULL launch in one
    # expression, so the two round differently
    tol = 1e-13 if dtype == "f64" else 1e-5
    assert max(field_errors(out["1"][0], out["0"][0])) <= tol
    assert max(dft_errors(out["1"][1], out["0"][1])) <= tol
    monkeypatch.setenv("KHRONOS_GB300_DISP_FIX", "1")
    compare(spec, 160, oracle, gpu_lib, TOL[dtype])


def _odd_sim(kh, semantics="cpml", dtype="f64", boundaries=((0.3, 0.2), (0.2, 0.4), (0.4, 0.3)), **kw):
    srcs = [
        kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3), component=kh.EZ,
                         center=(0.31, -0.22, 0.13), size=(0, 0, 0)),
        kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3), component=kh.EZ,
                         center=(0.31, -0.22, 0.13), size=(0, 0, 0), amplitude=0.5 - 0.25j),
        kh.UniformSource(time_profile=kh.ContinuousWaveSource(fcen=0.6), component=kh.HY,
                         center=(-0.5, 0.3, -0.2), size=(0, 0.4, 0)),
        kh.UniformSource(time_profile=kh.CustomSource(src_func=lambda t: math.sin(3 * t) * math.exp(-t / 4),
                                                      fcen=0.5, fwidth=0.3, end_time=6.0, table_steps=400),
                         component=kh.EX, center=(0.1, 0.1, -0.4), size=(0.3, 0, 0)),
    ]
    mons = [kh.DFTMonitor(component=kh.EZ, center=(0.2, 0, 0), size=(0, math.inf, math.inf),
                          frequencies=[0.7, 0.8]),
            kh.DFTMonitor(component=kh.HX, center=(0, 0, 0.3), size=(0.6, 0.5, 0), frequencies=[0.8],
                          decimation=3)]
    return kh.Simulation(cell_size=(3.7, 2.3, 1.9), resolution=10, sources=srcs, boundaries=boundaries,
                         monitors=mons, dtype=dtype, semantics=semantics, **kw)


@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_odd_grid_mixed_sources(kh, oracle, gpu_lib, semantics, dtype):
    """37×23×19 (not a multiple of the vector width), asymmetric PML, stacked
    sources on one cell, an H source, CW and tabulated time profiles, a monitor
    reaching the staggered wall layer, decimation."""
    sim = _odd_sim(kh, semantics, dtype)
    steps = 150 if semantics == "cpml" else 40
    compare(sim.spec(), steps, oracle, gpu_lib, TOL[dtype])


@pytest.mark.parametrize("boundaries", [None, ((0.5, 0.5), (0, 0), (0, 0)), ((0, 0), (0, 0), (0.3, 0.0))])
def test_partial_or_no_pml(kh, oracle, gpu_lib, boundaries):
    sim = _odd_sim(kh, "cpml", "f64", boundaries=boundaries)
    compare(sim.spec(), 120, oracle, gpu_lib, TOL["f64"])


@pytest.mark.parametrize("comp", ["EX", "EY", "HZ"])
@pytest.mark.parametrize("semantics", ["cpml", "reference_cpu"])
def test_source_inside_cpml(kh, oracle, gpu_lib, comp, semantics):
    """A source plane inside the x-CPML: with a W stage on its component (Ex)
    the source is applied in the full kernel, without one (Ey, Hz) after the
    lean kernel; both must equal the oracle."""
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3),
                           component=getattr(kh, comp), center=(-1.05, 0.1, 0.0), size=(0, 0.8, 0.6))
    mon = kh.DFTMonitor(component=kh.EY, center=(0.3, 0, 0), size=(0, 1.0, 1.0), frequencies=[0.8])
    sim = kh.Simulation(cell_size=(2.6, 2.0, 1.8), resolution=10, sources=[src], monitors=[mon],
                        boundaries=[[0.4, 0.4]] * 3, dtype="f64", semantics=semantics)
    steps = 120 if semantics == "cpml" else 50
    compare(sim.spec(), steps, oracle, gpu_lib, TOL["f64"])


def test_whole_axis_pml_fallback(kh, oracle, gpu_lib):
    """PML thicker than half the axis: the reference plans a single chunk whose
    PML flags cover whole axes (Chunking.jl:907-931)."""
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3), component=kh.EZ)
    sim = kh.Simulation(cell_size=(1.2, 1.0, 0.8), resolution=10, sources=[src],
                        boundaries=[[0.7, 0.7]] * 3, dtype="f64")
    sp = sim.spec()
    assert sp.pml_lo == sp.n and sp.pml_hi == (0, 0, 0)
    compare(sp, 80, oracle, gpu_lib, TOL["f64"], check_dft=False)


def test_source_cutoff_transition(kh, oracle, gpu_lib):
    """A short pulse whose cutoff falls inside the run: sources switch off on
    the same step in both (Kernels.jl:27-35)."""
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=1.0, fwidth=2.0), component=kh.EY,
                           center=(0.05, 0.0, -0.1), size=(0.4, 0.3, 0))
    sim = kh.Simulation(cell_size=(2.0, 2.0, 2.0), resolution=10, sources=[src],
                        boundaries=[[0.3, 0.3]] * 3, dtype="f64")
    sp = sim.spec()
    from khronos_gb300.device import GpuSim

    gpu = GpuSim(sp, lib=gpu_lib)
    ref = oracle.OracleSim(sp)
    n_cut = sim.steps_until(sp.sources[0].cutoff) + 1
    gpu.step(n_cut - 2)
    ref.step(n_cut - 2)
    assert gpu.sources_active and ref.sources_active
    gpu.step(4)
    ref.step(4)
    assert not gpu.sources_active and not ref.sources_active
    gpu.step(40)
    ref.step(40)
    errs = field_errors([gpu.field(c) for c in range(6)], [ref.field(c) for c in range(6)])
    assert max(errs) <= TOL["f64"]


def test_per_voxel_mu_and_chi3_without_pml(kh, oracle, gpu_lib):
    rng = np.random.default_rng(5)
    n = (24, 20, 16)
    mu = [1.0 / rng.uniform(1.0, 2.0, size=n) for _ in range(3)]
    eps = [1.0 / rng.uniform(1.0, 4.0, size=n) for _ in range(3)]
    chi3 = np.where(rng.uniform(size=n) > 0.7, 0.05, 0.0)
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EX,
                           center=(0, 0, 0), size=(0.5, 0.5, 0.5), amplitude=4.0)
    sim = kh.Simulation(cell_size=(2.4, 2.0, 1.6), resolution=10, sources=[src], dtype="f64",
                        eps_inv=eps, mu_inv=mu, chi3=chi3)
    compare(sim.spec(), 100, oracle, gpu_lib, TOL["f64"], check_dft=False)


def test_material_conductivity_reference_cpu(kh, oracle, gpu_lib):
    """σD/σB act only inside PML chunks on the CPU path; without PML they are
    ignored (step_curl_and_update! has no conductivity argument)."""
    n = (20, 18, 16)
    sd = [np.full(n, 0.3) for _ in range(3)]
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EZ)
    sim = kh.Simulation(cell_size=(2.0, 1.8, 1.6), resolution=10, sources=[src], dtype="f64",
                        sigma_d=sd, sigma_b=sd, semantics="reference_cpu")
    compare(sim.spec(), 60, oracle, gpu_lib, TOL["f64"], check_dft=False)


def test_material_conductivity_with_pml_is_rejected(kh, gpu_lib, oracle):
    """The reference has no generic_curl! method for conductivity in face
    chunks (C allocated without U): both refuse the configuration."""
    from khronos_gb300 import _abi
    from khronos_gb300.device import GpuSim

    n = (20, 18, 16)
    sd = [np.full(n, 0.3) for _ in range(3)]
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.4), component=kh.EZ)
    for sem in ("reference_cpu", "cpml"):
        sim = kh.Simulation(cell_size=(2.0, 1.8, 1.6), resolution=10, sources=[src], dtype="f64",
                            sigma_d=sd, boundaries=[[0.3, 0.3]] * 3, semantics=sem)
        with pytest.raises(_abi.KhError) as e:
            GpuSim(sim.spec(), lib=gpu_lib)
        assert e.value.status == _abi.KH_ERR_UNSUPPORTED
        with pytest.raises(RuntimeError):
            oracle.OracleSim(sim.spec())


def test_flux_on_device_matches_host(kh, oracle, gpu_lib):
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim
    from khronos_gb300.monitors import flux_from_dft

    w = configs.waveguide(dtype="f64", scale=0.25)
    sp = w.sim.spec()
    gpu = GpuSim(sp, lib=gpu_lib)
    ref = oracle.OracleSim(sp)
    gpu.step(200)
    ref.step(200)
    base = 0
    for fm in w.flux_monitors:
        ids = list(range(base, base + 4))
        base += 4
        dev = gpu.flux(ids, fm.normal_axis, fm.dA)
        host = flux_from_dft(fm.normal_axis, *[ref.dft(i) for i in ids], fm.dA)
        assert np.allclose(dev, host, rtol=1e-9, atol=1e-12 * np.max(np.abs(host)))


def test_reset_and_state_roundtrip(kh, gpu_lib):
    """N steps == k steps + export/import + N-k steps; reset() reproduces a fresh run."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.waveguide(dtype="f32", scale=0.25)
    sp = w.sim.spec()
    a = GpuSim(sp, lib=gpu_lib)
    a.step(90)
    fa = [a.field(c) for c in range(6)]
    da = a.dft(0)
    b = GpuSim(sp, lib=gpu_lib)
    b.step(37)
    blob = b.export_state()
    c = GpuSim(sp, lib=gpu_lib)
    c.import_state(blob)
    assert c.timestep == 37
    c.step(53)
    for comp in range(6):
        assert np.array_equal(c.field(comp), fa[comp])
    assert np.array_equal(c.dft(0), da)
    a.reset()
    assert a.timestep == 0 and a.sources_active
    a.step(90)
    for comp in range(6):
        assert np.array_equal(a.field(comp), fa[comp])


def test_z_tiling_is_invisible(kh, oracle, gpu_lib, monkeypatch):
    """The TMA kernel's z-tile depth changes nothing: tiles that cross a
    64-plane group of the special-cell bitmask (12, 7) give the same bits as
    aligned tiles (16, 64), and the default matches the oracle."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.waveguide(dtype="f32", scale=0.6)
    sp = w.sim.spec()
    assert sp.n[2] > 64
    runs = {}
    for zp in ("16", "12", "7", "64"):
        monkeypatch.setenv("KHRONOS_GB300_ZPLANES", zp)
        s = GpuSim(sp, lib=gpu_lib)
        s.step(70)
        runs[zp] = ([s.field(c) for c in range(6)], s.dft(0))
        s.close()
    for zp in ("12", "7", "64"):
        for c in range(6):
            assert np.array_equal(runs[zp][0][c], runs["16"][0][c]), (zp, c)
        assert np.array_equal(runs[zp][1], runs["16"][1]), zp
    monkeypatch.delenv("KHRONOS_GB300_ZPLANES")
    compare(sp, 70, oracle, gpu_lib, TOL["f32"])


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_step_graphs_are_invisible(kh, gpu_lib, dtype, monkeypatch):
    """Batches replayed from captured CUDA graphs give bit-identical fields and
    DFT values to directly launched batches, across the source cutoff.  A
    launch sequence is captured the second time it occurs, so the run ends
    with full batches that repeat."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.waveguide(dtype=dtype, scale=0.25)
    spec = w.sim.spec()
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("KHRONOS_GB300_GRAPHS", mode)
        g = GpuSim(spec, lib=gpu_lib)
        for n in (7, 1500, 64, 64, 300, 2500):  # irregular calls across the cutoff (step ~400)
            g.step(n)
        out[mode] = ([g.field(c) for c in range(6)], [g.dft(m) for m in range(len(spec.monitors))],
                     g.graph_replays)
        g.close()
    assert out["0"][2] == 0
    assert out["1"][2] > 0
    for a, b in zip(out["0"][0] + out["0"][1], out["1"][0] + out["1"][1]):
        assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,semantics", [("f32", "cpml"), ("f64", "cpml"), ("f32", "reference_cpu")])
def test_dft_batch_is_invisible(kh, gpu_lib, dtype, semantics, monkeypatch):
    """All monitors of a half-step accumulated by one launch give the same bits
    as one launch per monitor (KHRONOS_GB300_DFT_BATCH=0): the waveguide's two
    flux planes (Ey, Ez, Hy, Hz), with the source active and after its cutoff,
    in both CPML semantics."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.waveguide(dtype=dtype, scale=0.25)
    w.sim.semantics = semantics
    spec = w.sim.spec()
    steps = 700 if semantics == "cpml" else 60
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("KHRONOS_GB300_DFT_BATCH", mode)
        g = GpuSim(spec, lib=gpu_lib)
        g.step(steps)
        out[mode] = [g.field(c) for c in range(6)] + [g.dft(m) for m in range(len(spec.monitors))]
        g.close()
    assert any(np.any(d != 0) for d in out["1"][6:])
    for a, b in zip(out["0"], out["1"]):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_run_benchmark(kh, gpu_lib):
    """run_benchmark(sim, until) mirrors the reference: steps until times and
    returns a positive MCells/s rate."""
    from khronos_gb300 import configs

    w = configs.dipole(dtype="f32", resolution=10)
    rate = w.sim.run_benchmark(60)
    assert rate > 0 and w.sim.timestep == 60
    w.sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_field_view_is_the_field_in_place(kh, gpu_lib, dtype):
    """kh_sim_field_view: a zero-copy strided view equal to kh_sim_get_field,
    that follows later steps, and whose device-side norm matches
    kh_sim_field_sq_norms."""
    import torch

    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    w = configs.waveguide(dtype=dtype, scale=0.25)
    g = GpuSim(w.sim.spec(), lib=gpu_lib)
    g.step(120)
    g.synchronize()
    views = [g.field_view(c) for c in range(6)]
    for c in range(6):
        host = g.field(c)
        assert tuple(views[c].shape) == host.shape
        assert np.array_equal(views[c].double().cpu().numpy(), host)
    g.step(40)
    g.synchronize()
    norms = g.field_sq_norms()
    for c in range(6):
        assert np.array_equal(views[c].double().cpu().numpy(), g.field(c))
        dev = float(torch.sum(views[c].double() ** 2))
        assert math.isclose(dev, norms[c], rel_tol=1e-12, abs_tol=1e-300)
    # the reference's raw layout (ghost at 0, interior 1..N): what a Julia
    # shim puts back into sim.fields
    for c in range(6):
        gv = g.field_view(c, ghosted=True)
        host = g.field(c)
        assert tuple(gv.shape) == tuple(d + 1 for d in host.shape)
        assert np.array_equal(gv[1:, 1:, 1:].double().cpu().numpy(), host)
        for a in range(3):
            assert not torch.any(gv.select(a, 0) != 0)
    del views
    g.close()


@pytest.mark.gpu
def test_step_timed_is_invisible(kh, gpu_lib):
    """kh_sim_step_timed (events around the launches of every 8th step) gives
    the fields of a plain run and positive per-half times."""
    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim

    spec = configs.waveguide(dtype="f32", scale=0.25).sim.spec()
    a = GpuSim(spec, lib=gpu_lib)
    a.step(93)
    b = GpuSim(spec, lib=gpu_lib)
    h, e, d = b.step_timed(93)
    assert h > 0 and e > 0 and d >= 0
    for c in range(6):
        assert np.array_equal(a.field(c), b.field(c))
    assert np.array_equal(a.dft(0), b.dft(0))
    a.close()
    b.close()
