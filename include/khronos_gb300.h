/*
 * khronos_gb300.h — C ABI of the GB300-native FDTD step loop.
 *
 * One `kh_sim` handle owns the device state of one single-domain Yee grid
 * (fields, CPML auxiliaries, materials, dispersive poles, sources, DFT
 * monitors).  Every entry point returns a kh_status; nothing aborts or
 * throws across the boundary.  A handle is single-threaded; distinct handles
 * may run concurrently on distinct streams.  Device work is enqueued on the
 * stream passed to kh_sim_step (a cudaStream_t passed as void*, NULL = the
 * legacy default stream); the library uses the CUDA primary context of the
 * current device, exactly like CUDA.jl does.
 *
 * Reference interface each group of calls replaces (Khronos.jl sources):
 *   kh_sim_create / kh_sim_prepare   prepare_simulation!   src/Simulation.jl:92-283
 *                                    (field allocation Chunking.jl:1069-1146,
 *                                     PML σ Boundaries.jl:99-164)
 *   kh_sim_set_material              GeometryData arrays   src/DataStructures.jl:214-242,
 *                                    per-chunk slicing     src/Chunking.jl:1159-1213
 *   kh_sim_add_pole                  init_polarization!    src/Geometry.jl:1136-1355
 *   kh_sim_add_source                assemble_sources      src/Sources/Sources.jl:44-92
 *                                    eval_time_source      src/Sources/TimeSources.jl:61-132,178-184
 *   kh_sim_add_dft_monitor           init_monitors(::DFTMonitor) src/Monitors/Monitors.jl:202-272
 *   kh_sim_step                      step!(sim)            src/Kernels/Kernels.jl:20-88
 *                                    (one call = n iterations of the `run` loop,
 *                                     src/Simulation.jl:356-362)
 *   kh_sim_read_dft                  DFTMonitorData.fields download (Array(...))
 *   kh_sim_flux                      get_flux              src/Monitors/FluxMonitor.jl:92-156
 *   kh_sim_get_field                 _pull_fields_from_device src/Visualization.jl:294-331
 *   kh_sim_reset                     reset_fields!         src/Simulation.jl:571-637
 *   kh_sim_timestep / _sources_active  sim.timestep / sim.sources_active
 *
 * Index conventions.  Cells are 0-based: cell (i,j,k) of this ABI is the
 * reference's Center index (i+1, j+1, k+1).  Per-voxel material arrays are
 * given over the Center range, x fastest: value[(k*ny + j)*nx + i].  Field
 * snapshots use the reference's component dimensions (src/utils.jl:26-37),
 * e.g. Ex is nx × (ny+1) × (nz+1), x fastest; the extra staggered layer is the
 * zero Dirichlet wall.  Complex host arrays are interleaved (re, im) doubles.
 */
#ifndef KHRONOS_GB300_H
#define KHRONOS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t kh_status;
#define KH_OK 0
#define KH_ERR_INVALID 1     /* bad argument or call order */
#define KH_ERR_OOM 2         /* device or host allocation failed */
#define KH_ERR_CUDA 3        /* a CUDA runtime call failed */
#define KH_ERR_TIMEOUT 4     /* a bounded device-side wait gave up */
#define KH_ERR_NAN 5         /* non-finite field value detected */
#define KH_ERR_UNSUPPORTED 6 /* configuration the reference itself rejects */

#define KH_F32 0
#define KH_F64 1

/* Field components, in the reference's order Ex, Ey, Ez, Hx, Hy, Hz. */
#define KH_EX 0
#define KH_EY 1
#define KH_EZ 2
#define KH_HX 3
#define KH_HY 4
#define KH_HZ 5

/* Material array kinds for kh_sim_set_material (comp = 0,1,2 for x,y,z). */
#define KH_MAT_EPS_INV 0   /* ε⁻¹ per voxel, per component              */
#define KH_MAT_MU_INV 1    /* μ⁻¹ per voxel, per component              */
#define KH_MAT_SIGMA_D 2   /* electric conductivity σD (raw, not ×Δt/2) */
#define KH_MAT_SIGMA_B 3   /* magnetic conductivity σB (raw)            */
#define KH_MAT_CHI3 4      /* χ(3) on the Center grid (comp ignored)    */

/* Time profiles of a source. */
#define KH_TIME_GAUSSIAN 0 /* GaussianPulseData  TimeSources.jl:78-132  */
#define KH_TIME_CW 1       /* ContinuousWaveData TimeSources.jl:53-72   */
#define KH_TIME_TABLE 2    /* CustomSourceData   TimeSources.jl:157-190 (host-tabulated) */

typedef struct kh_sim kh_sim;

/* Grid and boundary description.  All floating values are the ones the
 * reference's SimulationData stores (already rounded to the run's precision
 * when dtype == KH_F32), passed as double. */
typedef struct {
  int32_t n[3];        /* Nx, Ny, Nz (cells)                                   */
  int32_t dtype;       /* KH_F32 or KH_F64: precision of fields and arithmetic */
  double delta[3];     /* Δx, Δy, Δz                                          */
  double dt;           /* Δt                                                   */
  /* PML region widths in cells per axis and side: ceil(L/Δ) as in
   * Chunking.jl:121-122 and 642-643; 0 = no PML on that side.  A width equal
   * to n[a] on the low side marks the whole axis as PML (single-chunk plan). */
  int32_t pml_lo[3];
  int32_t pml_hi[3];
  /* PML conductivities sampled at cell centres, length n[a], i.e. the
   * reference's σ[2i-1] samples of compute_sigma (Boundaries.jl:23-72), already
   * scaled by Δt/2.  NULL = all zero. */
  const double* sigma_b[3];
  const double* sigma_d[3];
  double eps_inv;      /* scalar ε⁻¹ used where no per-voxel array is set (1) */
  double mu_inv;       /* scalar μ⁻¹ (1)                                       */
  int32_t semantics;   /* KH_SEM_*: which of the reference's CPML paths to follow */
  /* Bit a set: axis a is periodic (Periodic, or Bloch with k = 0).  After each
   * half-step the updated field's last interior layer along a is copied into
   * the ghost layer below the first, and the first into the layer above the
   * last, over the Center range of the other axes (_add_periodic_connections!
   * single-chunk branch, Chunking.jl:1751-1768; _exchange_halos_local!,
   * Chunking.jl:2138-2172).  The E copy is taken before the χ3 correction:
   * exchange_halos!(:E) ends step_E_fused! (Kernels.jl:452), which step!
   * calls before step_chi3_correction! (Kernels.jl:76-79).  0 = zero ghost
   * walls on every side. */
  int32_t periodic;
} kh_sim_desc;

/* CPML stage semantics.
 * KH_SEM_REFERENCE_CPU: the reference's CPU (KernelAbstractions) path:
 *   generic_curl!/update_field_generic dispatch on the auxiliaries each
 *   PML-grid chunk allocates (Helpers.jl:39-366, Chunking.jl:1069-1146).  Where
 *   a chunk has no U array the σ_prev stage is skipped (Helpers.jl:208-223);
 *   with PML on any axis this makes the CPML grow without bound.
 * KH_SEM_CPML: the stage logic of the reference's CUDA PML kernels
 *   (_cuda_pml_BH_kernel!/_cuda_pml_DE_kernel!, CUDAKernels.jl:126-427): U
 *   (σ_next), T (σ_prev) and W (σ_own) stages each applied whenever their axis
 *   is PML in the cell's chunk; stable and absorbing. */
#define KH_SEM_REFERENCE_CPU 0
#define KH_SEM_CPML 1

/* ADE coefficients of one Lorentz/Drude pole (Susceptibility.jl:60-85). */
typedef struct {
  double gamma1_inv;
  double gamma1;
  double omega0_dt_sq;
  double sigma_omega0_dt_sq;
  double drude_coeff;
  int32_t is_drude;
} kh_pole_coeffs;

/* One source component (one SourceData entry, Sources.jl:44-92). */
typedef struct {
  int32_t component;   /* KH_EX..KH_HZ                                         */
  int32_t start[3];    /* 0-based cell of amplitude element (0,0,0)
                          (= GridVolume.start_idx - 1)                          */
  int32_t dims[3];     /* amplitude array extent                              */
  const double* amp;   /* complex amplitudes, interleaved, x fastest           */
  int32_t time_kind;   /* KH_TIME_*                                            */
  double fcen;         /* Gaussian / CW centre frequency                       */
  double width;        /* Gaussian width (1/fwidth_in)                         */
  double peak_time;    /* Gaussian peak time                                   */
  double cutoff;       /* Gaussian cutoff, or the TABLE source's end_time      */
  int64_t table_len;   /* KH_TIME_TABLE: number of steps tabulated             */
  const double* table; /* KH_TIME_TABLE: 2 complex values per step n:
                          f(nΔt) then f(nΔt+Δt/2), interleaved                  */
} kh_source_desc;

/* Geometry objects of kh_sim_set_geometry (GeometryPrimitives shapes the
 * reference paints, src/Geometry.jl:156-250): */
#define KH_SHAPE_BALL 0     /* center, size[0] = radius                        */
#define KH_SHAPE_CUBOID 1   /* axis-aligned box: center, size[0..2]             */
#define KH_SHAPE_CYLINDER 2 /* center, size[0] = radius, size[1] = height, axis */

/* Subpixel smoothing modes (src/Geometry.jl:795-990). */
#define KH_SMOOTH_NONE 0
#define KH_SMOOTH_VOLUME 1       /* VolumeAveraging: ε̄ = f·ε₁ + (1−f)·ε₂            */
#define KH_SMOOTH_ANISOTROPIC 2  /* AnisotropicSmoothing (Farjadpour et al. 2006) */

typedef struct {
  int32_t shape;     /* KH_SHAPE_*                                  */
  int32_t axis;      /* cylinder axis 0..2                          */
  double center[3];
  double size[3];
  double eps;        /* isotropic relative permittivity of the object */
} kh_object;

/* Library and device information. */
const char* kh_version(void);
/* Device allocations the library has made in this process, over all devices
 * (each request to its stream-ordered memory pool counts one).  Diagnostic
 * with no counterpart in the reference: lets a caller check that a call
 * allocates nothing. */
kh_status kh_device_alloc_count(int64_t* out);
kh_status kh_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* Lifecycle. */
kh_status kh_sim_create(const kh_sim_desc* desc, kh_sim** out);
void kh_sim_destroy(kh_sim* sim);
const char* kh_last_error(const kh_sim* sim);

/* Set-up (before kh_sim_prepare). */
kh_status kh_sim_set_material(kh_sim* sim, int32_t kind, int32_t comp, const double* values);
/* kh_sim_set_material for an array in its own precision (dtype KH_F32 or
 * KH_F64), the way GeometryData holds ε_inv_x … σD in the run's type T
 * (src/DataStructures.jl:214-242), so a Float32 run hands its arrays over
 * without a conversion pass.  Same layout (Center range, x fastest).
 * KH_MAT_EPS_INV and KH_MAT_MU_INV are not copied here: the library reads
 * `values` during kh_sim_prepare, with one host-to-device copy straight from
 * it (a DMA when the array is pinned) and the conversion, if the precisions
 * differ, on the device; the caller keeps the array valid and unchanged until
 * kh_sim_prepare returns (for a simulation handed to kh_server_submit: until
 * the request has been prepared).  The other kinds are classified on the host
 * and are copied before this call returns. */
kh_status kh_sim_attach_material(kh_sim* sim, int32_t kind, int32_t comp, const void* values, int32_t dtype);
kh_status kh_sim_add_pole(kh_sim* sim, const kh_pole_coeffs* coeffs, const double* sigma);
kh_status kh_sim_add_source(kh_sim* sim, const kh_source_desc* src);
kh_status kh_sim_add_dft_monitor(kh_sim* sim, int32_t component, const int32_t start[3],
                                 const int32_t dims[3], int32_t nfreq, const double* freqs,
                                 int32_t decimation, int32_t* out_id);
kh_status kh_sim_prepare(kh_sim* sim);

/* Per-voxel ε⁻¹ of all three E components computed on the device at
 * kh_sim_prepare from a list of objects (replaces init_geometry's host
 * rasterisation and _apply_subpixel_smoothing!, src/Geometry.jl:450-664,
 * 795-990).  Each component samples the objects at its own Yee position
 * origin + (i, j, k)·Δ + shift_c (shift of Ex (0, −Δy/2, −Δz/2), Ey
 * (−Δx/2, 0, −Δz/2), Ez (−Δx/2, −Δy/2, 0), src/utils.jl:139-170), `origin` being
 * the centre of cell (0,0,0); the first object containing the point wins
 * (objects are painted in reverse order, Geometry.jl:223-250); points in no
 * object get background_eps.  `smoothing` = KH_SMOOTH_* then averages
 * interface voxels (a voxel whose value differs from a face neighbour's)
 * with the fill fraction of the nearest object surface.  Before prepare; it
 * takes the place of kh_sim_set_material(KH_MAT_EPS_INV, ...).  The objects
 * are copied; at most 65536. */
kh_status kh_sim_set_geometry(kh_sim* sim, const kh_object* objects, int32_t n, double background_eps,
                              const double origin[3], int32_t smoothing);
/* Read back a per-voxel material array (Center range, x fastest): the
 * kh_sim_set_material kinds; after prepare. */
kh_status kh_sim_read_material(kh_sim* sim, int32_t kind, int32_t comp, double* out);

/* Time stepping: nsteps full steps of step!(sim) on `stream`. */
kh_status kh_sim_step(kh_sim* sim, int64_t nsteps, void* stream);
/* Block until the steps queued on this simulation (on any stream) have
 * finished; KH_ERR_TIMEOUT if a kernel gave up a bounded wait. */
kh_status kh_sim_synchronize(kh_sim* sim);
kh_status kh_sim_timestep(const kh_sim* sim, int64_t* out);
kh_status kh_sim_sources_active(const kh_sim* sim, int32_t* out);
/* Kernel launches issued since creation (fused half-step + DFT launches). */
kh_status kh_sim_launch_count(const kh_sim* sim, int64_t* out);
/* Step batches issued by replaying a captured CUDA graph
 * (_try_capture_graphs!, src/Kernels/Kernels.jl:99-145).  kh_sim_step issues
 * its steps in batches whose boundaries sit on multiples of the monitors'
 * decimation; each batch is captured once per distinct launch sequence
 * (sources on/off, DFT steps, table buffer) and replayed afterwards.
 * KHRONOS_GB300_GRAPHS=0 in the environment at prepare turns this off;
 * timed steps and steps that record history monitors are never captured. */
kh_status kh_sim_graph_replays(const kh_sim* sim, int64_t* out);

/* Results. */
kh_status kh_sim_get_field(kh_sim* sim, int32_t component, double* out);

/* A field component in place on the device, without a copy: element
 * (i, j, k) of the component's dims (the Center range plus the staggered
 * N+1 layer, as kh_sim_get_field) sits at
 *   data + i·strides[0] + j·strides[1] + k·strides[2]   (strides in elements),
 * of type dtype (KH_F32 / KH_F64).  Index −1 of every axis is the zero ghost
 * layer, so the view shifted by one cell per axis is the reference's raw
 * layout (ghost at raw index 1, interior at 2:N+1, Fields.jl:130-141); the
 * block holds at least (dims[2] + 1)·strides[2] elements from the ghost cell
 * (−1, −1, −1), so a dense wrapper of that extent starting there is in
 * bounds.  Along an axis without the staggered layer, index dims is the high
 * ghost layer too; along a staggered axis the N+1 layer sits on it and
 * nothing lies beyond.  The memory belongs to the simulation: valid until
 * kh_sim_destroy, its values current once the steps queued on it have
 * finished (kh_sim_synchronize, or an event on the stepping stream).
 * Writes through it change the simulation; values at cells that keep B/D
 * state (CPML, source, χ3, pole cells) are recomputed from that state at the
 * next step.  The zero-copy counterpart of the reference's fields
 * (sim.fields.fEx … as device arrays, DataStructures.jl:100-148) for
 * device-side post-processing; a Julia shim wraps it with unsafe_wrap and a
 * strided view. */
typedef struct {
  void* data;
  int32_t dtype;
  int32_t dims[3];
  int64_t strides[3];
} kh_field_view;
kh_status kh_sim_field_view(kh_sim* sim, int32_t component, kh_field_view* out);
kh_status kh_sim_read_dft(kh_sim* sim, int32_t monitor_id, double* out);
kh_status kh_sim_monitor_info(const kh_sim* sim, int32_t monitor_id, int32_t dims[3], int32_t* nfreq);
/* Poynting flux of four DFT monitors (E1, E2, H1, H2 tangential), FP64 on the
 * device: S(f) = Σ Re(E1·H2* − E2·H1*)·dA after averaging the two normal layers. */
kh_status kh_sim_flux(kh_sim* sim, const int32_t ids[4], int32_t normal_axis, double dA,
                      double* out);
/* kh_sim_flux without any device allocation (no counterpart in the reference).
 * For callers that must not allocate device memory while they run:
 * kh_sim_flux takes its per-frequency buffer from the library's device memory
 * pool, and a process whose device memory is fully committed to its
 * simulations may have nothing left for even that small allocation (nor may
 * code that forbids allocations inside its own critical sections).  The
 * per-frequency sums and the reduction's partial sums go to a fixed device
 * array inside the library instead:
 * at most 4096 frequencies (more returns KH_ERR_INVALID; use kh_sim_flux).
 * The first call on each device does a one-time set-up (it resolves that
 * array's device address with the device current); make it before any
 * stream capture begins.  The resolved address is kept for the life of the
 * process: it does not survive cudaDeviceReset (or any other teardown of the
 * device's primary context), after which this entry point must not be used
 * on that device.  kh_device_alloc_count shows that it allocates nothing.  The array is shared by all simulations of the
 * process on a device and keeps the last call's values: calls that overlap
 * on one device (from several host threads) race on it, so serialise them.
 * Same result as kh_sim_flux. */
kh_status kh_sim_flux_static(kh_sim* sim, const int32_t ids[4], int32_t normal_axis, double dA,
                             double* out);

/* ---------------------------------------------------------------------------
 * Adjoint (inverse design) support.  Replaces the reference's host-side
 * adjoint machinery (src/Adjoint/*.jl) behind its OptimizationProblem /
 * ChainRules rrule:
 *
 *   kh_sim_update_material_box   update_design! + reset_fields! per new design
 *                                (src/Adjoint/DesignRegion.jl, OptimizationProblem.jl:87-93)
 *   kh_sim_update_source         swapping in the adjoint sources of
 *                                adjoint_run! (OptimizationProblem.jl:237-277,
 *                                place_adjoint_source ObjectiveQuantities.jl:290-345)
 *   kh_sim_dft_overlap           evaluate(::FourierFieldsObjective) and the
 *                                objective's field overlap (ObjectiveQuantities.jl:282-288)
 *   kh_adjoint_accumulate        calculate_gradient! (src/Adjoint/GradientKernel.jl:35-109)
 *
 * The adjoint run is a forward run of the same kernels with sources on the
 * objective monitor's cells (Yee-scheme reciprocity: the transfer from a
 * current source at a to the E field at b equals that from b to a), so no
 * time history is stored: the gradient needs only the forward and adjoint DFT
 * fields on the design voxels.
 * ------------------------------------------------------------------------- */

/* Overwrite per-voxel ε⁻¹ (kind KH_MAT_EPS_INV) or μ⁻¹ (KH_MAT_MU_INV) of one
 * component in the cell box start..start+dims-1 after kh_sim_prepare; values
 * x fastest over the box.  The array must have been set with
 * kh_sim_set_material before prepare.  Waits for this simulation's queued
 * steps.  Pair it with kh_sim_reset for a new design. */
kh_status kh_sim_update_material_box(kh_sim* sim, int32_t kind, int32_t comp, const int32_t start[3],
                                     const int32_t dims[3], const double* values);

/* Replace, after kh_sim_prepare, the amplitudes of source `index` (the order
 * of kh_sim_add_source; complex interleaved over its dims, NULL = keep) and,
 * for a KH_TIME_TABLE source, its table (table_len steps, layout of
 * kh_source_desc.table; NULL = keep) and end time `cutoff`.  The cells a
 * source injects into are fixed at prepare (its nonzero amplitudes): a
 * nonzero amplitude elsewhere returns KH_ERR_INVALID.  Waits for this
 * simulation's queued steps.  The sources-active flag is not touched: call
 * kh_sim_reset before running the new sources from t = 0. */
kh_status kh_sim_update_source(kh_sim* sim, int32_t index, const double* amp, int64_t table_len,
                               const double* table, double cutoff);

/* out[f] = Σ_cells weights[cell, f] · F[cell, f] over DFT monitor
 * `monitor_id`, FP64 on the device (fixed reduction order).  weights and out
 * are complex interleaved host arrays; weights has the monitor's layout
 * (cell x fastest over its box, frequency slowest; dims × nfreq values), out
 * nfreq values. */
kh_status kh_sim_dft_overlap(kh_sim* sim, int32_t monitor_id, const double* weights, double* out);

/* Adjoint gradient reduction, FP64 on the device, accumulated into the host
 * array grad (one double per design voxel, x fastest over the design box):
 *   grad[v] += Re(coef · Σ_{c=x,y,z} F_c[v, fwd_freq] · A_c[v, adj_freq])
 * F_c: the forward run's DFT monitors fwd_ids[c] of E_c over the design box;
 * A_c: the adjoint run's monitors adj_ids[c] over the same box.  With coef =
 * −2·conj(∂J/∂Y)/Ŝ (Ŝ the adjoint source's DFT at that frequency) each call
 * adds one frequency's ∂J/∂ε per voxel (summed over the three components of
 * an isotropic voxel).  Both simulations must have the same precision. */
kh_status kh_adjoint_accumulate(kh_sim* fwd, const int32_t fwd_ids[3], int32_t fwd_freq, kh_sim* adj,
                                const int32_t adj_ids[3], int32_t adj_freq, double coef_re,
                                double coef_im, double* grad);

/* History monitor: records `component` over the cell box start..start+dims-1
 * after its half-step of every step n < capacity_steps, into a device buffer
 * of capacity_steps × box cells (values of the run's precision).  Before
 * kh_sim_prepare.  No counterpart in the reference, which keeps only DFT
 * monitors; it is the forward/adjoint field record of the windowed adjoint
 * (kh_history_correlate).  kh_sim_reset restarts recording at step 0. */
kh_status kh_sim_add_history_monitor(kh_sim* sim, int32_t component, const int32_t start[3],
                                     const int32_t dims[3], int64_t capacity_steps, int32_t* out_id);
/* One recorded step of a history monitor (box cells, x fastest) as doubles. */
kh_status kh_sim_read_history(kh_sim* sim, int32_t history_id, int64_t step, double* out);

/* Windowed adjoint reduction, FP64 on the device, accumulated into the host
 * array grad (one double per box cell, x fastest):
 *   grad[v] += coef · Σ_{c=x,y,z} Σ_{m<nsteps} F_c[m, v] · A_c[nsteps−1−m, v]
 * F_c: the forward run's history monitors fwd_ids[c] (E_c over the design
 * box); A_c: the adjoint run's history monitors over the same box, the
 * adjoint being driven by the time-reversed objective weights.  Exact for a
 * finite run (the DFT form of kh_adjoint_accumulate needs decayed fields).
 * Replaces calculate_gradient! (src/Adjoint/GradientKernel.jl:35-109) for
 * that case.  Both histories must hold at least nsteps steps. */
kh_status kh_history_correlate(kh_sim* fwd, const int32_t fwd_ids[3], kh_sim* adj, const int32_t adj_ids[3],
                               int64_t nsteps, double coef, double* grad);

/* Squared L2 norms Σ E_c² (out[0..2]) and Σ H_c² (out[3..5]) over the grid,
 * FP64 on the device: the field decay that stop_when_dft_decayed
 * (src/Simulation.jl:411-485) tracks through DFT norms, and a finiteness
 * check (a non-finite field gives a non-finite norm). */
kh_status kh_sim_field_sq_norms(kh_sim* sim, double out[6]);

/* L2 norm sqrt(Σ|F|²) of each DFT monitor's accumulated array (all cells and
 * frequencies), FP64 on the device, out[id] for id = 0 .. monitors−1:
 * dft_fields_norm (src/Simulation.jl:530-539), the quantity
 * stop_when_dft_decayed tracks (src/Simulation.jl:411-485). */
kh_status kh_sim_dft_norms(kh_sim* sim, double* out);

/* KH_OK while every E and H value is finite, KH_ERR_NAN (the message names
 * the first non-finite component) once a run has diverged, e.g. a time step
 * above the Courant limit.  One FP64 norm pass over the fields; the step
 * loop itself never checks, as the reference's run loop does not
 * (src/Simulation.jl:295-382). */
kh_status kh_sim_check_finite(kh_sim* sim);

/* Bounds-checked builds of the library (compiled with KH_DEBUG_BOUNDS, a
 * stand-in for a memory sanitizer): every global and shared-memory index of
 * the step kernels (half-steps, source terms, DFT, history recording) is
 * tested against its array's extent; a violating access is skipped and
 * recorded.  Returns (and clears) the number of violations since the last
 * call, with the first one's index and site code.  KH_ERR_UNSUPPORTED from
 * the regular build.  No counterpart in the reference. */
kh_status kh_debug_bounds(int64_t* count, int64_t* index, int32_t* site);

/* Device memory: what kh_sim_prepare will allocate (estimate, available
 * before prepare; estimate_memory, src/Memory.jl:120-251) and what it has
 * allocated (0 before prepare). */
kh_status kh_sim_memory_bytes(const kh_sim* sim, int64_t* estimate, int64_t* allocated);

/* State control. */
kh_status kh_sim_reset(kh_sim* sim);
kh_status kh_sim_state_bytes(const kh_sim* sim, int64_t* out);
kh_status kh_sim_export_state(kh_sim* sim, void* host_dst, int64_t bytes);
kh_status kh_sim_import_state(kh_sim* sim, const void* host_src, int64_t bytes);

/* Compulsory-traffic model of one full step (bytes): the reference's 9 + 12
 * words per cell (benchmark/benchmark_metrics.jl:236-241) plus CPML
 * auxiliaries, dispersive and χ3 terms, plus DFT monitor traffic amortised
 * over the decimation.  The split gives the H half-step kernel, the E
 * half-step kernel and the DFT launches separately. */
kh_status kh_sim_model_bytes_per_step(const kh_sim* sim, double* out);
kh_status kh_sim_model_bytes_split(const kh_sim* sim, double* h_half, double* e_half,
                                   double* dft);

/* kh_sim_step with CUDA events recorded on `stream` around the launch groups
 * (H half-step, E half-step, DFT) of every 8th step of the call (its first
 * step included); returns the device time (ms) of the H half-step kernels, the E
 * half-step kernels and the DFT launches of these nsteps, the sampled steps'
 * sums scaled to all nsteps.  No step-graph replay in timed runs. */
kh_status kh_sim_step_timed(kh_sim* sim, int64_t nsteps, void* stream, double* h_ms,
                            double* e_ms, double* dft_ms);

/* ---------------------------------------------------------------------------
 * Request server (continuous batching of independent simulations on one GPU).
 * Replaces run_batch / run_batch_concurrent / plan_batch (src/Batch.jl:21-263)
 * and the admission estimate of estimate_memory (src/Memory.jl:120-251):
 * requests are admitted in arrival order whenever the device-memory budget and
 * a resident slot allow, prepared on an admission thread while other requests
 * step, and stepped in quanta on per-slot streams so their kernels overlap.
 *
 * Ownership: kh_server_submit takes a created, configured, NOT prepared
 * kh_sim; from then on the server owns it.  When kh_server_wait reports the
 * request finished, its results are read with the kh_sim_* calls on the same
 * handle; kh_server_release then destroys it and frees its budget.  Requests
 * that are never released keep their memory (and budget) until
 * kh_server_destroy.
 * ------------------------------------------------------------------------- */
typedef struct kh_server kh_server;

enum {
  KH_REQ_QUEUED = 0,    /* submitted, waiting for budget or a slot */
  KH_REQ_ADMITTED = 1,  /* being prepared / waiting for the stepping thread */
  KH_REQ_RUNNING = 2,
  KH_REQ_DONE = 3,
  KH_REQ_FAILED = 4,
  KH_REQ_RELEASED = 5
};

typedef struct {
  int64_t budget_bytes;  /* device bytes the admitted, unreleased requests may hold */
  int32_t max_resident;  /* requests prepared and stepping at once (0: 16) */
  int32_t quantum_steps; /* steps issued per request per scheduling round (0: 64) */
} kh_server_desc;

typedef struct {
  int32_t state;   /* KH_REQ_* */
  int32_t status;  /* kh_status of a finished request */
  int64_t steps;   /* steps requested */
  int64_t bytes;   /* device bytes: estimate until admitted, then allocated */
  double t_submit, t_admit, t_start, t_done; /* seconds since kh_server_create; -1 = not yet */
} kh_request_info;

kh_status kh_server_create(const kh_server_desc* desc, kh_server** out);
/* Queue `sim` for nsteps steps; returns its ticket.  KH_ERR_OOM if its
 * estimated bytes exceed the whole budget. */
kh_status kh_server_submit(kh_server* s, kh_sim* sim, int64_t nsteps, int64_t* ticket);
/* Wait until the request finished (timeout_s < 0: no limit); returns the
 * request's status, or KH_ERR_TIMEOUT if it is still running. */
kh_status kh_server_wait(kh_server* s, int64_t ticket, double timeout_s);
/* Completion queue: the ticket of a finished request not reported before
 * (each finished request is reported once); KH_ERR_TIMEOUT if none finishes
 * within timeout_s (< 0: no limit). */
kh_status kh_server_wait_any(kh_server* s, double timeout_s, int64_t* ticket);
kh_status kh_server_info(kh_server* s, int64_t ticket, kh_request_info* out);
kh_status kh_server_release(kh_server* s, int64_t ticket);
kh_status kh_server_stats(kh_server* s, int64_t* queued, int64_t* resident, int64_t* budget_used);
const char* kh_server_last_error(const kh_server* s);
/* Stops admitting and issuing, waits for the work in flight, destroys every
 * request's simulation that was not released. */
void kh_server_destroy(kh_server* s);

#ifdef __cplusplus
}
#endif

#endif /* KHRONOS_GB300_H */
