// Shared declarations between the sm_103a kernels (kh_kernels.cu) and the
// host-side C-ABI implementation (kh_sim.cu).
//
// Device layout of every full-domain array (fields, materials, auxiliaries):
//   element (i, j, k), -1 <= i,j,k <= n, lives at
//     origin + (k * (ny + 2) + j) * pitch + i
//   with origin = ((ny + 2) + 1) * pitch + XOFF and XOFF = 32 bytes of
//   elements (xoff<T>()), so x = 0 of every row starts a 32-byte sector (a
//   row segment of 64 cells covers whole sectors) and the row pitch is a
//   multiple of 128 bytes.  The ring i,j,k in {-1, n} (and the row padding)
//   is never written: it is the reference's zero ghost layer / staggered wall.
#pragma once

#include <cuda.h>  // CUtensorMap (descriptors are encoded through the runtime's driver entry point)

#include <cstdint>

namespace kh {

#ifndef KH_XOFF_BYTES
#define KH_XOFF_BYTES 32
#endif
// Elements before x = 0 in every padded row (see the layout above).
template <typename T>
constexpr int xoff() {
  return KH_XOFF_BYTES / int(sizeof(T));
}

constexpr int kMaxPoles = 4;
constexpr int kBlockY = 4;      // rows per CTA
#ifndef KH_PLANES_PER_CTA
#define KH_PLANES_PER_CTA 16
#endif
constexpr int kPlanesPerCta = KH_PLANES_PER_CTA;
// Resident CTAs per SM the half-step kernels are compiled for (caps registers
// at 65536 / (kMinBlocks · 32 · kBlockY)).
#ifndef KH_MIN_BLOCKS
#define KH_MIN_BLOCKS 4
#endif
constexpr int kMinBlocks = KH_MIN_BLOCKS;

// cell_class bits (full-domain uint32 array, read only inside flagged tiles)
constexpr uint32_t kSpecialE = 1u << 0;  // D-state kept: E source, χ3 or pole
constexpr uint32_t kSpecialH = 1u << 1;  // B-state kept: H source
constexpr uint32_t kHasChi3 = 1u << 2;
constexpr uint32_t kHasPole = 1u << 3;
constexpr uint32_t kHasSrcE = 1u << 4;
constexpr uint32_t kHasSrcH = 1u << 5;
constexpr int kSlotShift = 8;            // source slot index in the upper 24 bits

// Bounds-checked builds (-DKH_DEBUG_BOUNDS, a stand-in for a memory
// sanitizer): every global and shared-memory index of the step kernels is
// tested against its array's extent before the access; a violation is
// counted, the first one's site and index recorded, and the access skipped
// (loads read 0).  No trap and no wait.  Each translation unit has its own
// record word, read back by kh_debug_bounds.  In other builds KH_IN is the
// constant true and the kernels are unchanged.
#ifdef KH_DEBUG_BOUNDS
struct DbgWord {
  unsigned long long count;
  long long index;
  int site;
};
static __device__ DbgWord kh_dbg;
__device__ __forceinline__ bool dbg_in(long long idx, long long n, int site) {
  if (idx >= 0 && idx < n) return true;
  if (atomicAdd(&kh_dbg.count, 1ull) == 0ull) {
    kh_dbg.index = idx;
    kh_dbg.site = site;
  }
  return false;
}
#define KH_IN(idx, n, site) ::kh::dbg_in((long long)(idx), (long long)(n), (site))
// Host side: read (and clear) this translation unit's record word.
#define KH_DBG_READER(name)                                                              \
  void name(unsigned long long* count, long long* index, int* site) {                   \
    DbgWord w{};                                                                         \
    cudaMemcpyFromSymbol(&w, kh_dbg, sizeof(w));                                         \
    *count = w.count;                                                                    \
    *index = w.index;                                                                    \
    *site = w.site;                                                                      \
    const DbgWord z{};                                                                   \
    cudaMemcpyToSymbol(kh_dbg, &z, sizeof(z));                                           \
  }
void dbg_read_tma(unsigned long long* count, long long* index, int* site);
void dbg_read_kernels(unsigned long long* count, long long* index, int* site);
#else
#define KH_IN(idx, n, site) true
#endif

// Row alignment unit of the layout: 16 bytes of the run's type.
template <typename T>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int N = 4;
};
template <>
struct Vec<double> {
  static constexpr int N = 2;
};

template <typename T>
struct PoleParams {
  T gamma1_inv, gamma1, coeff_p, drive;  // drive = sigma_omega0_dt_sq or drude_coeff
  int is_drude;
  const T* sigma;
  T* P[3];
  T* Pprev[3];
};

template <typename T>
struct Cplx {
  T re, im;
};

// CPML coefficients of one cell along one axis: the σ sample and the factors
// of update_field_from_curl ((1-σ)·A + B)/(1+σ) (Helpers.jl:30-33) with the
// division replaced by a multiplication with 1/(1+σ).
template <typename T>
struct AxisCoef {
  T s;    // σ (already scaled by Δt/2)
  T om;   // 1 - σ
  T ir;   // 1 / (1 + σ)
  T op;   // 1 + σ
};

// Source slot with a single entry, packed for one load (src < 0: the slot
// has several entries and takes the general entry loop).
template <typename T>
struct alignas(16) SlotPack {
  int src;       // source index (into f_now)
  int comp;      // component 0..5
  Cplx<T> amp;   // complex amplitude
};

// Parameters of one fused half-step launch.
template <typename T>
struct HalfStepParams {
  int nx, ny, nz;
  long long pitch, plane, origin;
  long long total;  // elements of every padded full-domain array
  int nxb;  // x tiles of 32*VN cells
  int full; // 1: cells with sources/χ3/poles/conductivity handled in-kernel (FULL variant)
  int zplanes;  // z planes marched by one CTA of the TMA-staged kernel
  int xprefetch;   // TMA-staged kernel, x-CPML state into L2: 0 tile-wide (H half), 1 per lane (H), 2 per lane (H, E)
  int xpf_dist;    // planes ahead of the per-lane x-CPML prefetch
  T dt, inv_d[3];
  T cd[3];  // Δt·(1/Δ_a): curl coefficients of the TMA-staged kernel

  const T* A[3];  // curl source field (E for the H half, H for the E half)
  T* O[3];        // updated field (H or E)
  T* Ts[3];       // B or D state where kept (nullptr if no cell keeps it)
  T* U[3];        // CPML U auxiliaries (nullptr if none)
  T* W[3];        // CPML W auxiliaries
  T* C[3];        // conductivity cascade C
  const T* m_inv[3];  // per-voxel μ⁻¹ / ε⁻¹ or nullptr
  T m_scalar;
  const T* msig[3];   // material conductivity σB / σD or nullptr
  const AxisCoef<T>* ax[3];  // CPML coefficients per axis at cell centres (length n_a)
  int pml_lo[3], pml_hi[3];
  int cpml;                    // 1: CUDA-path CPML stages, 0: CPU-path dispatch
  uint32_t sigma_region_mask;  // bit r (r = rx + 3 ry + 9 rz) set: region has conductivity

  // per (k/64, j, xb): bit k%64 set when that plane's row segment of 32·VN
  // cells holds special cells of this half
  const uint64_t* tile_bits;
  long long n_tile_words;     // entries of tile_bits
  const uint32_t* cell_class; // per cell

  // sources (folded into the half-step)
  int sources_active;
  const int* slot_off;        // slot -> [slot_off[s], slot_off[s+1]) entries
  const int* ent_src;         // source index of entry
  const int* ent_comp;        // component 0..2 within this half
  const Cplx<T>* ent_amp;     // complex amplitude of entry
  const Cplx<T>* f_now;       // per source: time factor f(t) of this half-step
  int n_slots, n_ent, n_src;  // extents of slot_off (n_slots + 1), ent_*, f_now

  // E half only
  const T* chi3;
  int npoles;
  PoleParams<T> poles[kMaxPoles];

  // bit a set: axis a is periodic.  E half: a χ3 cell on a wrap face stores
  // its pre-correction E into the ghost layer the wrap fills (the reference
  // exchanges E before the Kerr correction); the wrap kernel skips those cells.
  uint32_t periodic;

  int* err;  // set to KH_ERR_TIMEOUT by a kernel whose bounded wait gave up
  // Failure-detection test hook (0 in normal runs): nonzero launches the FP32
  // LEAN TMA kernels' test instantiation, whose first ring stage expects 16
  // bytes that never arrive, so its waits give up after 4096 polls.
  uint32_t stall_tx;
};

// TMA-staged half-step: tile of kTmaX × kTmaY cells per CTA (one warp per
// row, 2 cells per lane), kTmaStages-deep shared-memory ring per CTA.  Three
// stages (31 KB per FP32 CTA) keep five CTAs per SM, as four did, and leave
// the SM more of its unified L1 for the per-thread CPML state loads: 2 %
// faster than four, five (four CTAs per SM) 7 % slower.
#ifndef KH_TMA_ROWS
#define KH_TMA_ROWS 4
#endif
#ifndef KH_TMA_STAGES
#define KH_TMA_STAGES 3
#endif
#ifndef KH_TMA_MIN_BLOCKS
#define KH_TMA_MIN_BLOCKS 5
#endif
constexpr int kTmaX = 64;
constexpr int kTmaY = KH_TMA_ROWS;
constexpr int kTmaStages = KH_TMA_STAGES;
constexpr int kTmaMinBlocks = KH_TMA_MIN_BLOCKS;

// Tensor maps of one half-step over the padded layout (x = pitch, y = ny+2,
// z = nz+2): the curl-source arrays with a box of (kTmaX + 16 bytes) ×
// (kTmaY + 1) × 1 (x and y halo on the side the curl reads), the updated
// arrays and the per-voxel m⁻¹ with a box of kTmaX × kTmaY × 1.
struct alignas(128) TmaMaps {
  CUtensorMap a[3];
  CUtensorMap o[3];
  CUtensorMap m[3];
  // B|D state and CPML U, W (maps of the arrays that exist; box kTmaX × kTmaY),
  // used for L2 prefetch only
  CUtensorMap t[3];
  CUtensorMap u[3];
  CUtensorMap w[3];
};

template <typename T>
size_t tma_smem_bytes();

// Geometry set-up (kh_geometry.cu): one object with its bounding box.
struct GeomObj {
  int shape, axis;
  double c[3], s[3];
  double eps;
  double lo[3], hi[3];
};

// One component's rasterisation (+ smoothing) over the padded layout.
struct GeomArgs {
  const GeomObj* objs;  // device array
  int nobj;
  int n[3];
  long long pitch, plane, origin, total;
  double org[3];        // this component's position of cell (0,0,0)
  double d[3];
  double background;
  int smoothing;        // KH_SMOOTH_*
  int comp;             // 0..2 (anisotropic projection)
};

template <typename T>
void launch_geometry(const GeomArgs& a, T* eps_inv, T* scratch, void* stream);

template <typename T>
void launch_half_step_tma(bool h_half, const HalfStepParams<T>& p, const TmaMaps& maps, void* stream);

// Kernel attribute set-up (dynamic shared memory size), once per device.
template <typename T>
int prepare_tma_kernels();

// CTAs of the TMA-staged kernel resident on one SM (after prepare_tma_kernels).
template <typename T>
int tma_resident_ctas();

// History recording: copy one component over a cell box (x fastest) into a
// contiguous slot of a history buffer.
template <typename T>
struct RecordParams {
  const T* field;
  long long pitch, plane, origin, total;
  int start[3], dims[3];
  T* dst;
};

template <typename T>
void launch_record(const RecordParams<T>& p, void* stream);

template <typename T>
struct DftParams {
  const T* field;
  long long pitch, plane, origin, total;
  int start[3], dims[3];
  int nf;
  const Cplx<T>* phase;  // nf entries: Δt·exp(i 2π f t)
  Cplx<T>* F;            // (cells, nf) accumulators, cell-major per frequency
  Cplx<T>* comp;         // Kahan compensation (FP32) or nullptr
};

// Cells per thread along x in the half-step kernels (8-byte FP32 / 16-byte
// FP64 vectors; a 320-cell row is 5 full warps).
constexpr int kVN = 2;

// Sparse source application for cells the LEAN kernel updated as B|D-keeping
// cells: O = m⁻¹·(T + S) with S = Σ real(f(t)·amplitude) (Helpers.jl:329-332,
// Sources.jl:346-357).  Exact when the cell has no W stage for the component
// and no χ3/pole, which the host checks before choosing this path.  One
// thread per source cell; a cell with a single entry reads it packed.
template <typename T>
struct SourceFixParams {
  int nslots, n_ent, n_src;
  long long total;
  const long long* slot_cell;  // cell offset of each slot
  const SlotPack<T>* slot_pack;
  const int* slot_off;
  const int* ent_src;
  const int* ent_comp;         // 0..5
  const Cplx<T>* ent_amp;
  const Cplx<T>* f_now;
  T* O[3];
  const T* Ts[3];
  const T* m_inv[3];
  T m_scalar;
  int h_half;
  // CUDA-path CPML: a sourced component whose own axis is PML at the cell
  // has a W stage (update_field_generic, Helpers.jl:333-339).  The LEAN launch
  // stored w = m⁻¹·T and O = (O_old + (1+σ)·w) − (1−σ)·w_old; with the source
  // w becomes m⁻¹·(T + S), so O moves by (1+σ)·Δw.
  T* W[3];
  const AxisCoef<T>* ax[3];
  int n[3], pml_lo[3], pml_hi[3];
  long long pitch, plane, origin;
};

// Dispersive and Kerr cells of a LEAN E half-step (the launch kept their D
// state, E = ε⁻¹·D): over the z planes [k0, k1) that hold such cells, a pole
// cell gets E = ε⁻¹·(D − Σ_p P_p), a χ3 cell the Kerr correction, then every
// pole its ADE update with E^{n+1} — the order and arithmetic of the general
// cell update (step_curl_and_update!, step_chi3_correction!,
// step_polarization!; Kernels.jl:76-83).  Pole cells lie outside the CPML
// (the ADE σ is zeroed there), χ3 cells may lie inside it.
template <typename T>
struct DispFixParams {
  int nx, ny, nz;
  long long pitch, plane, origin, total;
  int nxb;                      // row segments of 32·kVN cells per row
  // row segments that hold χ3 or pole cells, in grid order: segment index
  // ((k·ny + j)·nxb + xb), bit 31 set when the segment holds pole cells
  const uint32_t* list;
  int n_list;
  const uint32_t* cell_class;
  const T* chi3;
  const T* D[3];
  T* E[3];
  const T* m_inv[3];
  T m_scalar;
  int npoles;
  PoleParams<T> poles[kMaxPoles];
  // W stage of pole cells in the CPML of their own axis (the LEAN launch
  // applied it without the polarisation): W auxiliaries and axis coefficients
  T* W[3];
  const AxisCoef<T>* ax[3];
  int pml_lo[3], pml_hi[3];
  // source terms of pole cells that are also source cells (a χ3-only source
  // cell already holds ε⁻¹·(D + S) from the source kernel, which runs first)
  int sources_active;
  const int* slot_off;
  const int* ent_src;
  const int* ent_comp;
  const Cplx<T>* ent_amp;
  const Cplx<T>* f_now;
  int n_slots, n_ent, n_src;
};

// DFT accumulation of every monitor of one half-step in one launch
// (update_dft_monitor!, Monitors.jl:361-379, for all monitors updated at this
// step): item t of monitor m (t < ncell·nf, cell fastest) is (cell, f).
constexpr int kMaxDftBatch = 16;
template <typename T>
struct DftBatchParams {
  int n;                             // monitors in this launch
  long long pitch, plane, origin, total;
  long long first[kMaxDftBatch + 1]; // prefix sums of the monitors' items
  struct Mon {
    const T* field;
    int start[3], dims[3];
    int nf;
    const Cplx<T>* phase;            // nf entries: Δt·exp(i 2π f t)
    Cplx<T>* F;
    Cplx<T>* comp;                   // Kahan compensation (FP32) or nullptr
  } mon[kMaxDftBatch];
};

// Periodic wrap of one field group after its half-step (_exchange_halos_local!
// single-chunk connections, Chunking.jl:1751-1768, 2138-2172): for each axis a
// in `periodic` and each component, layer n_a-1 → ghost layer -1 and layer 0 →
// layer n_a, over the Center range 0..n-1 of the other two axes.
template <typename T>
struct WrapParams {
  int n[3];
  long long pitch, plane, origin, total;
  uint32_t periodic;
  int axes[3];  // the periodic axes in order (filled by launch_wrap)
  T* O[3];
  const T* chi3;  // E group: cells with χ3 ≠ 0 already stored their pre-correction value
};

template <typename T>
void launch_half_step(bool h_half, const HalfStepParams<T>& p, void* stream);

template <typename T>
void launch_wrap(const WrapParams<T>& p, void* stream);

template <typename T>
void launch_source_fix(const SourceFixParams<T>& p, void* stream);

template <typename T>
void launch_dft(const DftParams<T>& p, void* stream);

template <typename T>
void launch_dft_batch(const DftBatchParams<T>& p, void* stream);

template <typename T>
void launch_disp_fix(const DispFixParams<T>& p, void* stream);

// ---- set-up kernels (kh_setup.cu) ----
// Compact Center-range array (x fastest) → padded layout, converted to T.
template <typename Tin, typename T>
void launch_scatter_center(const Tin* src, T* dst, const int n[3], long long pitch, long long plane,
                           long long origin, void* stream);

// Cell classes of χ3 and pole cells (ORed into cls) from the device arrays.
template <typename T>
struct ClassifyArgs {
  int n[3];
  long long pitch, plane, origin;
  const T* chi3;                     // nullptr if no χ3 array
  int npoles;
  const T* pole_sigma[kMaxPoles];
  uint32_t* cls;
};
template <typename T>
void launch_classify(const ClassifyArgs<T>& a, void* stream);

// cls[cell[s]] |= bits[s] for s < n (source cells: class bits and slot index).
void launch_mark_cells(const long long* cell, const uint32_t* bits, int n, uint32_t* cls, void* stream);

// Plane bitmasks of special cells per row segment, and CPML-region flags.
struct TileBitsArgs {
  int n[3];
  long long pitch, plane, origin;
  int nxb;
  int lo[3], hi[3];
  const uint32_t* cls;
  unsigned long long* bits_e;
  unsigned long long* bits_h;
  unsigned int* region_flags;  // bit 0: special E cell in a CPML region; bit 1: special H cell
};
void launch_tile_bits(const TileBitsArgs& a, void* stream);

// Row-segment list of the dispersive-cell pass (DispFixParams::list), built
// in grid order on the device: *count entries written to list (capacity
// n[2]·n[1]·nxb), flags is scratch of one byte per segment.
struct DispListArgs {
  int n[3];
  long long pitch, plane, origin;
  int nxb;
  const uint32_t* cls;
  unsigned char* flags;
  uint32_t* list;
  int* count;
};
void launch_disp_list(const DispListArgs& a, void* stream);

// DFT accumulators (with Kahan compensation C, or nullptr) → interleaved
// (re, im) doubles, value = F − C.
template <typename T>
void launch_dft_read(const Cplx<T>* F, const Cplx<T>* C, double* out, long long n, void* stream);

// FP64 flux reduction in two passes with a fixed summation order: blocks of
// 1024 cells per frequency write partial sums into `partial` (room for
// partial_cap doubles, partial_cap >= nf; at most partial_cap / nf blocks per
// frequency), one warp per frequency adds them in block order into out[f].
template <typename T>
void launch_flux(const Cplx<T>* e1, const Cplx<T>* e2, const Cplx<T>* h1, const Cplx<T>* h2,
                 const Cplx<T>* c_e1, const Cplx<T>* c_e2, const Cplx<T>* c_h1,
                 const Cplx<T>* c_h2, const int dims_e1[3], const int dims_e2[3],
                 const int dims_h1[3], const int dims_h2[3], int normal_axis, int nf, double dA,
                 double* out, double* partial, int partial_cap, void* stream);
// Blocks per frequency launch_flux uses for a plane of `cells` cells.
int flux_blocks(long long cells, int nf, int partial_cap);

}  // namespace kh
