// sm_103a kernels of the FDTD step loop.
//
// One fused kernel per half-step replaces the reference's per-chunk dispatch
// (step_H_fused!/step_E_fused!, src/Kernels/Kernels.jl:164-454): the curl,
// the CPML cascade (Helpers.jl:30-270, CUDAKernels.jl:150-281), the
// constitutive update (Helpers.jl:323-409), source injection
// (Sources.jl:346-357) and, on the E half, the χ3 correction
// (Dispersive.jl:127-147) and the ADE pole update (Dispersive.jl:25-88) all
// happen in one pass over the grid.
//
// Work decomposition: a warp owns 32 × VN consecutive x cells of one row and
// marches over kPlanesPerCta z planes; the CTA holds kBlockY rows.  x
// neighbours come from warp shuffles, the z-neighbour plane is carried in
// registers from the previous plane (2.5D register rotation), y neighbours are
// vector loads that hit L1/L2 (the row above belongs to the next warp of the
// same CTA).
//
// Every array a thread needs for its VN cells is loaded as one vector before
// any arithmetic, so a plane costs one memory round trip also in CPML rows.
//
// Which arrays a cell touches is a static property of the cell:
//  * plain cells (no CPML region flag, no source/χ3/pole) keep no B/D state:
//    O += m⁻¹·K.  This equals m⁻¹·(T + K) of the reference up to rounding and
//    is exact when m⁻¹ = 1;
//  * all other cells keep B/D and follow the reference's stage logic for the
//    CPML auxiliaries their region allocates (Chunking.jl:1069-1146).
#include <cuda_runtime.h>

#include <algorithm>

#include "kh_cell.cuh"

namespace kh {

#ifdef KH_DEBUG_BOUNDS
KH_DBG_READER(dbg_read_kernels)
#endif

template <typename T, int VN>
struct PlaneLoads {
  T l0[VN], l1[VN], a2[VN], y0[VN], y2[VN];  // A0/A1 fresh plane, A2, y neighbours
  T xn1, xn2;                                // x neighbours of A1/A2 for the edge lane
  T O[3][VN], m[3][VN];
  T t[3][VN], u[3][VN], w[3][VN], c3[VN];
  uint32_t cls[VN];
  bool tf;                                   // plane's tile holds special cells
};

template <typename T, int VN, bool H, bool FULL>
__device__ __forceinline__ void load_plane(const HalfStepParams<T>& p, PlaneLoads<T, VN>& L, int k,
                                           long long row, int lane, bool lane_ok, bool pervox, bool fy,
                                           bool anyfx, uint64_t tbits) {
  constexpr int s = H ? 1 : -1;
  const long long q = row + (long long)k * p.plane;
  vzero(L.l0); vzero(L.l1); vzero(L.a2); vzero(L.y0); vzero(L.y2);
  L.xn1 = T(0);
  L.xn2 = T(0);
  L.tf = ((tbits >> (k & 63)) & 1ull) != 0;
  const bool fz = k < p.pml_lo[2] || k >= p.nz - p.pml_hi[2];
  const bool anyRegion = fy || fz || anyfx;
  const bool axis_any[3] = {anyfx, fy, fz};
  if (lane_ok) {
    if constexpr (H) {  // l = A(k+1)
      vld_at(p.A[0], q + p.plane, p.total, 3001, L.l0);
      vld_at(p.A[1], q + p.plane, p.total, 3001, L.l1);
    } else {  // l = A(k)
      vld_at(p.A[0], q, p.total, 3001, L.l0);
      vld_at(p.A[1], q, p.total, 3001, L.l1);
    }
    vld_at(p.A[2], q, p.total, 3002, L.a2);
    vld_at(p.A[0], q + s * p.pitch, p.total, 3003, L.y0);
    vld_at(p.A[2], q + s * p.pitch, p.total, 3003, L.y2);
    if constexpr (H) {
      if (lane == 31 && KH_IN(q + VN, p.total, 3004)) {
        L.xn1 = p.A[1][q + VN];
        L.xn2 = p.A[2][q + VN];
      }
    } else {
      if (lane == 0 && KH_IN(q - 1, p.total, 3004)) {
        L.xn1 = p.A[1][q - 1];
        L.xn2 = p.A[2][q - 1];
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) vld_at(p.O[c], q, p.total, 3005, L.O[c]);
    if (pervox) {
#pragma unroll
      for (int c = 0; c < 3; ++c) vld_at(p.m_inv[c], q, p.total, 3006, L.m[c]);
    }
#pragma unroll
    for (int v = 0; v < VN; ++v)
      L.cls[v] = (L.tf && lane_ok && KH_IN(q + v, p.total, 3007)) ? p.cell_class[q + v] : 0u;
    const bool aux = anyRegion || L.tf;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (aux && p.Ts[c]) vld_at(p.Ts[c], q, p.total, 3008, L.t[c]); else vzero(L.t[c]);
      if (anyRegion && p.U[c] && axis_any[(c + 1) % 3]) vld_at(p.U[c], q, p.total, 3009, L.u[c]);
      else vzero(L.u[c]);
      if (anyRegion && p.W[c] && axis_any[c]) vld_at(p.W[c], q, p.total, 3010, L.w[c]); else vzero(L.w[c]);
    }
    if (FULL && !H && L.tf && p.chi3) vld_at(p.chi3, q, p.total, 3011, L.c3); else vzero(L.c3);
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      vzero(L.O[c]); vzero(L.t[c]); vzero(L.u[c]); vzero(L.w[c]);
    }
    vzero(L.c3);
#pragma unroll
    for (int v = 0; v < VN; ++v) L.cls[v] = 0u;
  }
  if (!pervox) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int v = 0; v < VN; ++v) L.m[c][v] = p.m_scalar;
  }
}

// Update of plane k from its loads L; r0/r1 carry the rotated z-neighbour
// plane of A0/A1 in and out.
template <typename T, int VN, bool H, bool CPML, bool FULL>
__device__ __forceinline__ void compute_plane(const HalfStepParams<T>& p, PlaneLoads<T, VN>& L, int k,
                                              long long row, int lane, bool lane_ok, int x0, int j,
                                              bool fy, bool anyfx, const bool (&fxv)[VN],
                                              const AxisCoef<T> (&axv)[VN], const AxisCoef<T>& ay,
                                              T (&r0)[VN], T (&r1)[VN]) {
  const long long q = row + (long long)k * p.plane;
  // cur = A0/A1 at plane k, nb = at plane k+s
  const T(&cur0)[VN] = H ? r0 : L.l0;
  const T(&cur1)[VN] = H ? r1 : L.l1;
  const T(&nb0)[VN] = H ? L.l0 : r0;
  const T(&nb1)[VN] = H ? L.l1 : r1;

  // x neighbours of A1 and A2 at plane k
  T x1s[VN], x2s[VN];
  if constexpr (H) {
    T n1 = __shfl_down_sync(0xffffffffu, cur1[0], 1);
    T n2 = __shfl_down_sync(0xffffffffu, L.a2[0], 1);
    if (lane == 31) {
      n1 = L.xn1;
      n2 = L.xn2;
    }
#pragma unroll
    for (int v = 0; v < VN - 1; ++v) { x1s[v] = cur1[v + 1]; x2s[v] = L.a2[v + 1]; }
    x1s[VN - 1] = n1;
    x2s[VN - 1] = n2;
  } else {
    T n1 = __shfl_up_sync(0xffffffffu, cur1[VN - 1], 1);
    T n2 = __shfl_up_sync(0xffffffffu, L.a2[VN - 1], 1);
    if (lane == 0) {
      n1 = L.xn1;
      n2 = L.xn2;
    }
#pragma unroll
    for (int v = 1; v < VN; ++v) { x1s[v] = cur1[v - 1]; x2s[v] = L.a2[v - 1]; }
    x1s[0] = n1;
    x2s[0] = n2;
  }

  if (lane_ok) {
    T K[3][VN];
#pragma unroll
    for (int v = 0; v < VN; ++v) {
      K[0][v] = p.dt * (p.inv_d[2] * (nb1[v] - cur1[v]) - p.inv_d[1] * (L.y2[v] - L.a2[v]));
      K[1][v] = p.dt * (p.inv_d[0] * (x2s[v] - L.a2[v]) - p.inv_d[2] * (nb0[v] - cur0[v]));
      K[2][v] = p.dt * (p.inv_d[1] * (L.y0[v] - cur0[v]) - p.inv_d[0] * (x1s[v] - cur1[v]));
    }
    const bool fz = k < p.pml_lo[2] || k >= p.nz - p.pml_hi[2];
    const bool anyRegion = fy || fz || anyfx;
    bool anySpecial = false;
#pragma unroll
    for (int v = 0; v < VN; ++v) anySpecial |= (L.cls[v] & (H ? kSpecialH : kSpecialE)) != 0;
    if (!anyRegion && !anySpecial) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int v = 0; v < VN; ++v) L.O[c][v] = L.O[c][v] + L.m[c][v] * K[c][v];
    } else {
      const AxisCoef<T> az = KH_IN(k, p.nz, 3012) ? p.ax[2][k] : AxisCoef<T>{T(0), T(1), T(1), T(1)};
#pragma unroll
      for (int v = 0; v < VN; ++v) {
        const int i = x0 + v;
        if (i >= p.nx) continue;
        const bool special = (L.cls[v] & (H ? kSpecialH : kSpecialE)) != 0;
        if (!(fxv[v] || fy || fz || special)) {
#pragma unroll
          for (int c = 0; c < 3; ++c) L.O[c][v] = L.O[c][v] + L.m[c][v] * K[c][v];
          continue;
        }
        const bool fc[3] = {fxv[v], fy, fz};
        const AxisCoef<T> ac[3] = {axv[v], ay, az};
        const T Kc[3] = {K[0][v], K[1][v], K[2][v]};
        const T mc[3] = {L.m[0][v], L.m[1][v], L.m[2][v]};
        T Oc[3] = {L.O[0][v], L.O[1][v], L.O[2][v]};
        T tc[3] = {L.t[0][v], L.t[1][v], L.t[2][v]};
        T uc[3] = {L.u[0][v], L.u[1][v], L.u[2][v]};
        T wc[3] = {L.w[0][v], L.w[1][v], L.w[2][v]};
        if constexpr (FULL) {
          general_cell<T, H>(p, q + v, i, j, k, fc, ac, L.cls[v], special, Kc, mc, Oc, tc, uc, wc, L.c3[v]);
        } else {
          if (fc[0] || fc[1] || fc[2]) {
            pml_cell<T, CPML>(fc, ac, Kc, mc, Oc, tc, uc, wc);
          } else {  // source cell outside CPML: keeps its B|D state
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              tc[c] = tc[c] + Kc[c];
              Oc[c] = mc[c] * tc[c];
            }
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          L.O[c][v] = Oc[c];
          L.t[c][v] = tc[c];
          L.u[c][v] = uc[c];
          L.w[c][v] = wc[c];
        }
      }
      const bool axis_any[3] = {anyfx, fy, fz};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (p.Ts[c]) vst_at(p.Ts[c], q, p.total, 3013, L.t[c]);
        if (p.U[c] && axis_any[(c + 1) % 3]) vst_at(p.U[c], q, p.total, 3014, L.u[c]);
        if (p.W[c] && axis_any[c]) vst_at(p.W[c], q, p.total, 3015, L.w[c]);
      }
    }
    if (x0 + VN <= p.nx) {
#pragma unroll
      for (int c = 0; c < 3; ++c) vst_at(p.O[c], q, p.total, 3016, L.O[c]);
    } else {
#pragma unroll
      for (int v = 0; v < VN; ++v) {
        if (x0 + v < p.nx && KH_IN(q + v, p.total, 3017)) {
#pragma unroll
          for (int c = 0; c < 3; ++c) p.O[c][q + v] = L.O[c][v];
        }
      }
    }
  }
  // rotate: H half keeps A(k+1) as the next plane's A(k); E half keeps
  // A(k) as the next plane's A(k-1)
#pragma unroll
  for (int v = 0; v < VN; ++v) { r0[v] = L.l0[v]; r1[v] = L.l1[v]; }
}

// One fused half-step.  H = true: B/H from curl E; H = false: D/E from curl H.
// FULL = false (LEAN) compiles only plain and CPML cells; cells marked special
// there are source cells, updated as B|D-keeping cells (O = m⁻¹·T) and given
// their source term by source_fix_kernel when sources are active.
//
// The z march is double-buffered with a prefetch distance of two planes: the
// loads of plane k+2 are issued as soon as plane k has been consumed, so each
// warp keeps about two planes of memory traffic in flight.
template <typename T, int VN, bool H, bool CPML, bool FULL>
__global__ void __launch_bounds__(32 * kBlockY, sizeof(T) == 4 ? kMinBlocks : 2)
    half_step_kernel(const HalfStepParams<T> p) {
  const int lane = threadIdx.x;
  const int j = blockIdx.y * kBlockY + threadIdx.y;
  if (j >= p.ny) return;  // warp-uniform: blockDim.x == 32
  const int xb = blockIdx.x;
  const int x0 = (xb * 32 + lane) * VN;
  const bool lane_ok = x0 < p.nx;
  const int k0 = blockIdx.z * kPlanesPerCta;
  const int k1 = min(k0 + kPlanesPerCta, p.nz);
  const long long row = p.origin + (long long)j * p.pitch + x0;
  const bool fy = j < p.pml_lo[1] || j >= p.ny - p.pml_hi[1];
  const bool pervox = p.m_inv[0] != nullptr;
  // special-tile bits of planes [64·(k0/64), +64) of this warp's row segment
  const long long tbi = ((long long)(k0 >> 6) * p.ny + j) * p.nxb + xb;
  const uint64_t tbits = (p.tile_bits && KH_IN(tbi, p.n_tile_words, 3018)) ? p.tile_bits[tbi] : 0ull;

  // per-cell x flags and CPML coefficients of this thread's vector and the
  // row's y coefficients: static along the z march
  bool fxv[VN];
  AxisCoef<T> axv[VN];
  bool anyfx = false;
#pragma unroll
  for (int v = 0; v < VN; ++v) {
    const int i = x0 + v;
    fxv[v] = i < p.nx && (i < p.pml_lo[0] || i >= p.nx - p.pml_hi[0]);
    anyfx |= fxv[v];
    axv[v] = (i < p.nx && KH_IN(i, p.nx, 3019)) ? p.ax[0][i] : AxisCoef<T>{T(0), T(1), T(1), T(1)};
  }
  const AxisCoef<T> ay = KH_IN(j, p.ny, 3020) ? p.ax[1][j] : AxisCoef<T>{T(0), T(1), T(1), T(1)};

  // rotated z-neighbour plane of A0, A1: A(k0) for the H half, A(k0-1) for E
  T r0[VN], r1[VN];
  vzero(r0);
  vzero(r1);
  if (lane_ok) {
    const long long q0 = row + (long long)k0 * p.plane + (H ? 0 : -p.plane);
    vld_at(p.A[0], q0, p.total, 3021, r0);
    vld_at(p.A[1], q0, p.total, 3021, r1);
  }
  PlaneLoads<T, VN> A, B;
  load_plane<T, VN, H, FULL>(p, A, k0, row, lane, lane_ok, pervox, fy, anyfx, tbits);
  if (k0 + 1 < k1) load_plane<T, VN, H, FULL>(p, B, k0 + 1, row, lane, lane_ok, pervox, fy, anyfx, tbits);
  for (int k = k0; k < k1; k += 2) {
    compute_plane<T, VN, H, CPML, FULL>(p, A, k, row, lane, lane_ok, x0, j, fy, anyfx, fxv, axv, ay, r0, r1);
    if (k + 2 < k1) load_plane<T, VN, H, FULL>(p, A, k + 2, row, lane, lane_ok, pervox, fy, anyfx, tbits);
    if (k + 1 < k1) {
      compute_plane<T, VN, H, CPML, FULL>(p, B, k + 1, row, lane, lane_ok, x0, j, fy, anyfx, fxv, axv, ay, r0, r1);
      if (k + 3 < k1) load_plane<T, VN, H, FULL>(p, B, k + 3, row, lane, lane_ok, pervox, fy, anyfx, tbits);
    }
  }
}

template <typename T, bool CPML, bool FULL>
static void launch_variant(bool h_half, const HalfStepParams<T>& p, cudaStream_t st) {
  dim3 block(32, kBlockY, 1);
  dim3 grid(p.nxb, (p.ny + kBlockY - 1) / kBlockY, (p.nz + kPlanesPerCta - 1) / kPlanesPerCta);
  if (h_half) half_step_kernel<T, kVN, true, CPML, FULL><<<grid, block, 0, st>>>(p);
  else half_step_kernel<T, kVN, false, CPML, FULL><<<grid, block, 0, st>>>(p);
}

template <typename T>
void launch_half_step(bool h_half, const HalfStepParams<T>& p, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (p.cpml) {
    if (p.full) launch_variant<T, true, true>(h_half, p, st);
    else launch_variant<T, true, false>(h_half, p, st);
  } else {
    if (p.full) launch_variant<T, false, true>(h_half, p, st);
    else launch_variant<T, false, false>(h_half, p, st);
  }
}

// Source term of the cells a LEAN half-step updated as B|D-keeping cells:
// O = m⁻¹·(T + S), the same arithmetic update_field_generic performs
// (net = T; net += S; A = m⁻¹·net, Helpers.jl:329-347).
// Component c of source cell q: O = m⁻¹·(T + S), or through the W stage
// when the cell lies in the CPML of c's own axis (SourceFixParams).
template <typename T>
__device__ __forceinline__ void source_fix_one(const SourceFixParams<T>& p, long long q, int c, T S) {
  const T m = p.m_inv[c] ? p.m_inv[c][q] : p.m_scalar;
  T net = p.Ts[c][q];
  net += S;
  if (p.W[c]) {
    const long long rel = q - p.origin;
    const long long k = rel / p.plane, rem = rel % p.plane;
    const int idx = c == 0 ? int(rem % p.pitch) : (c == 1 ? int(rem / p.pitch) : int(k));
    if ((idx < p.pml_lo[c] || idx >= p.n[c] - p.pml_hi[c]) && KH_IN(idx, p.n[c], 3031)) {
      const AxisCoef<T> ao = p.ax[c][idx];
      if (ao.s != T(0)) {
        const T wl = p.W[c][q];
        const T wn = m * net;
        p.W[c][q] = wn;
        p.O[c][q] = p.O[c][q] + ao.op * (wn - wl);
        return;
      }
    }
  }
  p.O[c][q] = m * net;
}

template <typename T>
__global__ void source_fix_kernel(const SourceFixParams<T> p) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= p.nslots) return;
  const long long q = p.slot_cell[slot];
  const SlotPack<T> pk = p.slot_pack[slot];
  if (!KH_IN(q, p.total, 3022)) return;
  const int base = p.h_half ? 3 : 0;
  if (pk.src >= 0) {  // a single entry: one component, S = real(f(t)·amplitude)
    const int c = pk.comp - base;
    if (c < 0 || c > 2 || !KH_IN(pk.src, p.n_src, 3024)) return;
    const Cplx<T> f = p.f_now[pk.src];
    T S = T(0);
    S += f.re * pk.amp.re - f.im * pk.amp.im;
    source_fix_one(p, q, c, S);
    return;
  }
  T S[3] = {T(0), T(0), T(0)};
  bool has[3] = {false, false, false};
  for (int e = p.slot_off[slot]; e < p.slot_off[slot + 1]; ++e) {
    if (!KH_IN(e, p.n_ent, 3023)) break;
    const int c = p.ent_comp[e] - base;
    if (c < 0 || c > 2) continue;
    const Cplx<T> a = p.ent_amp[e];
    if (!KH_IN(p.ent_src[e], p.n_src, 3024)) continue;
    const Cplx<T> f = p.f_now[p.ent_src[e]];
    const T v = f.re * a.re - f.im * a.im;
    if (c == 0) { S[0] += v; has[0] = true; }
    else if (c == 1) { S[1] += v; has[1] = true; }
    else { S[2] += v; has[2] = true; }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
    if (has[c]) source_fix_one(p, q, c, S[c]);
}

template <typename T>
void launch_source_fix(const SourceFixParams<T>& p, void* stream) {
  if (p.nslots <= 0) return;
  const int threads = 128;
  source_fix_kernel<T><<<(p.nslots + threads - 1) / threads, threads, 0, static_cast<cudaStream_t>(stream)>>>(p);
}

// ---------------------------------------------------------------------------
// Dispersive and Kerr cells after a LEAN E half-step (DispFixParams).  One
// warp per entry of the row-segment list (32·kVN cells).  A segment without
// pole cells needs no class words: its lanes load the pair of E vectors and
// χ3 values of their two cells at once and correct the cells with χ3 ≠ 0
// (the cells the LEAN launch left uncorrected).  Pole segments go cell by
// cell through the class words.
template <typename T>
__global__ void disp_fix_kernel(const DispFixParams<T> p) {
  static_assert(kVN == 2, "paired loads of the χ3 path");
  const long long w = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (w >= p.n_list) return;  // warp-uniform
  const uint32_t ent = p.list[w];
  const long long seg = ent & 0x7fffffffu;
  const int xb = int(seg % p.nxb);
  const long long r = seg / p.nxb;
  const int j = int(r % p.ny);
  const int k = int(r / p.ny);
  const int lane = threadIdx.x & 31;
  const int i0 = xb * 32 * kVN + lane * kVN;
  const long long q0 = p.origin + (long long)k * p.plane + (long long)j * p.pitch + i0;
  if (!(ent >> 31)) {
    if (!p.chi3 || i0 >= p.nx) return;
    if (i0 + 1 < p.nx && KH_IN(q0 + 1, p.total, 3045)) {
      using V2 = typename VT<T, 2>::V;  // q0 is even: 8/16-byte aligned
      // the E pair is loaded with the χ3 pair (one round trip, not two):
      // in a Kerr segment nearly every cell has χ3
      const V2 c3 = *reinterpret_cast<const V2*>(p.chi3 + q0);
      V2 e[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) e[c] = *reinterpret_cast<const V2*>(p.E[c] + q0);
      if (c3.x == T(0) && c3.y == T(0)) return;
      // χ3 Kerr correction (Dispersive.jl:127-147), same operation order as below
      if (c3.x != T(0)) {
        const T esq = (e[0].x * e[0].x + e[1].x * e[1].x) + e[2].x * e[2].x;
        const T corr = T(1) / (T(1) + c3.x * esq);
#pragma unroll
        for (int c = 0; c < 3; ++c) e[c].x = e[c].x * corr;
      }
      if (c3.y != T(0)) {
        const T esq = (e[0].y * e[0].y + e[1].y * e[1].y) + e[2].y * e[2].y;
        const T corr = T(1) / (T(1) + c3.y * esq);
#pragma unroll
        for (int c = 0; c < 3; ++c) e[c].y = e[c].y * corr;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) *reinterpret_cast<V2*>(p.E[c] + q0) = e[c];
      return;
    }
  }
#pragma unroll 1
  for (int v = 0; v < kVN; ++v) {
    const int i = i0 + v;
    if (i >= p.nx) continue;
    const long long q = q0 + v;
    if (!KH_IN(q, p.total, 3040)) continue;
    const uint32_t cls = p.cell_class[q];
    if (!(cls & (kHasChi3 | kHasPole))) continue;
    T O[3];
    if (cls & kHasPole) {
      // E = ε⁻¹·(D + S − Σ P) (update_field_generic: net = T; net += S; net -= P)
      T S[3] = {T(0), T(0), T(0)};
      bool hasS[3] = {false, false, false};
      if (p.sources_active && (cls & kHasSrcE)) {
        const int slot = int(cls >> kSlotShift);
        if (KH_IN(slot + 1, p.n_slots + 1, 3041)) {
          for (int e = p.slot_off[slot]; e < p.slot_off[slot + 1]; ++e) {
            if (!KH_IN(e, p.n_ent, 3042) || !KH_IN(p.ent_src[e], p.n_src, 3043)) continue;
            const int c = p.ent_comp[e];
            const Cplx<T> am = p.ent_amp[e];
            const Cplx<T> fv = p.f_now[p.ent_src[e]];
            const T v = fv.re * am.re - fv.im * am.im;  // real(f(t) · amplitude)
            if (c >= 0 && c < 3) {
              S[c] += v;
              hasS[c] = true;
            }
          }
        }
      }
      T Ptot[3] = {T(0), T(0), T(0)};
      for (int pp = 0; pp < p.npoles; ++pp) {
        Ptot[0] += p.poles[pp].P[0][q];
        Ptot[1] += p.poles[pp].P[1][q];
        Ptot[2] += p.poles[pp].P[2][q];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        T net = p.D[c][q];
        if (hasS[c]) net += S[c];
        net -= Ptot[c];
        const T m = p.m_inv[c] ? p.m_inv[c][q] : p.m_scalar;
        O[c] = m * net;
        // in the CPML of its own axis the cell's E comes out of the W stage
        // (update_field_generic, Helpers.jl:333-339): E = E' + op·(W_new − W')
        // on top of the W' and E' that the LEAN launch (or the source kernel)
        // left, W_new = ε⁻¹·net
        if (p.W[c]) {
          const int idx = c == 0 ? i : (c == 1 ? j : k);
          const int nn = c == 0 ? p.nx : (c == 1 ? p.ny : p.nz);
          if ((idx < p.pml_lo[c] || idx >= nn - p.pml_hi[c]) && KH_IN(idx, nn, 3046)) {
            const AxisCoef<T> ao = p.ax[c][idx];
            if (ao.s != T(0)) {
              const T wl = p.W[c][q];
              const T wn = m * net;
              p.W[c][q] = wn;
              O[c] = p.E[c][q] + ao.op * (wn - wl);
            }
          }
        }
      }
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) O[c] = p.E[c][q];
    }
    // χ3 Kerr correction (Dispersive.jl:127-147)
    if (cls & kHasChi3) {
      const T c3 = p.chi3[q];
      if (c3 != T(0)) {
        const T esq = (O[0] * O[0] + O[1] * O[1]) + O[2] * O[2];
        const T corr = T(1) / (T(1) + c3 * esq);
        O[0] = O[0] * corr;
        O[1] = O[1] * corr;
        O[2] = O[2] * corr;
      }
    }
    // ADE poles with E^{n+1} (Dispersive.jl:25-88)
    if (cls & kHasPole) {
      for (int pp = 0; pp < p.npoles; ++pp) {
        const PoleParams<T>& P = p.poles[pp];
        const T s = P.sigma[q];
        if (s == T(0)) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T px = P.P[c][q];
          const T pprev = P.Pprev[c][q];
          T pn;
          if (P.is_drude) pn = P.gamma1_inv * ((T(2) * px - P.gamma1 * pprev) + (P.drive * s) * O[c]);
          else pn = P.gamma1_inv * ((P.coeff_p * px - P.gamma1 * pprev) + (P.drive * s) * O[c]);
          P.P[c][q] = pn;
          P.Pprev[c][q] = px;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) p.E[c][q] = O[c];
  }
}

template <typename T>
void launch_disp_fix(const DispFixParams<T>& p, void* stream) {
  if (p.n_list <= 0) return;
  const int warps = 8;
  disp_fix_kernel<T><<<unsigned((p.n_list + warps - 1) / warps), 32 * warps, 0,
                       static_cast<cudaStream_t>(stream)>>>(p);
}

// ---------------------------------------------------------------------------
// Periodic wrap.  One block row per periodic axis and component:
// blockIdx.y = 3·(index of the axis in p.axes) + component; threads stride
// over the face's (n_t1 × n_t2) cells, t1 the lower of the face's two axes;
// each copies both directions of one cell.
template <typename T>
__global__ void wrap_kernel(const WrapParams<T> p) {
  const int a = p.axes[blockIdx.y / 3], c = blockIdx.y % 3;
  // the face's lower axis runs fastest across threads: x on the y and z
  // faces (coalesced rows), y on the x face (one element per row there)
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const long long st[3] = {1, p.pitch, p.plane};
  const long long face = (long long)p.n[t1] * p.n[t2];
  T* f = p.O[c];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < face;
       e += (long long)gridDim.x * blockDim.x) {
    const long long u = e % p.n[t1], v = e / p.n[t1];
    const long long base = p.origin + u * st[t1] + v * st[t2];
    const long long lo = base, hi = base + (long long)(p.n[a] - 1) * st[a];
    const long long ghost_lo = base - st[a], ghost_hi = base + (long long)p.n[a] * st[a];
    if (!(KH_IN(ghost_lo, p.total, 3028) && KH_IN(ghost_hi, p.total, 3029))) continue;
    if (!(p.chi3 && p.chi3[hi] != T(0))) f[ghost_lo] = f[hi];
    if (!(p.chi3 && p.chi3[lo] != T(0))) f[ghost_hi] = f[lo];
  }
}

template <typename T>
void launch_wrap(const WrapParams<T>& p0, void* stream) {
  if (!(p0.periodic & 7u)) return;
  WrapParams<T> p = p0;
  int na = 0;
  long long face = 0;
  for (int a = 0; a < 3; ++a)
    if ((p.periodic >> a) & 1u) {
      p.axes[na++] = a;
      face = std::max(face, (long long)p.n[(a + 1) % 3] * p.n[(a + 2) % 3]);
    }
  const int threads = 256;
  const long long blocks = std::min<long long>((face + threads - 1) / threads, 1024);
  wrap_kernel<T><<<dim3(unsigned(std::max<long long>(blocks, 1)), unsigned(3 * na)), threads, 0,
                   static_cast<cudaStream_t>(stream)>>>(p);
}

// ---------------------------------------------------------------------------
// DFT accumulation (update_dft_monitor!, Monitors.jl:361-379):
//   F[cell, f] += Δt·exp(i2πf t)·field[cell]
// FP32 accumulators carry a Kahan compensation term.  One update, shared by
// the per-monitor and the batched kernels so both give the same bits.
template <typename T>
__device__ __forceinline__ void dft_update(Cplx<T>* F, Cplx<T>* comp, long long t, Cplx<T> ph, T v) {
  Cplx<T> acc = F[t];
  if (comp) {
    Cplx<T> c = comp[t];
    const T yr = ph.re * v - c.re;
    const T yi = ph.im * v - c.im;
    const T tr = acc.re + yr;
    const T ti = acc.im + yi;
    c.re = (tr - acc.re) - yr;
    c.im = (ti - acc.im) - yi;
    acc.re = tr;
    acc.im = ti;
    comp[t] = c;
  } else {
    acc.re = acc.re + ph.re * v;
    acc.im = acc.im + ph.im * v;
  }
  F[t] = acc;
}

template <typename T>
__global__ void dft_kernel(const DftParams<T> p) {
  const long long ncell = (long long)p.dims[0] * p.dims[1] * p.dims[2];
  const long long total = ncell * p.nf;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int f = int(t / ncell);
    const long long cell = t - (long long)f * ncell;
    const int i = int(cell % p.dims[0]);
    const long long r = cell / p.dims[0];
    const int jj = int(r % p.dims[1]);
    const int kk = int(r / p.dims[1]);
    const long long q = p.origin + (long long)(p.start[2] + kk) * p.plane +
                        (long long)(p.start[1] + jj) * p.pitch + (p.start[0] + i);
    if (!KH_IN(q, p.total, 3025)) continue;
    dft_update(p.F, p.comp, t, p.phase[f], p.field[q]);
  }
}

// All monitors of one half-step in one grid: item u < first[n] belongs to the
// monitor m with first[m] <= u < first[m+1].
template <typename T>
__global__ void dft_batch_kernel(const DftBatchParams<T> p) {
  const long long total = p.first[p.n];
  for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
       u += (long long)gridDim.x * blockDim.x) {
    int m = 0;
    while (m + 1 < p.n && u >= p.first[m + 1]) ++m;
    const auto& M = p.mon[m];
    const long long t = u - p.first[m];
    const long long ncell = (long long)M.dims[0] * M.dims[1] * M.dims[2];
    const int f = int(t / ncell);
    const long long cell = t - (long long)f * ncell;
    const int i = int(cell % M.dims[0]);
    const long long r = cell / M.dims[0];
    const int jj = int(r % M.dims[1]);
    const int kk = int(r / M.dims[1]);
    const long long q = p.origin + (long long)(M.start[2] + kk) * p.plane +
                        (long long)(M.start[1] + jj) * p.pitch + (M.start[0] + i);
    if (!KH_IN(q, p.total, 3030)) continue;
    dft_update(M.F, M.comp, t, M.phase[f], M.field[q]);
  }
}

template <typename T>
void launch_dft_batch(const DftBatchParams<T>& p, void* stream) {
  if (p.n <= 0) return;
  const long long total = p.first[p.n];
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  dft_batch_kernel<T><<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(p);
}

template <typename T>
void launch_dft(const DftParams<T>& p, void* stream) {
  const long long total = (long long)p.dims[0] * p.dims[1] * p.dims[2] * p.nf;
  int blocks = int((total + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  dft_kernel<T><<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(p);
}

// ---------------------------------------------------------------------------
// History recording: one thread per x-row segment element, rows of the box
// laid out x fastest in the destination slot.
template <typename T>
__global__ void record_kernel(const RecordParams<T> p) {
  const int rows = p.dims[1] * p.dims[2];
  for (int r = blockIdx.y; r < rows; r += gridDim.y) {
    const int jj = r % p.dims[1], kk = r / p.dims[1];
    const T* src = p.field + p.origin + (long long)(p.start[2] + kk) * p.plane +
                   (long long)(p.start[1] + jj) * p.pitch + p.start[0];
    T* dst = p.dst + (long long)r * p.dims[0];
    const long long s0 = src - p.field;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.dims[0]; i += gridDim.x * blockDim.x)
      if (KH_IN(s0 + i, p.total, 3026) && KH_IN((long long)r * p.dims[0] + i, (long long)rows * p.dims[0], 3027))
        dst[i] = src[i];
  }
}

template <typename T>
void launch_record(const RecordParams<T>& p, void* stream) {
  const int rows = p.dims[1] * p.dims[2];
  const int tx = p.dims[0] >= 128 ? 128 : 64;
  dim3 grid((p.dims[0] + tx - 1) / tx, rows < 65535 ? rows : 65535);
  record_kernel<T><<<grid, tx, 0, static_cast<cudaStream_t>(stream)>>>(p);
}

// ---------------------------------------------------------------------------
// Flux (get_flux, FluxMonitor.jl:92-156) in FP64: one block per frequency,
// fixed-order tree reduction so the result is reproducible.
template <typename T>
__device__ __forceinline__ void load_c(const Cplx<T>* F, const Cplx<T>* C, long long q, double& re,
                                       double& im) {
  re = double(F[q].re);
  im = double(F[q].im);
  if (C) {  // Kahan: sum - compensation
    re -= double(C[q].re);
    im -= double(C[q].im);
  }
}

struct FluxArgs {
  int d[4][3];
  int normal;
  int nf;
  double dA;
};

template <typename T>
__device__ __forceinline__ void avg_at(const Cplx<T>* F, const Cplx<T>* C, const int* d, int normal,
                                       int a1, int a2, int i1, int i2, int f, double& re,
                                       double& im) {
  int idx[3];
  idx[normal] = 0;
  idx[a1] = i1;
  idx[a2] = i2;
  const long long ncell = (long long)d[0] * d[1] * d[2];
  long long q = (long long)f * ncell + ((long long)idx[2] * d[1] + idx[1]) * d[0] + idx[0];
  load_c(F, C, q, re, im);
  if (d[normal] >= 2) {  // _avg_dim: (layer 1 + layer 2) / 2
    idx[normal] = 1;
    long long q2 = (long long)f * ncell + ((long long)idx[2] * d[1] + idx[1]) * d[0] + idx[0];
    double r2, i2v;
    load_c(F, C, q2, r2, i2v);
    re = (re + r2) / 2;
    im = (im + i2v) / 2;
  }
}

constexpr int kFluxCellsPerBlock = 1024;

template <typename T>
__global__ void flux_partial_kernel(const Cplx<T>* e1, const Cplx<T>* e2, const Cplx<T>* h1,
                                    const Cplx<T>* h2, const Cplx<T>* ce1, const Cplx<T>* ce2,
                                    const Cplx<T>* ch1, const Cplx<T>* ch2, const FluxArgs a,
                                    double* partial) {
  const int f = blockIdx.y;
  const int n = a.normal;
  const int a1 = n == 0 ? 1 : 0;
  const int a2 = n == 2 ? 1 : 2;
  int n1 = a.d[0][a1], n2 = a.d[0][a2];
  for (int m = 1; m < 4; ++m) {
    n1 = min(n1, a.d[m][a1]);
    n2 = min(n2, a.d[m][a2]);
  }
  const long long cells = (long long)n1 * n2;
  // block b takes cells [b·span, (b+1)·span), span a multiple of blockDim
  const long long span = ((cells + gridDim.x - 1) / gridDim.x + blockDim.x - 1) / blockDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * span;
  const long long t1 = t0 + span < cells ? t0 + span : cells;
  double acc = 0.0;
  for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const int i1 = int(t % n1), i2 = int(t / n1);
    double E1r, E1i, E2r, E2i, H1r, H1i, H2r, H2i;
    avg_at(e1, ce1, a.d[0], n, a1, a2, i1, i2, f, E1r, E1i);
    avg_at(e2, ce2, a.d[1], n, a1, a2, i1, i2, f, E2r, E2i);
    avg_at(h1, ch1, a.d[2], n, a1, a2, i1, i2, f, H1r, H1i);
    avg_at(h2, ch2, a.d[3], n, a1, a2, i1, i2, f, H2r, H2i);
    // Re(E1·conj(H2) − E2·conj(H1))
    acc += ((E1r * H2r + E1i * H2i) - (E2r * H1r + E2i * H1i)) * a.dA;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(long long)f * gridDim.x + blockIdx.x] = red[0];
}

// One warp per frequency: lane l adds partials l, l+32, … in order, then a
// fixed shuffle tree.
__global__ void flux_final_kernel(const double* partial, int nb, double* out) {
  const int f = blockIdx.x;
  const int lane = threadIdx.x;
  double s = 0.0;
  for (int b = lane; b < nb; b += 32) s += partial[(long long)f * nb + b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[f] = s;
}

int flux_blocks(long long cells, int nf, int partial_cap) {
  long long b = (cells + kFluxCellsPerBlock - 1) / kFluxCellsPerBlock;
  const long long fill = (4LL * 152 + nf - 1) / (nf > 0 ? nf : 1);  // about four blocks per SM in all
  if (b > fill) b = fill;
  if (nf > 0 && b > partial_cap / nf) b = partial_cap / nf;
  return int(b < 1 ? 1 : b);
}

template <typename T>
void launch_flux(const Cplx<T>* e1, const Cplx<T>* e2, const Cplx<T>* h1, const Cplx<T>* h2,
                 const Cplx<T>* c_e1, const Cplx<T>* c_e2, const Cplx<T>* c_h1,
                 const Cplx<T>* c_h2, const int dims_e1[3], const int dims_e2[3],
                 const int dims_h1[3], const int dims_h2[3], int normal_axis, int nf, double dA,
                 double* out, double* partial, int partial_cap, void* stream) {
  FluxArgs a;
  for (int q = 0; q < 3; ++q) {
    a.d[0][q] = dims_e1[q];
    a.d[1][q] = dims_e2[q];
    a.d[2][q] = dims_h1[q];
    a.d[3][q] = dims_h2[q];
  }
  a.normal = normal_axis;
  a.nf = nf;
  a.dA = dA;
  if (nf <= 0) return;
  const int na1 = normal_axis == 0 ? 1 : 0, na2 = normal_axis == 2 ? 1 : 2;
  long long n1 = dims_e1[na1], n2 = dims_e1[na2];
  for (const int* d : {dims_e2, dims_h1, dims_h2}) {
    n1 = std::min<long long>(n1, d[na1]);
    n2 = std::min<long long>(n2, d[na2]);
  }
  const int nb = flux_blocks(n1 * n2, nf, partial_cap);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  flux_partial_kernel<T><<<dim3(unsigned(nb), unsigned(nf)), 256, 0, st>>>(e1, e2, h1, h2, c_e1, c_e2, c_h1,
                                                                          c_h2, a, partial);
  flux_final_kernel<<<unsigned(nf), 32, 0, st>>>(partial, nb, out);
}

template void launch_half_step<float>(bool, const HalfStepParams<float>&, void*);
template void launch_half_step<double>(bool, const HalfStepParams<double>&, void*);
template void launch_wrap<float>(const WrapParams<float>&, void*);
template void launch_wrap<double>(const WrapParams<double>&, void*);
template void launch_source_fix<float>(const SourceFixParams<float>&, void*);
template void launch_source_fix<double>(const SourceFixParams<double>&, void*);
template void launch_record<float>(const RecordParams<float>&, void*);
template void launch_record<double>(const RecordParams<double>&, void*);
template void launch_dft<float>(const DftParams<float>&, void*);
template void launch_dft_batch<float>(const DftBatchParams<float>&, void*);
template void launch_disp_fix<float>(const DispFixParams<float>&, void*);
template void launch_disp_fix<double>(const DispFixParams<double>&, void*);
template void launch_dft_batch<double>(const DftBatchParams<double>&, void*);
template void launch_dft<double>(const DftParams<double>&, void*);
template void launch_flux<float>(const Cplx<float>*, const Cplx<float>*, const Cplx<float>*,
                                 const Cplx<float>*, const Cplx<float>*, const Cplx<float>*,
                                 const Cplx<float>*, const Cplx<float>*, const int*, const int*,
                                 const int*, const int*, int, int, double, double*, double*, int, void*);
template void launch_flux<double>(const Cplx<double>*, const Cplx<double>*, const Cplx<double>*,
                                  const Cplx<double>*, const Cplx<double>*, const Cplx<double>*,
                                  const Cplx<double>*, const Cplx<double>*, const int*, const int*,
                                  const int*, const int*, int, int, double, double*, double*, int, void*);

}  // namespace kh
