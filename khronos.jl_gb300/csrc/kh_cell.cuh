// Per-cell device code shared by the half-step kernels (kh_kernels.cu, the
// register-pipelined kernel; kh_tma.cu, the TMA-staged kernel): vector
// helpers, the general cell update (sources, χ3, poles, conductivity, either
// CPML semantics) and the lean CPML cell update.
#pragma once

#include <cuda_runtime.h>

#include "kh_kernels.cuh"

namespace kh {

template <typename T, int VN>
struct VT;
template <>
struct VT<float, 2> {
  using V = float2;
};
template <>
struct VT<double, 2> {
  using V = double2;
};

template <typename T, int VN>
__device__ __forceinline__ void vld(const T* ptr, T (&v)[VN]) {
  using V = typename VT<T, VN>::V;
  V x = *reinterpret_cast<const V*>(ptr);
  if constexpr (VN == 4) {
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
  } else {
    v[0] = x.x; v[1] = x.y;
  }
}

template <typename T, int VN>
__device__ __forceinline__ void vst(T* ptr, const T (&v)[VN]) {
  using V = typename VT<T, VN>::V;
  V x;
  if constexpr (VN == 4) {
    x.x = v[0]; x.y = v[1]; x.z = v[2]; x.w = v[3];
  } else {
    x.x = v[0]; x.y = v[1];
  }
  *reinterpret_cast<V*>(ptr) = x;
}

template <typename T, int VN>
__device__ __forceinline__ void vzero(T (&v)[VN]) {
#pragma unroll
  for (int q = 0; q < VN; ++q) v[q] = T(0);
}

// Vector load / store of elements base[q .. q+VN-1] of an array of n
// elements, bounds-checked in KH_DEBUG_BOUNDS builds (a load out of range
// reads zeros, a store is skipped).
template <typename T, int VN>
__device__ __forceinline__ void vld_at(const T* base, long long q, long long n, int site, T (&v)[VN]) {
  if (KH_IN(q, n, site) && KH_IN(q + VN - 1, n, site)) vld(base + q, v);
  else vzero(v);
}

template <typename T, int VN>
__device__ __forceinline__ void vst_at(T* base, long long q, long long n, int site, const T (&v)[VN]) {
  if (KH_IN(q, n, site) && KH_IN(q + VN - 1, n, site)) vst(base + q, v);
}

// E of a χ3 cell before its Kerr correction, into the ghost layers that the
// periodic wrap fills from this cell: the reference exchanges E halos at the
// end of step_E_fused! (Kernels.jl:452), before step_chi3_correction!.
template <typename T>
__device__ __forceinline__ void wrap_pre_chi3(const HalfStepParams<T>& p, long long q, int i, int j, int k,
                                              const T (&O)[3]) {
  const int co[3] = {i, j, k};
  const int na[3] = {p.nx, p.ny, p.nz};
  const long long st[3] = {1, p.pitch, p.plane};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!((p.periodic >> a) & 1u)) continue;
    const long long to[2] = {co[a] == na[a] - 1 ? q - (long long)na[a] * st[a] : -1,
                             co[a] == 0 ? q + (long long)na[a] * st[a] : -1};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      if (to[s] < 0 || !KH_IN(to[s], p.total, 1008)) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) p.O[c][to[s]] = O[c];
    }
  }
}

// Update of one cell that carries a source, χ3, a pole or a material
// conductivity (and may also sit in a CPML region).  t/u/w are the cell's B|D
// state and CPML U/W values (loaded and stored by the caller), m its μ⁻¹|ε⁻¹,
// a[] its CPML coefficients along x, y, z, c3 its χ3.  Conductivity (C, σ)
// and pole arrays are rare and read here directly.
template <typename T, bool H>
__device__ __forceinline__ void general_cell(const HalfStepParams<T>& p, long long q, int i, int j,
                                             int k, const bool (&f)[3], const AxisCoef<T> (&a)[3],
                                             uint32_t cls, bool special, const T (&K)[3],
                                             const T (&m)[3], T (&O)[3], T (&t)[3], T (&u)[3],
                                             T (&w)[3], T c3) {
  const bool region = f[0] || f[1] || f[2];
  bool regC = false;
  if (region && p.sigma_region_mask) {
    const int rx = i < p.pml_lo[0] ? 0 : (i >= p.nx - p.pml_hi[0] ? 2 : 1);
    const int ry = j < p.pml_lo[1] ? 0 : (j >= p.ny - p.pml_hi[1] ? 2 : 1);
    const int rz = k < p.pml_lo[2] ? 0 : (k >= p.nz - p.pml_hi[2] ? 2 : 1);
    regC = (p.sigma_region_mask >> (rx + 3 * ry + 9 * rz)) & 1u;
  }

  // Source term S of this half-step (update_source!, Sources.jl:346-357).
  T S0 = T(0), S1 = T(0), S2 = T(0);
  bool h0 = false, h1 = false, h2 = false;
  if (p.sources_active && (cls & (H ? kHasSrcH : kHasSrcE))) {
    const int slot = int(cls >> kSlotShift);
    const bool slot_ok = KH_IN(slot + 1, p.n_slots + 1, 1001);
    const int e1 = slot_ok ? p.slot_off[slot + 1] : 0;
    for (int e = slot_ok ? p.slot_off[slot] : 0; e < e1; ++e) {
      if (!KH_IN(e, p.n_ent, 1002)) break;
      const int c = p.ent_comp[e] - (H ? 3 : 0);  // entries carry components 0..5
      const Cplx<T> am = p.ent_amp[e];
      if (!KH_IN(p.ent_src[e], p.n_src, 1003)) continue;
      const Cplx<T> fv = p.f_now[p.ent_src[e]];
      const T v = fv.re * am.re - fv.im * am.im;  // real(f(t) · amplitude)
      if (c == 0) { S0 += v; h0 = true; }
      else if (c == 1) { S1 += v; h1 = true; }
      else if (c == 2) { S2 += v; h2 = true; }
    }
  }
  const T S[3] = {S0, S1, S2};
  const bool hasS[3] = {h0, h1, h2};

  // Total polarisation Σ_p P_p (accumulate_polarization_kernel!, Dispersive.jl:95-104).
  T Ptot[3] = {T(0), T(0), T(0)};
  if constexpr (!H) {
    if ((cls & kHasPole) && KH_IN(q, p.total, 1004)) {
      for (int pp = 0; pp < p.npoles; ++pp) {
        Ptot[0] += p.poles[pp].P[0][q];
        Ptot[1] += p.poles[pp].P[1][q];
        Ptot[2] += p.poles[pp].P[2][q];
      }
    }
  }

#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int nx_ = (c + 1) % 3, pv = (c + 2) % 3;
    const AxisCoef<T>& an = a[nx_];
    const AxisCoef<T>& ap = a[pv];
    const AxisCoef<T>& ao = a[c];
    const bool hasU = region && f[nx_];
    const bool hasW = region && f[c];
    const bool hasC = regC && (f[nx_] || f[pv]);
    const bool hasSD = region && p.msig[c] != nullptr;
    const bool keepT = special || (p.cpml ? region : (hasU || hasW || hasC || hasSD));
    if (!keepT) {
      O[c] = O[c] + m[c] * K[c];
      continue;
    }
    T tc = t[c];
    if (!region) {
      tc = tc + K[c];  // step_curl_and_update! (ReferenceKernels.jl:340-345)
    } else if (p.cpml) {
      // _cuda_pml_BH_kernel!/_cuda_pml_DE_kernel! stages (CUDAKernels.jl:150-281)
      T in_t = K[c];
      if (f[nx_] && an.s != T(0)) {
        const T un = (an.om * u[c] + K[c]) * an.ir;
        in_t = un - u[c];
        u[c] = un;
      }
      tc = (f[pv] && ap.s != T(0)) ? (ap.om * tc + in_t) * ap.ir : tc + in_t;
    } else {
      if (hasC && hasU && KH_IN(q, p.total, 1005)) {
        const T sD = hasSD ? T(0.5) * (p.dt * p.msig[c][q]) : T(0);
        const T uo = u[c];
        if (hasSD && sD != T(0)) {  // three-stage cascade (Helpers.jl:60-67)
          const T cc = p.C[c][q];
          const T cn = ((T(1) - sD) * cc + K[c]) / (T(1) + sD);
          p.C[c][q] = cn;
          u[c] = ((an.om * uo + cn) - cc) * an.ir;
        } else {  // two-stage cascade (Helpers.jl:53-59, 72-78)
          u[c] = (an.om * uo + K[c]) * an.ir;
        }
        tc = ((ap.om * tc + u[c]) - uo) * ap.ir;
      } else if (hasU) {  // C absent (Helpers.jl:113-139)
        if (an.s == T(0)) {
          tc = (ap.om * tc + K[c]) * ap.ir;
        } else {
          const T uo = u[c];
          u[c] = (an.om * uo + K[c]) * an.ir;
          tc = ((ap.om * tc + u[c]) - uo) * ap.ir;
        }
      } else if (hasSD && KH_IN(q, p.total, 1006)) {  // C and U absent, conductivity present (Helpers.jl:225-240)
        const T sD = T(0.5) * (p.dt * p.msig[c][q]);
        tc = ((T(1) - sD) * tc + K[c]) / (T(1) + sD);
      } else {  // C and U absent: σ_prev dropped (Helpers.jl:208-223)
        tc = tc + K[c];
      }
    }
    t[c] = tc;
    T net = tc;
    if (hasS[c]) net += S[c];
    if constexpr (!H) {
      if (cls & kHasPole) net -= Ptot[c];
    }
    if (hasW && ao.s != T(0)) {  // update_field_generic W cascade (Helpers.jl:333-339)
      const T wo = w[c];
      const T wn = m[c] * net;
      w[c] = wn;
      O[c] = (O[c] + ao.op * wn) - ao.om * wo;
    } else {
      O[c] = m[c] * net;
    }
  }

  if constexpr (!H) {
    // χ3 Kerr correction (Dispersive.jl:127-147)
    if ((cls & kHasChi3) && c3 != T(0)) {
      if (p.periodic) wrap_pre_chi3(p, q, i, j, k, O);
      const T esq = (O[0] * O[0] + O[1] * O[1]) + O[2] * O[2];
      const T corr = T(1) / (T(1) + c3 * esq);
      O[0] = O[0] * corr;
      O[1] = O[1] * corr;
      O[2] = O[2] * corr;
    }
    // ADE poles with E^{n+1} (Dispersive.jl:25-88)
    if ((cls & kHasPole) && KH_IN(q, p.total, 1007)) {
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
  }
}

// Update of a CPML-region cell without sources, χ3, poles or conductivity:
// the common case of the absorbing shell, with the stage logic fixed at
// compile time (CPML: CUDA-path stages; otherwise the CPU-path dispatch).
template <typename T, bool CPML>
__device__ __forceinline__ void pml_cell(const bool (&f)[3], const AxisCoef<T> (&a)[3], const T (&K)[3],
                                         const T (&m)[3], T (&O)[3], T (&t)[3], T (&u)[3], T (&w)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int nx_ = (c + 1) % 3, pv = (c + 2) % 3;
    const AxisCoef<T>& an = a[nx_];
    const AxisCoef<T>& ap = a[pv];
    const AxisCoef<T>& ao = a[c];
    if constexpr (CPML) {
      T in_t = K[c];
      if (f[nx_] && an.s != T(0)) {
        const T un = (an.om * u[c] + K[c]) * an.ir;
        in_t = un - u[c];
        u[c] = un;
      }
      t[c] = (f[pv] && ap.s != T(0)) ? (ap.om * t[c] + in_t) * ap.ir : t[c] + in_t;
    } else {
      if (!(f[nx_] || f[c])) {  // no auxiliary in this chunk: plain update
        O[c] = O[c] + m[c] * K[c];
        continue;
      }
      if (f[nx_]) {
        if (an.s == T(0)) {
          t[c] = (ap.om * t[c] + K[c]) * ap.ir;
        } else {
          const T un = (an.om * u[c] + K[c]) * an.ir;
          t[c] = ((ap.om * t[c] + un) - u[c]) * ap.ir;
          u[c] = un;
        }
      } else {
        t[c] = t[c] + K[c];  // σ_prev dropped (Helpers.jl:208-223)
      }
    }
    const T net = t[c];
    if (f[c] && ao.s != T(0)) {
      const T wn = m[c] * net;
      O[c] = (O[c] + ao.op * wn) - ao.om * w[c];
      w[c] = wn;
    } else {
      O[c] = m[c] * net;
    }
  }
}

// One fused half-step.  H = true: B/H from curl E; H = false: D/E from curl H.
// FULL = false (LEAN) compiles only plain and CPML cells; cells marked special
// there are source cells, updated as B|D-keeping cells (O = m⁻¹·T) and given
// their source term by source_fix_kernel when sources are active.
//
// The z march is software-pipelined: every load of plane k+1 (fields,
// neighbours, CPML state, cell classes) is issued before plane k is computed
// and stored, so each warp keeps two planes of memory traffic in flight.
}  // namespace kh
