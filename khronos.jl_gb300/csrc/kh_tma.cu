// TMA-staged fused half-step kernel for sm_103a.
//
// Same arithmetic as the register-pipelined kernel (general_cell / pml_cell
// of kh_cell.cuh), with the plane data moved by the Tensor Memory
// Accelerator: one elected thread per CTA issues cp.async.bulk.tensor loads of
// plane z (the three curl-source arrays with their x/y halo, the three
// updated arrays, the three m⁻¹ arrays) into a kTmaStages-deep shared-memory
// ring whose stages complete on mbarriers.  Bytes in flight then cost shared
// memory instead of registers, so a CTA keeps several planes of HBM traffic in
// flight while its warps compute.  The z neighbour of the curl comes from the
// adjacent stage; x and y neighbours from the halo in the same stage.
//
// CPML state (B|D, U, W) and cell classes are per-cell arrays with no
// neighbour reuse and exist only in part of the grid; they are prefetched into
// registers one plane ahead.
//
// Every mbarrier wait is bounded: after kWaitLimit polls the thread records
// KH_ERR_TIMEOUT in p.err, the CTA stops computing, waits (bounded) for the
// copies it issued and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/khronos_gb300.h"
#include "kh_cell.cuh"

namespace kh {

#ifdef KH_DEBUG_BOUNDS
KH_DBG_READER(dbg_read_tma)
#endif

namespace {

constexpr long long kWaitLimit = 1ll << 22;
constexpr long long kStallWaitLimit = 4096;  // the failure-detection test hook's limit

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with parity `parity`; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kWaitLimit) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// L2 prefetch of one tensor-map tile (no shared memory, no completion).
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}

__device__ __forceinline__ void l2_prefetch(const void* ptr) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
}

template <typename T>
struct TmaGeom {
  static constexpr int HX = 16 / int(sizeof(T));  // x halo of the curl-source box (16 bytes)
  static constexpr int XO = xoff<T>();             // padded x of cell x = 0
  static constexpr int AX = kTmaX + HX;          // A box row length
  static constexpr int A_BYTES = AX * (kTmaY + 1) * int(sizeof(T));
  static constexpr int A_ELEMS = ((A_BYTES + 127) / 128 * 128) / int(sizeof(T));
  static constexpr int O_ELEMS = kTmaX * kTmaY;
  static constexpr int STAGE = 3 * A_ELEMS + 6 * O_ELEMS;  // A0..2, O0..2, m0..2
  static constexpr size_t SMEM = size_t(kTmaStages) * STAGE * sizeof(T) + kTmaStages * sizeof(uint64_t);
};

// CPML state and cell classes of one thread's 2 cells, prefetched one plane ahead.
template <typename T>
struct AuxLoads {
  T t[3][2], u[3][2], w[3][2], c3[2];
  uint32_t cls[2];
  bool tf;
};

template <typename T, bool H, bool FULL>
__device__ __forceinline__ void load_aux(const HalfStepParams<T>& p, AuxLoads<T>& L, int k, long long row,
                                         bool lane_ok, bool fy, bool anyfx, uint64_t tbits) {
  const long long q = row + (long long)k * p.plane;
  L.tf = ((tbits >> (k & 63)) & 1ull) != 0;
  const bool fz = k < p.pml_lo[2] || k >= p.nz - p.pml_hi[2];
  const bool anyRegion = fy || fz || anyfx;
  const bool axis_any[3] = {anyfx, fy, fz};
  const bool aux = lane_ok && (anyRegion || L.tf);
#pragma unroll
  for (int v = 0; v < 2; ++v) L.cls[v] = (L.tf && lane_ok && KH_IN(q + v, p.total, 2001)) ? p.cell_class[q + v] : 0u;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (aux && p.Ts[c]) vld_at(p.Ts[c], q, p.total, 2002, L.t[c]); else vzero(L.t[c]);
    if (aux && anyRegion && p.U[c] && axis_any[(c + 1) % 3]) vld_at(p.U[c], q, p.total, 2003, L.u[c]);
    else vzero(L.u[c]);
    if (aux && anyRegion && p.W[c] && axis_any[c]) vld_at(p.W[c], q, p.total, 2004, L.w[c]); else vzero(L.w[c]);
  }
  if (FULL && !H && lane_ok && L.tf && p.chi3) vld_at(p.chi3, q, p.total, 2005, L.c3); else vzero(L.c3);
}

}  // namespace

// Resident CTAs per SM each variant is compiled for: the FULL variants
// (sources, χ3, poles, conductivity in-kernel) need more registers than the
// LEAN ones and would spill under the LEAN cap.
template <typename T, bool FULL>
constexpr int tma_min_blocks() {
  return sizeof(T) == 4 ? (FULL ? kTmaMinBlocks - 1 : kTmaMinBlocks) : 2;
}

template <typename T, bool H, bool CPML, bool FULL, bool STALL = false>
__global__ void __launch_bounds__(32 * kTmaY, (tma_min_blocks<T, FULL>()))
    half_step_tma_kernel(const HalfStepParams<T> p, const __grid_constant__ TmaMaps maps) {
  using G = TmaGeom<T>;
  constexpr int VN = 2;
  constexpr int s = H ? 1 : -1;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  T* stages = reinterpret_cast<T*>(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + size_t(kTmaStages) * G::STAGE * sizeof(T));

  const int lane = threadIdx.x;
  const int wy = threadIdx.y;
  const int tid = wy * 32 + lane;
  const int x_tile = blockIdx.x * kTmaX;
  const int y_tile = blockIdx.y * kTmaY;
  const int j = y_tile + wy;
  const bool row_ok = j < p.ny;
  const int x0 = x_tile + lane * VN;
  const bool lane_ok = row_ok && x0 < p.nx;
  const int k0 = blockIdx.z * p.zplanes;
  const int k1 = min(k0 + p.zplanes, p.nz);
  const int N = k1 - k0;  // planes computed; loads n = 0..N
  const bool pervox = p.m_inv[0] != nullptr;
  // the failure-detection test instantiation waits briefly for bytes that never come
  constexpr long long kLimit = STALL ? kStallWaitLimit : kWaitLimit;

  if (tid == 0) {
    for (int st = 0; st < kTmaStages; ++st) mbar_init(&bars[st], 1);
    mbar_fence_init();
  }
  __syncthreads();
  // tile-wide CPML flags along x and y: which CPML state tiles a plane needs
  const bool tfx = x_tile < p.pml_lo[0] || x_tile + kTmaX > p.nx - p.pml_hi[0];
  const bool tfy = y_tile < p.pml_lo[1] || y_tile + kTmaY > p.ny - p.pml_hi[1];

  // Load n brings the A arrays of plane (H: k0+n, E: k0-1+n) and, when that
  // plane is computed, its O and m⁻¹ tiles.
  const uint32_t a_bytes = 3u * uint32_t(G::A_BYTES);
  const uint32_t o_bytes = (pervox ? 6u : 3u) * uint32_t(G::O_ELEMS * sizeof(T));
  auto issue = [&](int n) {
    const int st = n % kTmaStages;
    T* dst = stages + st * G::STAGE;
    const int plane = H ? k0 + n : k0 - 1 + n;
    const bool comp = H ? (n < N) : (n >= 1);
    if (STALL && n == 0) {
      // failure-detection test instantiation: the first stage expects 16
      // bytes and no copy is issued into it, so the wait on it runs out and
      // nothing is left in flight when the CTA returns
      mbar_arrive_expect_tx(&bars[st], 16u);
      return;
    }
    mbar_arrive_expect_tx(&bars[st], a_bytes + (comp ? o_bytes : 0u));
    const int zc = plane + 1;                      // padded plane index
    const int ax = H ? G::XO + x_tile : G::XO - G::HX + x_tile;  // padded x of the A box
    const int ay = H ? 1 + y_tile : y_tile;        // padded y of the A box
#pragma unroll
    for (int c = 0; c < 3; ++c) tma_load_3d(dst + c * G::A_ELEMS, &maps.a[c], ax, ay, zc, &bars[st]);
    if (comp) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        tma_load_3d(dst + 3 * G::A_ELEMS + c * G::O_ELEMS, &maps.o[c], G::XO + x_tile, 1 + y_tile, zc,
                    &bars[st]);
      if (pervox) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          tma_load_3d(dst + 3 * G::A_ELEMS + (3 + c) * G::O_ELEMS, &maps.m[c], G::XO + x_tile, 1 + y_tile,
                      zc, &bars[st]);
      }
      // LEAN variants: the CPML state of the plane (B|D, U, W where the tile
      // touches the CPML of their axis) into L2, so that the per-thread
      // register loads a plane ahead of its update find it there.  Tiles that
      // keep state only for special cells are left to those loads (the
      // tile-bit lookup on the issuing thread would delay the ring); the FULL
      // variants, at their register limit, do without.  A tile that meets the
      // CPML only along x has state in 12 of its 64 columns: the whole-tile
      // prefetch pays off on the H half, while the E half, which runs at its
      // DRAM limit, loses more to the unused bytes than it gains.
      const bool tfz = plane < p.pml_lo[2] || plane >= p.nz - p.pml_hi[2];
      if (!FULL && (tfy || tfz || (H && tfx && p.xprefetch == 0))) {
        const bool af[3] = {tfx, tfy, tfz};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (p.Ts[c]) tma_prefetch_3d(&maps.t[c], G::XO + x_tile, 1 + y_tile, zc);
          if (p.U[c] && af[(c + 1) % 3]) tma_prefetch_3d(&maps.u[c], G::XO + x_tile, 1 + y_tile, zc);
          if (p.W[c] && af[c]) tma_prefetch_3d(&maps.w[c], G::XO + x_tile, 1 + y_tile, zc);
        }
      }
    }
  };
  if (tid == 0) {
    const int first = min(kTmaStages, N + 1);
    for (int n = 0; n < first; ++n) issue(n);
  }

  // static per-thread data along the march
  const long long row = p.origin + (long long)j * p.pitch + x0;
  const bool fy = row_ok && (j < p.pml_lo[1] || j >= p.ny - p.pml_hi[1]);
  // special-cell plane bits of this row segment for planes 64·g .. 64·g+63,
  // re-read when the march enters the next group of 64 planes
  const long long tb_base = (long long)j * p.nxb + blockIdx.x;
  const uint64_t* tb_row = (p.tile_bits && row_ok) ? p.tile_bits + tb_base : nullptr;
  const long long tb_group = (long long)p.ny * p.nxb;
  uint64_t tbits = (tb_row && KH_IN(tb_base + (long long)(k0 >> 6) * tb_group, p.n_tile_words, 2006))
                       ? tb_row[(long long)(k0 >> 6) * tb_group] : 0ull;
  bool fxv[VN];
  AxisCoef<T> axv[VN];
  bool anyfx = false;
#pragma unroll
  for (int v = 0; v < VN; ++v) {
    const int i = x0 + v;
    fxv[v] = lane_ok && i < p.nx && (i < p.pml_lo[0] || i >= p.nx - p.pml_hi[0]);
    anyfx |= fxv[v];
    axv[v] = (lane_ok && i < p.nx && KH_IN(i, p.nx, 2007)) ? p.ax[0][i] : AxisCoef<T>{T(0), T(1), T(1), T(1)};
  }
  const AxisCoef<T> ay = (row_ok && KH_IN(j, p.ny, 2008)) ? p.ax[1][j] : AxisCoef<T>{T(0), T(1), T(1), T(1)};
  // box coordinates of this thread's first cell in the A and O tiles
  const int bx = (H ? 0 : G::HX) + lane * VN;
  const int by = H ? wy : wy + 1;
  const int ob = wy * kTmaX + lane * VN;

  AuxLoads<T> cur;
  load_aux<T, H, FULL>(p, cur, k0, row, lane_ok, fy, anyfx, tbits);

  bool bad = false;
  AuxLoads<T> nxt;
  for (int c = 0; c < N; ++c) {
    const int k = k0 + c;
    if (c + 1 < N) {
      if (tb_row && ((k + 1) & 63) == 0 &&
          KH_IN(tb_base + (long long)((k + 1) >> 6) * tb_group, p.n_tile_words, 2009))
        tbits = tb_row[(long long)((k + 1) >> 6) * tb_group];
      load_aux<T, H, FULL>(p, nxt, k + 1, row, lane_ok, fy, anyfx, tbits);
    }
    // x-CPML lanes of rows outside the y and z CPML: their own state into L2
    // xpf_dist planes ahead (the tile-wide prefetch above would also pull the
    // columns that keep no state)
    if (!FULL && p.xprefetch > (H ? 0 : 1) && anyfx && !fy && lane_ok) {
      const int kp = k + p.xpf_dist;
      if (kp < k1 && !(kp < p.pml_lo[2] || kp >= p.nz - p.pml_hi[2])) {
        const long long qp = row + (long long)kp * p.plane;
        if (KH_IN(qp + 1, p.total, 2015)) {
#pragma unroll
          for (int cc = 0; cc < 3; ++cc)
            if (p.Ts[cc]) l2_prefetch(p.Ts[cc] + qp);
          if (p.U[2]) l2_prefetch(p.U[2] + qp);
          if (p.W[0]) l2_prefetch(p.W[0] + qp);
        }
      }
    }
    const int ncur = H ? c : c + 1;
    const int nnb = H ? c + 1 : c;
    bool ok = mbar_wait(&bars[ncur % kTmaStages], uint32_t((ncur / kTmaStages) & 1), kLimit);
    ok = ok && mbar_wait(&bars[nnb % kTmaStages], uint32_t((nnb / kTmaStages) & 1), kLimit);
    if (!ok) {
      bad = true;
      if (p.err) atomicExch(p.err, KH_ERR_TIMEOUT);
    }
    // shared-memory reach of this thread's cells (checked in KH_DEBUG_BOUNDS builds)
    const int a_chk = by * G::AX + bx;
    const bool smem_ok = KH_IN(a_chk + (H ? 0 : -1), G::A_ELEMS, 2010) && KH_IN(a_chk + (H ? 2 : 1), G::A_ELEMS, 2011) &&
                         KH_IN(a_chk + s * G::AX, G::A_ELEMS, 2012) &&
                         KH_IN(a_chk + s * G::AX + 1, G::A_ELEMS, 2013) && KH_IN(ob + 1, G::O_ELEMS, 2014);
    if (!bad && lane_ok && smem_ok) {
      using V2 = typename VT<T, 2>::V;
      const T* Sc = stages + (ncur % kTmaStages) * G::STAGE;
      const T* Sn = stages + (nnb % kTmaStages) * G::STAGE;
      const T* A0 = Sc;
      const T* A1 = Sc + G::A_ELEMS;
      const T* A2 = Sc + 2 * G::A_ELEMS;
      const T* B0 = Sn;
      const T* B1 = Sn + G::A_ELEMS;
      const T* Os = Sc + 3 * G::A_ELEMS;
      const T* Ms = Sc + 3 * G::A_ELEMS + 3 * G::O_ELEMS;
      const long long q = row + (long long)k * p.plane;
      // Both cells of the thread in one 8/16-byte shared load per array (a
      // is even and every tile row starts 16-byte aligned); the x neighbour
      // of one cell is the other cell of the pair, the other one a scalar load.
      const int a = by * G::AX + bx;
      const V2 c0 = *reinterpret_cast<const V2*>(A0 + a);
      const V2 c1 = *reinterpret_cast<const V2*>(A1 + a);
      const V2 c2 = *reinterpret_cast<const V2*>(A2 + a);
      const V2 n0 = *reinterpret_cast<const V2*>(B0 + a);
      const V2 n1 = *reinterpret_cast<const V2*>(B1 + a);
      const V2 y0 = *reinterpret_cast<const V2*>(A0 + a + s * G::AX);
      const V2 y2 = *reinterpret_cast<const V2*>(A2 + a + s * G::AX);
      T x1[VN], x2[VN];
      if constexpr (H) {  // forward difference: cell v reads x + 1
        x1[0] = c1.y; x2[0] = c2.y;
        x1[1] = A1[a + 2]; x2[1] = A2[a + 2];
      } else {            // backward difference: cell v reads x - 1
        x1[0] = A1[a - 1]; x2[0] = A2[a - 1];
        x1[1] = c1.x; x2[1] = c2.x;
      }
      const T cur0[VN] = {c0.x, c0.y}, cur1[VN] = {c1.x, c1.y}, cur2[VN] = {c2.x, c2.y};
      const T nb0[VN] = {n0.x, n0.y}, nb1[VN] = {n1.x, n1.y};
      const T yy0[VN] = {y0.x, y0.y}, yy2[VN] = {y2.x, y2.y};
      T K[3][VN], O[3][VN], m[3][VN];
#pragma unroll
      for (int v = 0; v < VN; ++v) {
        K[0][v] = p.cd[2] * (nb1[v] - cur1[v]) - p.cd[1] * (yy2[v] - cur2[v]);
        K[1][v] = p.cd[0] * (x2[v] - cur2[v]) - p.cd[2] * (nb0[v] - cur0[v]);
        K[2][v] = p.cd[1] * (yy0[v] - cur0[v]) - p.cd[0] * (x1[v] - cur1[v]);
      }
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        const V2 o = *reinterpret_cast<const V2*>(Os + cc * G::O_ELEMS + ob);
        O[cc][0] = o.x;
        O[cc][1] = o.y;
        if (pervox) {
          const V2 mm = *reinterpret_cast<const V2*>(Ms + cc * G::O_ELEMS + ob);
          m[cc][0] = mm.x;
          m[cc][1] = mm.y;
        } else {
          m[cc][0] = m[cc][1] = p.m_scalar;
        }
      }
      const bool fz = k < p.pml_lo[2] || k >= p.nz - p.pml_hi[2];
      // this thread's two cells have no CPML flag and no special class
      // (measured faster than a warp-uniform decision per row segment)
      bool plain = !(anyfx || fy || fz);
#pragma unroll
      for (int v = 0; v < VN; ++v) plain = plain && !(cur.cls[v] & (H ? kSpecialH : kSpecialE));
      if (plain) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
#pragma unroll
          for (int v = 0; v < VN; ++v) O[cc][v] = O[cc][v] + m[cc][v] * K[cc][v];
      } else {
        const AxisCoef<T> az = KH_IN(k, p.nz, 2020) ? p.ax[2][k] : AxisCoef<T>{T(0), T(1), T(1), T(1)};
#pragma unroll
        for (int v = 0; v < VN; ++v) {
          const int i = x0 + v;
          if (i >= p.nx) continue;
          const bool special = (cur.cls[v] & (H ? kSpecialH : kSpecialE)) != 0;
          if (!(fxv[v] || fy || fz || special)) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) O[cc][v] = O[cc][v] + m[cc][v] * K[cc][v];
            continue;
          }
          const bool fc[3] = {fxv[v], fy, fz};
          const AxisCoef<T> ac[3] = {axv[v], ay, az};
          const T Kc[3] = {K[0][v], K[1][v], K[2][v]};
          const T mc[3] = {m[0][v], m[1][v], m[2][v]};
          T Oc[3] = {O[0][v], O[1][v], O[2][v]};
          T tc[3] = {cur.t[0][v], cur.t[1][v], cur.t[2][v]};
          T uc[3] = {cur.u[0][v], cur.u[1][v], cur.u[2][v]};
          T wc[3] = {cur.w[0][v], cur.w[1][v], cur.w[2][v]};
          if constexpr (FULL) {
            if (!H && cur.cls[v] == (kSpecialE | kHasChi3) && !(fc[0] || fc[1] || fc[2])) {
              // χ3-only cell outside CPML: D += curl; E = ε⁻¹D; Kerr correction
              // (step_curl_and_update! + step_chi3_correction!, Dispersive.jl:127-147)
#pragma unroll
              for (int cc = 0; cc < 3; ++cc) {
                tc[cc] = tc[cc] + Kc[cc];
                Oc[cc] = mc[cc] * tc[cc];
              }
              if (cur.c3[v] != T(0)) {
                if (p.periodic) wrap_pre_chi3(p, q + v, i, j, k, Oc);
                const T esq = (Oc[0] * Oc[0] + Oc[1] * Oc[1]) + Oc[2] * Oc[2];
                const T corr = T(1) / (T(1) + cur.c3[v] * esq);
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) Oc[cc] = Oc[cc] * corr;
              }
            } else {
              general_cell<T, H>(p, q + v, i, j, k, fc, ac, cur.cls[v], special, Kc, mc, Oc, tc, uc, wc,
                                 cur.c3[v]);
            }
          } else {
            if (fc[0] || fc[1] || fc[2]) {
              pml_cell<T, CPML>(fc, ac, Kc, mc, Oc, tc, uc, wc);
            } else {  // source cell outside CPML: keeps its B|D state
#pragma unroll
              for (int cc = 0; cc < 3; ++cc) {
                tc[cc] = tc[cc] + Kc[cc];
                Oc[cc] = mc[cc] * tc[cc];
              }
            }
          }
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) {
            O[cc][v] = Oc[cc];
            cur.t[cc][v] = tc[cc];
            cur.u[cc][v] = uc[cc];
            cur.w[cc][v] = wc[cc];
          }
        }
        const bool anyRegion = fy || fz || anyfx;
        bool anySpecial = false;
#pragma unroll
        for (int v = 0; v < VN; ++v) anySpecial |= (cur.cls[v] & (H ? kSpecialH : kSpecialE)) != 0;
        if (anyRegion || anySpecial) {
          const bool axis_any[3] = {anyfx, fy, fz};
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) {
            if (p.Ts[cc]) vst_at(p.Ts[cc], q, p.total, 2015, cur.t[cc]);
            if (p.U[cc] && axis_any[(cc + 1) % 3]) vst_at(p.U[cc], q, p.total, 2016, cur.u[cc]);
            if (p.W[cc] && axis_any[cc]) vst_at(p.W[cc], q, p.total, 2017, cur.w[cc]);
          }
        }
      }
      if (x0 + VN <= p.nx) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) vst_at(p.O[cc], q, p.total, 2018, O[cc]);
      } else {
#pragma unroll
        for (int v = 0; v < VN; ++v)
          if (x0 + v < p.nx && KH_IN(q + v, p.total, 2019)) {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) p.O[cc][q + v] = O[cc][v];
          }
      }
    }
    // every thread is done with load c (H: current, E: z neighbour); its
    // stage takes load c + kTmaStages
    if (__syncthreads_or(bad)) {
      // stop: wait (bounded) for the copies this CTA issued, then leave
      if (tid == 0) {
        const int issued = min(c + kTmaStages, N + 1);
        for (int n = c; n < issued; ++n) mbar_wait(&bars[n % kTmaStages], uint32_t((n / kTmaStages) & 1), kLimit);
      }
      return;
    }
    if (tid == 0 && c + kTmaStages <= N) {
      fence_proxy_async();
      issue(c + kTmaStages);
    }
    cur = nxt;
  }
}

template <typename T>
size_t tma_smem_bytes() {
  return TmaGeom<T>::SMEM;
}

template <typename T, bool CPML, bool FULL>
static void launch_tma_variant(bool h_half, const HalfStepParams<T>& p, const TmaMaps& maps,
                               cudaStream_t st) {
  dim3 block(32, kTmaY, 1);
  dim3 grid((p.nx + kTmaX - 1) / kTmaX, (p.ny + kTmaY - 1) / kTmaY, (p.nz + p.zplanes - 1) / p.zplanes);
  const size_t smem = TmaGeom<T>::SMEM;
  if constexpr (sizeof(T) == 4 && !FULL) {
    if (p.stall_tx) {  // failure-detection test instantiation (FP32 LEAN only)
      if (h_half) half_step_tma_kernel<T, true, CPML, FULL, true><<<grid, block, smem, st>>>(p, maps);
      else half_step_tma_kernel<T, false, CPML, FULL, true><<<grid, block, smem, st>>>(p, maps);
      return;
    }
  }
  if (h_half) half_step_tma_kernel<T, true, CPML, FULL><<<grid, block, smem, st>>>(p, maps);
  else half_step_tma_kernel<T, false, CPML, FULL><<<grid, block, smem, st>>>(p, maps);
}

template <typename T>
void launch_half_step_tma(bool h_half, const HalfStepParams<T>& p, const TmaMaps& maps, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (p.cpml) {
    if (p.full) launch_tma_variant<T, true, true>(h_half, p, maps, st);
    else launch_tma_variant<T, true, false>(h_half, p, maps, st);
  } else {
    if (p.full) launch_tma_variant<T, false, true>(h_half, p, maps, st);
    else launch_tma_variant<T, false, false>(h_half, p, maps, st);
  }
}

template <typename T, bool H, bool CPML, bool FULL, bool STALL = false>
static int set_smem_attr() {
  return int(cudaFuncSetAttribute(half_step_tma_kernel<T, H, CPML, FULL, STALL>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(TmaGeom<T>::SMEM)));
}

template <typename T>
int prepare_tma_kernels() {
  int e = 0;
  e |= set_smem_attr<T, true, true, true>();
  e |= set_smem_attr<T, true, true, false>();
  e |= set_smem_attr<T, true, false, true>();
  e |= set_smem_attr<T, true, false, false>();
  e |= set_smem_attr<T, false, true, true>();
  e |= set_smem_attr<T, false, true, false>();
  e |= set_smem_attr<T, false, false, true>();
  e |= set_smem_attr<T, false, false, false>();
  if constexpr (sizeof(T) == 4) {
    e |= set_smem_attr<T, true, true, false, true>();
    e |= set_smem_attr<T, true, false, false, true>();
    e |= set_smem_attr<T, false, true, false, true>();
    e |= set_smem_attr<T, false, false, false, true>();
  }
  return e;
}

template <typename T>
int tma_resident_ctas() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, half_step_tma_kernel<T, true, true, false>, 32 * kTmaY,
                                                    TmaGeom<T>::SMEM) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

template size_t tma_smem_bytes<float>();
template size_t tma_smem_bytes<double>();
template void launch_half_step_tma<float>(bool, const HalfStepParams<float>&, const TmaMaps&, void*);
template void launch_half_step_tma<double>(bool, const HalfStepParams<double>&, const TmaMaps&, void*);
template int prepare_tma_kernels<float>();
template int prepare_tma_kernels<double>();
template int tma_resident_ctas<float>();
template int tma_resident_ctas<double>();

}  // namespace kh
