// Set-up kernels of kh_sim_prepare (prepare_simulation!, src/Simulation.jl:92-283):
//   * material arrays uploaded compact (Center range, x fastest, in the
//     caller's precision) and scattered into the padded layout, converted to
//     the run's precision on the way;
//   * cell classification: χ3 and pole cells from the device material arrays,
//     source cells from the sparse source table;
//   * per-row-segment plane bitmasks of special cells that the half-step
//     kernels test before reading a cell class, and whether any special cell
//     lies in a CPML region (decides the CPU-path semantics' kernel variant);
//   * read-out of DFT accumulators with the Kahan compensation applied.
// All are one-pass HBM-bound kernels launched once per simulation (the
// read-out once per read).
#include <cuda_runtime.h>

#include <algorithm>

#include "kh_kernels.cuh"

namespace kh {

namespace {

// One CTA per (j, k) row of the Center range; threads stride along x.
template <typename Tin, typename T>
__global__ void scatter_center_kernel(const Tin* __restrict__ src, T* __restrict__ dst, int nx, int ny,
                                      long long pitch, long long plane, long long origin) {
  const long long row = blockIdx.x;
  const int j = int(row % ny);
  const long long k = row / ny;
  const Tin* s = src + row * nx;
  T* d = dst + origin + k * plane + (long long)j * pitch;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) d[i] = T(s[i]);
}

template <typename T>
__global__ void classify_kernel(const ClassifyArgs<T> a) {
  const long long row = blockIdx.x;
  const int j = int(row % a.n[1]);
  const long long k = row / a.n[1];
  const long long base = a.origin + k * a.plane + (long long)j * a.pitch;
  for (int i = threadIdx.x; i < a.n[0]; i += blockDim.x) {
    const long long q = base + i;
    uint32_t bits = 0;
    if (a.chi3 && a.chi3[q] != T(0)) bits |= kSpecialE | kHasChi3;
    for (int p = 0; p < a.npoles; ++p)
      if (a.pole_sigma[p][q] != T(0)) bits |= kSpecialE | kHasPole;
    if (bits) a.cls[q] |= bits;
  }
}

__global__ void mark_cells_kernel(const long long* __restrict__ cell, const uint32_t* __restrict__ bits, int n,
                                  uint32_t* cls) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) cls[cell[s]] |= bits[s];
}

// One warp per row segment of 32·kVN cells of plane k, row j: bit k%64 of
// word ((k/64)·ny + j)·nxb + xb is set when the segment holds special cells of
// that half.  Bit 0 / 1 of region_flags: a special E / H cell lies in a CPML
// region (a cell whose index is in the PML slab of any axis).
__global__ void tile_bits_kernel(const TileBitsArgs a) {
  const long long seg = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const long long nseg = (long long)a.n[2] * a.n[1] * a.nxb;
  if (seg >= nseg) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  const int xb = int(seg % a.nxb);
  const long long r = seg / a.nxb;
  const int j = int(r % a.n[1]);
  const int k = int(r / a.n[1]);
  auto flag = [&](int ax, int idx) { return idx < a.lo[ax] || idx >= a.n[ax] - a.hi[ax]; };
  const bool fjk = flag(1, j) || flag(2, k);
  bool e = false, h = false, er = false, hr = false;
#pragma unroll
  for (int v = 0; v < kVN; ++v) {
    const int i = xb * 32 * kVN + lane * kVN + v;
    if (i >= a.n[0]) continue;
    const uint32_t c = a.cls[a.origin + (long long)k * a.plane + (long long)j * a.pitch + i];
    const bool reg = fjk || flag(0, i);
    if (c & kSpecialE) { e = true; er |= reg; }
    if (c & kSpecialH) { h = true; hr |= reg; }
  }
  const bool ae = __any_sync(0xffffffffu, e), ah = __any_sync(0xffffffffu, h);
  const bool aer = __any_sync(0xffffffffu, er), ahr = __any_sync(0xffffffffu, hr);
  if (lane == 0) {
    const long long w = ((long long)(k >> 6) * a.n[1] + j) * a.nxb + xb;
    const unsigned long long bit = 1ull << (k & 63);
    if (ae) atomicOr(&a.bits_e[w], bit);
    if (ah) atomicOr(&a.bits_h[w], bit);
    if (aer) atomicOr(a.region_flags, 1u);
    if (ahr) atomicOr(a.region_flags, 2u);
  }
}

// One warp per row segment: flag 2 when it holds a pole cell, 1 when it holds
// χ3 cells only, 0 otherwise.
__global__ void disp_flags_kernel(const DispListArgs a) {
  const long long seg = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const long long nseg = (long long)a.n[2] * a.n[1] * a.nxb;
  if (seg >= nseg) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  const int xb = int(seg % a.nxb);
  const long long r = seg / a.nxb;
  const int j = int(r % a.n[1]);
  const int k = int(r / a.n[1]);
  bool c3 = false, pl = false;
#pragma unroll
  for (int v = 0; v < kVN; ++v) {
    const int i = xb * 32 * kVN + lane * kVN + v;
    if (i >= a.n[0]) continue;
    const uint32_t c = a.cls[a.origin + (long long)k * a.plane + (long long)j * a.pitch + i];
    c3 |= (c & kHasChi3) != 0;
    pl |= (c & kHasPole) != 0;
  }
  const bool apl = __any_sync(0xffffffffu, pl), ac3 = __any_sync(0xffffffffu, c3);
  if (lane == 0) a.flags[seg] = apl ? 2 : (ac3 ? 1 : 0);
}

// Ordered compaction of the flagged segments by one block: thread t scans a
// contiguous chunk, a shared-memory prefix sum gives its first output slot.
constexpr int kCompactThreads = 1024;
__global__ void __launch_bounds__(kCompactThreads) compact_segments_kernel(const DispListArgs a) {
  __shared__ int part[kCompactThreads];
  const long long nseg = (long long)a.n[2] * a.n[1] * a.nxb;
  const long long chunk = (nseg + kCompactThreads - 1) / kCompactThreads;
  const long long b = (long long)threadIdx.x * chunk;
  const long long e = b + chunk < nseg ? b + chunk : nseg;
  int n = 0;
  for (long long q = b; q < e; ++q) n += a.flags[q] != 0;
  part[threadIdx.x] = n;
  __syncthreads();
  for (int off = 1; off < kCompactThreads; off <<= 1) {
    const int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int pos = part[threadIdx.x] - n;
  for (long long q = b; q < e; ++q) {
    const unsigned char f = a.flags[q];
    if (f) a.list[pos++] = uint32_t(q) | (f == 2 ? 0x80000000u : 0u);
  }
  if (threadIdx.x == kCompactThreads - 1) *a.count = part[threadIdx.x];
}

template <typename T>
__global__ void dft_read_kernel(const Cplx<T>* __restrict__ F, const Cplx<T>* __restrict__ C, double* out,
                                long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    double re = double(F[q].re), im = double(F[q].im);
    if (C) {  // value = sum − compensation
      re -= double(C[q].re);
      im -= double(C[q].im);
    }
    out[2 * q] = re;
    out[2 * q + 1] = im;
  }
}

}  // namespace

template <typename Tin, typename T>
void launch_scatter_center(const Tin* src, T* dst, const int n[3], long long pitch, long long plane,
                           long long origin, void* stream) {
  const long long rows = (long long)n[1] * n[2];
  if (rows <= 0 || n[0] <= 0) return;
  const int threads = n[0] >= 256 ? 256 : 128;
  scatter_center_kernel<Tin, T><<<unsigned(rows), threads, 0, static_cast<cudaStream_t>(stream)>>>(
      src, dst, n[0], n[1], pitch, plane, origin);
}

template <typename T>
void launch_classify(const ClassifyArgs<T>& a, void* stream) {
  const long long rows = (long long)a.n[1] * a.n[2];
  if (rows <= 0 || (!a.chi3 && a.npoles == 0)) return;
  const int threads = a.n[0] >= 256 ? 256 : 128;
  classify_kernel<T><<<unsigned(rows), threads, 0, static_cast<cudaStream_t>(stream)>>>(a);
}

void launch_mark_cells(const long long* cell, const uint32_t* bits, int n, uint32_t* cls, void* stream) {
  if (n <= 0) return;
  mark_cells_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(cell, bits, n, cls);
}

void launch_tile_bits(const TileBitsArgs& a, void* stream) {
  const long long nseg = (long long)a.n[2] * a.n[1] * a.nxb;
  if (nseg <= 0) return;
  const int warps = 8;
  tile_bits_kernel<<<unsigned((nseg + warps - 1) / warps), 32 * warps, 0, static_cast<cudaStream_t>(stream)>>>(a);
}

void launch_disp_list(const DispListArgs& a, void* stream) {
  const long long nseg = (long long)a.n[2] * a.n[1] * a.nxb;
  if (nseg <= 0) return;
  const int warps = 8;
  disp_flags_kernel<<<unsigned((nseg + warps - 1) / warps), 32 * warps, 0, static_cast<cudaStream_t>(stream)>>>(a);
  compact_segments_kernel<<<1, kCompactThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
}

template <typename T>
void launch_dft_read(const Cplx<T>* F, const Cplx<T>* C, double* out, long long n, void* stream) {
  if (n <= 0) return;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 8);
  dft_read_kernel<T><<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(F, C, out, n);
}

template void launch_scatter_center<float, float>(const float*, float*, const int*, long long, long long,
                                                  long long, void*);
template void launch_scatter_center<double, float>(const double*, float*, const int*, long long, long long,
                                                   long long, void*);
template void launch_scatter_center<float, double>(const float*, double*, const int*, long long, long long,
                                                   long long, void*);
template void launch_scatter_center<double, double>(const double*, double*, const int*, long long, long long,
                                                    long long, void*);
template void launch_classify<float>(const ClassifyArgs<float>&, void*);
template void launch_classify<double>(const ClassifyArgs<double>&, void*);
template void launch_dft_read<float>(const Cplx<float>*, const Cplx<float>*, double*, long long, void*);
template void launch_dft_read<double>(const Cplx<double>*, const Cplx<double>*, double*, long long, void*);

}  // namespace kh
