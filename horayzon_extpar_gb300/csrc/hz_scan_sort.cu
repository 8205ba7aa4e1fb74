// hz_scan_sort.cu -- device prefix sums and a stable LSD radix sort.
//
// Scan: three launches (tile reductions, one-block scan of the tile sums,
// tile scans with the carried offsets); 4096 elements per 1024-thread tile.
// Radix sort: 8-bit digits; per pass a per-tile digit histogram, an exclusive
// scan of the (digit-major, tile-minor) histogram, and a stable scatter that
// ranks keys inside a tile with warp match masks and per-warp digit counts.
#include "hz_internal.h"

namespace hz {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Inclusive block scan of one value per thread; returns the block total.
template <typename T>
__device__ __forceinline__ T block_incl_scan(T& v, T* warp_sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  v = warp_incl_scan(v);
  if (lane == 31) warp_sums[warp] = v;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nwarps ? warp_sums[lane] : T(0);
    w = warp_incl_scan(w);
    warp_sums[lane] = w;
  }
  __syncthreads();
  T total = warp_sums[nwarps - 1];
  if (warp > 0) v += warp_sums[warp - 1];
  __syncthreads();
  return total;
}

template <typename T>
__global__ void k_tile_reduce(const T* __restrict__ in, long long n, T* __restrict__ partials) {
  __shared__ T ws[32];
  long long base = (long long)blockIdx.x * kScanTile;
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    long long i = base + (long long)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  T total = block_incl_scan(s, ws);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

template <typename T>
__global__ void k_partials_scan(T* __restrict__ partials, long long np, T* __restrict__ total) {
  __shared__ T ws[32];
  T carry = 0;
  for (long long base = 0; base < np; base += kScanThreads) {
    long long i = base + threadIdx.x;
    T v = i < np ? partials[i] : T(0);
    T orig = v;
    T t = block_incl_scan(v, ws);
    if (i < np) partials[i] = carry + v - orig;
    carry += t;
  }
  if (threadIdx.x == 0) *total = carry;
}

template <typename T>
__global__ void k_tile_scan(const T* __restrict__ in, T* __restrict__ out, long long n,
                            const T* __restrict__ partials) {
  __shared__ T ws[32];
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  T loc[kScanItems];
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    long long i = base + k;
    loc[k] = i < n ? in[i] : T(0);
    s += loc[k];
  }
  T v = s;
  block_incl_scan(v, ws);
  T run = partials[blockIdx.x] + v - s;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    long long i = base + k;
    if (i < n) out[i] = run;
    run += loc[k];
  }
}

template <typename T>
cudaError_t scan_impl(const T* in, T* out, long long n, T* d_total, T* partials,
                      cudaStream_t s) {
  long long nb = (n + kScanTile - 1) / kScanTile;
  if (nb < 1) nb = 1;
  k_tile_reduce<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partials);
  k_partials_scan<T><<<1, kScanThreads, 0, s>>>(partials, nb, d_total);
  k_tile_scan<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, partials);
  note_launches(3);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsBins = 256;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void k_rs_hist(const uint32_t* __restrict__ keys, long long n, int shift,
                          uint32_t* __restrict__ hist, long long ntiles) {
  __shared__ uint32_t h[kRsBins];
  h[threadIdx.x] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * kRsTile;
#pragma unroll 4
  for (int k = 0; k < kRsItems; k++) {
    long long i = base + (long long)k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_rs_scatter(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                             uint32_t* __restrict__ kout, int32_t* __restrict__ vout,
                             long long n, int shift, const uint32_t* __restrict__ offs,
                             long long ntiles) {
  __shared__ uint32_t base_off[kRsBins];
  __shared__ uint32_t wcnt[kRsWarps][kRsBins];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  base_off[tid] = offs[(long long)tid * ntiles + blockIdx.x];
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kRsItems; r++) {
    long long i = (long long)blockIdx.x * kRsTile + (long long)r * kRsThreads + tid;
    bool valid = i < n;
    uint32_t key = valid ? kin[i] : 0u;
    int32_t val = valid ? vin[i] : 0;
    int digit = valid ? (int)((key >> shift) & 0xFFu) : kRsBins;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) wcnt[w][tid] = 0;
    __syncthreads();
    unsigned peers = __match_any_sync(0xffffffffu, digit);
    int rank = __popc(peers & lt_mask);
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) {
      uint32_t c = wcnt[w][tid];
      wcnt[w][tid] = run;
      run += c;
    }
    __syncthreads();
    if (valid) {
      uint32_t pos = base_off[digit] + wcnt[warp][digit] + rank;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    base_off[tid] += run;
  }
}

}  // namespace

long long scan_partials(long long n) {
  long long nb = (n + kScanTile - 1) / kScanTile;
  return nb < 1 ? 1 : nb;
}

cudaError_t scan_exclusive_u64(const unsigned long long* in, unsigned long long* out,
                               long long n, unsigned long long* d_total,
                               unsigned long long* partials, cudaStream_t s) {
  return scan_impl<unsigned long long>(in, out, n, d_total, partials, s);
}

cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n,
                               uint32_t* d_total, uint32_t* partials, cudaStream_t s) {
  return scan_impl<uint32_t>(in, out, n, d_total, partials, s);
}

// Scratch: hist[256 * ntiles] + offs[256 * ntiles] + scan partials + total.
size_t radix_scratch_u32(long long n) {
  long long ntiles = (n + kRsTile - 1) / kRsTile;
  if (ntiles < 1) ntiles = 1;
  long long nh = (long long)kRsBins * ntiles;
  return sizeof(uint32_t) * (size_t)(2 * nh + scan_partials(nh) + 4);
}

cudaError_t radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_alt,
                             int32_t* vals_alt, long long n, int bits, void* scratch,
                             cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  long long ntiles = (n + kRsTile - 1) / kRsTile;
  long long nh = (long long)kRsBins * ntiles;
  uint32_t* hist = (uint32_t*)scratch;
  uint32_t* offs = hist + nh;
  uint32_t* partials = offs + nh;
  uint32_t* total = partials + scan_partials(nh);
  uint32_t *ki = keys, *ko = keys_alt;
  int32_t *vi = vals, *vo = vals_alt;
  int passes = (bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    int shift = 8 * p;
    k_rs_hist<<<(unsigned)ntiles, kRsThreads, 0, s>>>(ki, n, shift, hist, ntiles);
    cudaError_t e = scan_exclusive_u32(hist, offs, nh, total, partials, s);
    if (e != cudaSuccess) return e;
    k_rs_scatter<<<(unsigned)ntiles, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, offs,
                                                         ntiles);
    note_launches(2);
    uint32_t* tk = ki; ki = ko; ko = tk;
    int32_t* tv = vi; vi = vo; vo = tv;
  }
  if (ki != keys) {
    cudaError_t e =
        cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(vals, vi, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace hz
