// hz_common.cuh -- shared device types, constants and helpers of the
// horizon / sky-view-factor library.
//
// Every translation unit of the library is compiled with -fmad=false: the
// reference's FP64 geometry (mo_lradtopo_horayzon.cpp:78-201, 490-555,
// 694-754) and the FP32 triangle test are evaluated with one rounding per
// operation, exactly as the host code does, so that hit decisions and the
// lattice of tested elevation angles are reproduced bit for bit. Multiply-adds
// that do not need to match are written explicitly with __fmaf_rn.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hz {

constexpr double kEarthRadius = 6371229.0;  // mo_lradtopo_horayzon.cpp:584
constexpr double kPi = 3.14159265358979323846;
constexpr double kInvPi = 1.0 / kPi;       // RN(1 / kPi) = 0x1.45f306dc9c883p-2
constexpr int kLeafMax = 2;                 // default triangles per BVH leaf (<= 8)
constexpr int kStackDepth = 64;             // >= LBVH depth (32 key + 32 index bits)
constexpr int kEmptyRef = INT32_MIN;        // no child / empty tree
constexpr int kMaxUpSteps = 720;            // one full turn of 0.5 deg steps

// Error bits raised by kernels (device word, read back by the host).
enum : int {
  kErrBadIndex = 1,     // cells_of_vertex entry outside [0, ncell) and != -2
  kErrStack = 2,        // traversal stack overflow
  kErrMeshCapacity = 4,  // mesh emission beyond the sized buffers
  kErrBounds = 8         // checked builds (HZ_CHECKED): an index outside its array
};

// Leaf references are negative: ~(start << 3 | (count - 1)).
__host__ __device__ __forceinline__ int leaf_ref(int start, int count) {
  return ~((start << 3) | (count - 1));
}
__host__ __device__ __forceinline__ int leaf_start(int ref) { return (~ref) >> 3; }
__host__ __device__ __forceinline__ int leaf_count(int ref) { return ((~ref) & 7) + 1; }

// BVH2 node, 64 bytes: both child boxes and both child references.
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (child0, child1, -, -) as int bits
struct __align__(16) Node {
  float4 a, b, c, d;
};

// BVH4 node, 128 bytes: the boxes of up to four children as structure of
// arrays (lane j of each float4 is child j) and their references; missing
// children have the reference kEmptyRef. Node i of the BVH4 array is BVH2 node
// i with each internal child replaced by that child's two children, so the
// internal children of a BVH4 node are BVH2 nodes two levels down and the
// BVH4 array is indexed like the BVH2 array (odd-level entries are unused).
struct __align__(16) Node4 {
  float4 lox, hix, loy, hiy, loz, hiz;
  int4 child;
  int4 pad;
};
constexpr int kStackDepth4 = 96;  // 3 pushes per BVH4 level

// Triangle record, 48 bytes, one float4 per axis: x = (v0.x, v1.x, v2.x,
// original id), y = (v0.y, v1.y, v2.y, 0), z = (v0.z, v1.z, v2.z, 0). A ray
// loads the axes in its own (kx, ky, kz) order by address offset.
struct __align__(16) Tri {
  float4 x, y, z;
};

// Global ENU frame of the domain (mo_lradtopo_horayzon.cpp:611-644).
struct Frame {
  double sin_lon, cos_lon, sin_lat, cos_lat;
  double xe, ye, ze;          // ECEF of the ENU origin on the sphere
  double cyx, cyy, czx, czy;  // (-sin_lat)*cos_lon, sin_lat*sin_lon,
                              // cos_lat*cos_lon, cos_lat*sin_lon
  double3 centre;             // Earth centre in ENU
  double3 pole;               // North Pole in ENU
};

// Order-preserving float <-> uint mapping for atomicMin/atomicMax.
__device__ __forceinline__ unsigned f2ord(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
// Block-wide bounds of ordered keys: v[0 .. kMin) reduced by min, v[kMin ..
// kMin + kMax) by max, over the whole block (blockDim.x a multiple of 32, at
// most 1024; every thread of the block calls it), then one atomicMin /
// atomicMax per value and block into out[]. Per-warp atomics on the same few
// addresses serialise at L2; per block there are 8 (or 32) times fewer.
template <int kMin, int kMax>
__device__ __forceinline__ void block_bounds_atomic(unsigned (&v)[kMin + kMax],
                                                    unsigned* out) {
  constexpr int kN = kMin + kMax;
  __shared__ unsigned part[kN][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < kN; i++) {
    v[i] = i < kMin ? __reduce_min_sync(0xffffffffu, v[i]) : __reduce_max_sync(0xffffffffu, v[i]);
    if (l == 0) part[i][w] = v[i];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int i = 0; i < kN; i++) {
      unsigned x = l < nw ? part[i][l] : (i < kMin ? 0xFFFFFFFFu : 0u);
      x = i < kMin ? __reduce_min_sync(0xffffffffu, x) : __reduce_max_sync(0xffffffffu, x);
      if (l == 0) {
        if (i < kMin) atomicMin(out + i, x);
        else atomicMax(out + i, x);
      }
    }
  }
}

__host__ __forceinline__ float ord2f_host(unsigned u) {
  unsigned v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  __builtin_memcpy(&f, &v, 4);
  return f;
}

// ---------------------------------------------------------------------------
// Launch helpers (host side, defined in hz_kernels_*.cu)
// ---------------------------------------------------------------------------

inline unsigned grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace hz
