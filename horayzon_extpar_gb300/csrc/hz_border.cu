// hz_border.cu -- distance of every cell circumcentre to the mesh border.
//
// Replaces functions.distance_to_border (functions.py:58-97), the diagnostic
// the reference's verification uses to set apart cells whose horizon is cut
// by the domain edge (verification.py:302-304): border vertices are the ICON
// vertices with a missing neighbour cell (a -2 in cells_of_vertex); cells and
// border vertices go to spherical ECEF with R = 6371.0087714 km; the result is
// the chord (Euclidean) distance from each cell to its nearest border vertex,
// in km, as the reference's KD-tree query returns it.
//
// On the GPU the nearest vertex is found by brute force over the border
// vertices, which a regional domain has along its perimeter only (thousands
// for millions of cells): a first sweep finds the FP32 minimum with both
// point sets relative to a reference point of the domain (coordinates below
// ~1e3 km, FP32 error below 1e-4 km); a second sweep evaluates the FP64
// distance, in the reference's expression order, for every vertex whose FP32
// distance lies within 1e-3 km of that minimum, and keeps the smallest.
#include <cmath>
#include <cstdio>

#include "../../include/horayzon_gb300.h"
#include "hz_internal.h"

namespace hz {
namespace {

constexpr double kRadE = 6371.0087714;  // functions.py:89 [km]
constexpr int kBorderTile = 1024;
constexpr float kRefineMargin = 1e-3f;  // km

// functions.py:90-92 / 95-97: rad_e * cos(lat) * cos(lon), ... (left to right)
__device__ __forceinline__ double3 ecef_km(double lon, double lat) {
  const double cl = cos(lat);
  return make_double3((kRadE * cl) * cos(lon), (kRadE * cl) * sin(lon), kRadE * sin(lat));
}

__global__ void k_border_collect(const double* __restrict__ vlon, const double* __restrict__ vlat,
                                 const int* __restrict__ cov, int nv, double3 ref,
                                 double3* __restrict__ bv64, float4* __restrict__ bv32,
                                 int* __restrict__ count) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  bool border = false;
#pragma unroll
  for (int k = 0; k < 6; k++) border |= cov[(long long)k * nv + v] == -2;  // functions.py:88
  if (!border) return;
  const int slot = atomicAdd(count, 1);
  const double3 p = ecef_km(vlon[v], vlat[v]);
  bv64[slot] = p;
  bv32[slot] = make_float4((float)(p.x - ref.x), (float)(p.y - ref.y), (float)(p.z - ref.z), 0.f);
}

__global__ void __launch_bounds__(256) k_border_nearest(
    const double* __restrict__ clon, const double* __restrict__ clat, int nc, double3 ref,
    const double3* __restrict__ bv64, const float4* __restrict__ bv32,
    const int* __restrict__ count, double* __restrict__ dist) {
  __shared__ float4 tile[kBorderTile];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = *count;
  double3 p = make_double3(0.0, 0.0, 0.0);
  float px = 0.f, py = 0.f, pz = 0.f;
  if (c < nc) {
    p = ecef_km(clon[c], clat[c]);
    px = (float)(p.x - ref.x);
    py = (float)(p.y - ref.y);
    pz = (float)(p.z - ref.z);
  }
  // Sweep 1: FP32 minimum of the squared distance.
  float best = INFINITY;
  for (int base = 0; base < nb; base += kBorderTile) {
    const int n = min(kBorderTile, nb - base);
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) tile[k] = bv32[base + k];
    __syncthreads();
    for (int k = 0; k < n; k++) {
      const float dx = px - tile[k].x, dy = py - tile[k].y, dz = pz - tile[k].z;
      best = fminf(best, dx * dx + dy * dy + dz * dz);
    }
  }
  // Sweep 2: FP64 distances of the candidates within the margin.
  const float lim = sqrtf(best) + kRefineMargin;
  const float lim2 = lim * lim;
  double d64 = INFINITY;
  for (int base = 0; base < nb; base += kBorderTile) {
    const int n = min(kBorderTile, nb - base);
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) tile[k] = bv32[base + k];
    __syncthreads();
    for (int k = 0; k < n; k++) {
      const float dx = px - tile[k].x, dy = py - tile[k].y, dz = pz - tile[k].z;
      if (dx * dx + dy * dy + dz * dz <= lim2) {
        const double3 q = bv64[base + k];
        const double ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
        d64 = fmin(d64, sqrt(((ex * ex) + (ey * ey)) + (ez * ez)));
      }
    }
  }
  if (c < nc) dist[c] = d64;
}

}  // namespace
}  // namespace hz

using namespace hz;

extern "C" int hz_distance_to_border(const double* clon, const double* clat,
                                     const double* vlon, const double* vlat,
                                     const int32_t* cells_of_vertex, int num_cell,
                                     int num_vertex, double* dist, int on_device,
                                     void* stream) {
  set_last_error("");
  if (num_cell < 0 || num_vertex < 0) {
    set_last_error("invalid array sizes");
    return HZ_ERR_VALUE;
  }
  if (num_cell == 0) return HZ_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t nc = (size_t)num_cell, nv = (size_t)(num_vertex > 0 ? num_vertex : 1);
  // One allocation: inputs (host calls), border points, counter, output.
  const size_t in_bytes = on_device ? 0 : (2 * nc + 2 * nv) * 8 + 6 * nv * 4;
  const size_t bytes = in_bytes + nv * (sizeof(double3) + sizeof(float4)) + 256 + nc * 8 + 1024;
  char* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "cudaMalloc failed: %s", cudaGetErrorString(e));
    set_last_error(msg);
    return HZ_ERR_CUDA;
  }
  size_t off = 0;
  auto take = [&](size_t n) {
    char* q = buf + off;
    off += (n + 255) & ~size_t(255);
    return q;
  };
  const double *d_clon = clon, *d_clat = clat, *d_vlon = vlon, *d_vlat = vlat;
  const int* d_cov = cells_of_vertex;
  double* d_dist = dist;
  // The first failing call is reported (after the buffer is freed).
  cudaError_t first = cudaSuccess;
  auto ck = [&](cudaError_t r) {
    if (first == cudaSuccess && r != cudaSuccess) first = r;
  };
  if (!on_device) {
    double* a = (double*)take(nc * 8);
    double* b = (double*)take(nc * 8);
    double* c = (double*)take(nv * 8);
    double* d = (double*)take(nv * 8);
    int* cv = (int*)take(6 * nv * 4);
    ck(cudaMemcpyAsync(a, clon, nc * 8, cudaMemcpyHostToDevice, s));
    ck(cudaMemcpyAsync(b, clat, nc * 8, cudaMemcpyHostToDevice, s));
    if (num_vertex > 0) {
      ck(cudaMemcpyAsync(c, vlon, nv * 8, cudaMemcpyHostToDevice, s));
      ck(cudaMemcpyAsync(d, vlat, nv * 8, cudaMemcpyHostToDevice, s));
      ck(cudaMemcpyAsync(cv, cells_of_vertex, 6 * nv * 4, cudaMemcpyHostToDevice, s));
    }
    d_clon = a;
    d_clat = b;
    d_vlon = c;
    d_vlat = d;
    d_cov = cv;
    d_dist = (double*)take(nc * 8);
  }
  double3* bv64 = (double3*)take(nv * sizeof(double3));
  float4* bv32 = (float4*)take(nv * sizeof(float4));
  int* count = (int*)take(4);
  // Reference point of the domain for the FP32 sweep: the first cell.
  double lon0 = 0.0, lat0 = 0.0;
  if (on_device) {
    ck(cudaMemcpyAsync(&lon0, clon, 8, cudaMemcpyDeviceToHost, s));
    ck(cudaMemcpyAsync(&lat0, clat, 8, cudaMemcpyDeviceToHost, s));
    ck(cudaStreamSynchronize(s));
  } else {
    lon0 = clon[0];
    lat0 = clat[0];
  }
  const double cl = std::cos(lat0);
  const double3 ref = make_double3((kRadE * cl) * std::cos(lon0), (kRadE * cl) * std::sin(lon0),
                                   kRadE * std::sin(lat0));
  ck(cudaMemsetAsync(count, 0, 4, s));
  if (num_vertex > 0) {
    k_border_collect<<<grid_for(num_vertex, 256), 256, 0, s>>>(d_vlon, d_vlat, d_cov,
                                                               num_vertex, ref, bv64, bv32,
                                                               count);
    ck(cudaGetLastError());
  }
  k_border_nearest<<<grid_for(num_cell, 256), 256, 0, s>>>(d_clon, d_clat, num_cell, ref, bv64,
                                                           bv32, count, d_dist);
  ck(cudaGetLastError());
  if (!on_device) ck(cudaMemcpyAsync(dist, d_dist, nc * 8, cudaMemcpyDeviceToHost, s));
  ck(cudaStreamSynchronize(s));
  e = first;
  cudaFree(buf);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "distance to border: %s", cudaGetErrorString(e));
    set_last_error(msg);
    return HZ_ERR_CUDA;
  }
  return HZ_OK;
}
