// hz_mesh.cu -- triangle-mesh assembly from the ICON grid and the geodetic
// frame transforms, one thread per ICON vertex / mesh vertex.
//
// mesh_count + scan + mesh_emit restate build_triangle_mesh
// (mo_lradtopo_horayzon.cpp:228-317) as a data-parallel pass: each vertex
// counts its triangles (and, for grid_type 1, its appended vertex), an
// exclusive scan turns the counts into output offsets, and each vertex then
// writes its triangles at its offset. The output order is the reference's:
// triangles by ICON vertex, appended vertices numbered ncell + k in vertex
// order. Neighbour cells are ordered by atan2(dlon, dlat) wrapped to [0, 2pi)
// with a stable insertion sort (std::sort of <= 16 elements, cpp:137-146, is
// an insertion sort). Sorted positions are mapped back to their
// cells_of_vertex slots; the reference indexes rows by position among the
// valid entries (cpp:265-271), which is the same whenever -2 entries trail.
#include "hz_internal.h"

namespace hz {

namespace {

__global__ void k_mesh_count(const int* __restrict__ cov, int nv, int ncell,
                             int grid_type, unsigned long long* __restrict__ packed,
                             int* __restrict__ err) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  int n = 0;
  bool bad = false;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    int c = cov[(long long)nv * j + v];
    if (c != -2) {
      if (c < 0 || c >= ncell) bad = true;
      else n++;
    }
  }
  if (bad) atomicOr(err, kErrBadIndex);
  unsigned tri, add;
  if (grid_type == 0) {
    tri = n >= 3 ? (unsigned)(n - 2) : 0u;
    add = 0u;
  } else {
    tri = n == 6 ? 6u : 0u;
    add = n == 6 ? 1u : 0u;
  }
  packed[v] = ((unsigned long long)add << 32) | tri;
}

__global__ void k_mesh_emit(const double* __restrict__ clon, const double* __restrict__ clat,
                            const double* __restrict__ hsurf, const double* __restrict__ vlon,
                            const double* __restrict__ vlat, const int* __restrict__ cov,
                            int nv, int ncell, int grid_type,
                            const unsigned long long* __restrict__ offsets,
                            int* __restrict__ vot, double* __restrict__ add_lon,
                            double* __restrict__ add_lat, double* __restrict__ add_h) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  // Order of the cells around the vertex by the reference's FP64 angle
  // atan2(dlon, dlat) in [0, 2 pi), stable (sort_index, cpp:137-146). The
  // order is taken from FP32 angles of the same differences (within 2e-6 rad
  // of the FP64 angle: argument rounding, atan2f, the 2 pi wrap) when every
  // gap between sorted angles, and to the wrap at 0 / 2 pi, exceeds
  // kAngleGap; then it is the FP64 order, with no ties. Otherwise (near-collinear
  // cells, or a cell due north) the FP64 angles are computed and sorted.
  constexpr float kAngleGap = 1e-5f;
  float ang[6];
  int cell[6], slot_cell[6];
  int n = 0;
  double hsum = 0.0;
  const double lon_v = vlon[v], lat_v = vlat[v];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    int c = cov[(long long)nv * j + v];
    if (c != -2 && c >= 0 && c < ncell) {
      float a = atan2f((float)(clon[c] - lon_v), (float)(clat[c] - lat_v));
      if (a < 0.f) a += 2.f * (float)kPi;
      ang[n] = a;
      cell[n] = c;
      slot_cell[n] = c;
      n++;
      hsum += hsurf[c];
    }
  }
  // Stable insertion sort of (angle, cell) pairs by angle.
  for (int k = 1; k < n; k++) {
    const float a = ang[k];
    const int c = cell[k];
    int m = k - 1;
    while (m >= 0 && a < ang[m]) {
      ang[m + 1] = ang[m];
      cell[m + 1] = cell[m];
      m--;
    }
    ang[m + 1] = a;
    cell[m + 1] = c;
  }
  bool clear = n == 0 || (ang[0] > kAngleGap && ang[n - 1] < 2.f * (float)kPi - kAngleGap);
  for (int k = 1; k < n; k++) clear = clear && ang[k] - ang[k - 1] > kAngleGap;
  if (!clear) {
    double a64[6];
    for (int k = 0; k < n; k++) {
      const int c = slot_cell[k];
      double a = atan2(clon[c] - lon_v, clat[c] - lat_v);
      if (a < 0.0) a += 2.0 * kPi;
      a64[k] = a;
      cell[k] = c;
    }
    for (int k = 1; k < n; k++) {
      const double a = a64[k];
      const int c = cell[k];
      int m = k - 1;
      while (m >= 0 && a < a64[m]) {
        a64[m + 1] = a64[m];
        cell[m + 1] = cell[m];
        m--;
      }
      a64[m + 1] = a;
      cell[m + 1] = c;
    }
  }
  const unsigned long long off = offsets[v];
  long long t = (long long)(off & 0xFFFFFFFFull);
  if (grid_type == 0) {
    if (n >= 3) {
      for (int k = 0; k < n - 2; k++, t++) {
        vot[3 * t + 0] = cell[0];
        vot[3 * t + 1] = cell[k + 1];
        vot[3 * t + 2] = cell[k + 2];
      }
    }
  } else if (n == 6) {
    int add = (int)(off >> 32);
    add_lon[add] = lon_v;
    add_lat[add] = lat_v;
    add_h[add] = hsum / 6.0;
    const int id = ncell + add;
#pragma unroll
    for (int k = 0; k < 6; k++, t++) {
      vot[3 * t + 0] = cell[k];
      vot[3 * t + 1] = cell[k == 5 ? 0 : k + 1];
      vot[3 * t + 2] = id;
    }
  }
}

constexpr int kEcefThreads = 256;

__global__ void k_mesh_ecef(const double* __restrict__ clon, const double* __restrict__ clat,
                            const double* __restrict__ hsurf,
                            const double* __restrict__ add_lon,
                            const double* __restrict__ add_lat,
                            const double* __restrict__ add_h, int ncell, int nadd,
                            double* __restrict__ ecef, double* __restrict__ block_sums) {
  __shared__ double sx[kEcefThreads], sy[kEcefThreads], sz[kEcefThreads];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nmv = ncell + nadd;
  double x = 0.0, y = 0.0, z = 0.0;
  if (i < nmv) {
    double lon, lat, h;
    if (i < ncell) {
      lon = clon[i]; lat = clat[i]; h = hsurf[i];
    } else {
      lon = add_lon[i - ncell]; lat = add_lat[i - ncell]; h = add_h[i - ncell];
    }
    // sincos: one argument reduction for both; the same bits as sin and cos
    // (compared on 2e8 arguments over [-pi, pi] on sm_103a).
    double sin_lon, cos_lon, sin_lat, cos_lat;
    sincos(lon, &sin_lon, &cos_lon);
    sincos(lat, &sin_lat, &cos_lat);
    x = (kEarthRadius + h) * cos_lat * cos_lon;
    y = (kEarthRadius + h) * cos_lat * sin_lon;
    z = (kEarthRadius + h) * sin_lat;
    ecef[3LL * i + 0] = x;
    ecef[3LL * i + 1] = y;
    ecef[3LL * i + 2] = z;
  }
  // Partial sums over cells only (fixed tree order: deterministic).
  const bool is_cell = i < ncell;
  sx[threadIdx.x] = is_cell ? x : 0.0;
  sy[threadIdx.x] = is_cell ? y : 0.0;
  sz[threadIdx.x] = is_cell ? z : 0.0;
  __syncthreads();
  for (int o = kEcefThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
      sz[threadIdx.x] += sz[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    block_sums[3LL * blockIdx.x + 0] = sx[0];
    block_sums[3LL * blockIdx.x + 1] = sy[0];
    block_sums[3LL * blockIdx.x + 2] = sz[0];
  }
}

__global__ void k_sum_blocks(const double* __restrict__ block_sums, int nb,
                             double* __restrict__ out) {
  __shared__ double sx[1024], sy[1024], sz[1024];
  double x = 0.0, y = 0.0, z = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    x += block_sums[3LL * b + 0];
    y += block_sums[3LL * b + 1];
    z += block_sums[3LL * b + 2];
  }
  sx[threadIdx.x] = x;
  sy[threadIdx.x] = y;
  sz[threadIdx.x] = z;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
      sz[threadIdx.x] += sz[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sx[0];
    out[1] = sy[0];
    out[2] = sz[0];
  }
}

__global__ void k_mesh_enu(const double* __restrict__ ecef, int nmv, int ncell, Frame f,
                           float* __restrict__ vert32, double* __restrict__ cell_enu,
                           float* __restrict__ vert_lo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nmv) return;
  const double dx = ecef[3LL * i + 0] - f.xe;
  const double dy = ecef[3LL * i + 1] - f.ye;
  const double dz = ecef[3LL * i + 2] - f.ze;
  // mo_lradtopo_horayzon.cpp:189-196, operation for operation.
  const double xn = (-f.sin_lon) * dx + f.cos_lon * dy;
  const double yn = f.cyx * dx - f.cyy * dy + f.cos_lat * dz;
  const double zn = f.czx * dx + f.czy * dy + f.sin_lat * dz;
  const float hx = (float)xn, hy = (float)yn, hz = (float)zn;
  vert32[3LL * i + 0] = hx;
  vert32[3LL * i + 1] = hy;
  vert32[3LL * i + 2] = hz;
  if (vert_lo) {
    // Residual of the FP32 rounding: hi + lo carries ~48 bits of the FP64 value.
    vert_lo[3LL * i + 0] = (float)(xn - (double)hx);
    vert_lo[3LL * i + 1] = (float)(yn - (double)hy);
    vert_lo[3LL * i + 2] = (float)(zn - (double)hz);
  }
  if (i < ncell) {
    cell_enu[3LL * i + 0] = xn;
    cell_enu[3LL * i + 1] = yn;
    cell_enu[3LL * i + 2] = zn;
  }
}

}  // namespace

cudaError_t mesh_count(const int* cov, int nv, int ncell, int grid_type,
                       unsigned long long* packed, int* err, cudaStream_t s) {
  if (nv <= 0) return cudaSuccess;
  k_mesh_count<<<grid_for(nv, 256), 256, 0, s>>>(cov, nv, ncell, grid_type, packed, err);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t mesh_emit(const double* clon, const double* clat, const double* hsurf,
                      const double* vlon, const double* vlat, const int* cov, int nv,
                      int ncell, int grid_type, const unsigned long long* offsets,
                      int* vot, double* add_lon, double* add_lat, double* add_h,
                      cudaStream_t s) {
  if (nv <= 0) return cudaSuccess;
  k_mesh_emit<<<grid_for(nv, 128), 128, 0, s>>>(clon, clat, hsurf, vlon, vlat, cov, nv,
                                                ncell, grid_type, offsets, vot, add_lon,
                                                add_lat, add_h);
  note_launches(1);
  return cudaGetLastError();
}

int ecef_blocks(int ncell_plus_nadd) { return (int)grid_for(ncell_plus_nadd, kEcefThreads); }

cudaError_t mesh_ecef(const double* clon, const double* clat, const double* hsurf,
                      const double* add_lon, const double* add_lat, const double* add_h,
                      int ncell, int nadd, double* ecef, double* block_sums,
                      double* d_origin_sum, cudaStream_t s) {
  int nb = ecef_blocks(ncell + nadd);
  k_mesh_ecef<<<nb, kEcefThreads, 0, s>>>(clon, clat, hsurf, add_lon, add_lat, add_h, ncell,
                                          nadd, ecef, block_sums);
  k_sum_blocks<<<1, 1024, 0, s>>>(block_sums, nb, d_origin_sum);
  note_launches(2);
  return cudaGetLastError();
}

// mo_lradtopo_horayzon.cpp:624-644 on the host (glibc), from the device sum
// of the cells' ECEF coordinates: origin direction, its lon / lat, the
// rotation terms and the Earth centre and North Pole in ENU. Every entry
// point builds its frame here, so the FP64 frame is the same bits for all.
Frame enu_frame_from_sum(double xo, double yo, double zo) {
  const double R = kEarthRadius;
  Frame f;
  const double radius = sqrt(xo * xo + yo * yo + zo * zo);
  const double lon_o = atan2(yo, xo);
  const double lat_o = asin(zo / radius);
  f.sin_lon = sin(lon_o);
  f.cos_lon = cos(lon_o);
  f.sin_lat = sin(lat_o);
  f.cos_lat = cos(lat_o);
  f.xe = R * cos(lat_o) * cos(lon_o);
  f.ye = R * cos(lat_o) * sin(lon_o);
  f.ze = R * sin(lat_o);
  f.cyx = (-f.sin_lat) * f.cos_lon;
  f.cyy = f.sin_lat * f.sin_lon;
  f.czx = f.cos_lat * f.cos_lon;
  f.czy = f.cos_lat * f.sin_lon;
  auto enu = [&](double x, double y, double z) {
    const double dx = x - f.xe, dy = y - f.ye, dz = z - f.ze;
    double3 r;
    r.x = (-f.sin_lon) * dx + f.cos_lon * dy;
    r.y = f.cyx * dx - f.cyy * dy + f.cos_lat * dz;
    r.z = f.czx * dx + f.czy * dy + f.sin_lat * dz;
    return r;
  };
  f.centre = enu(0.0, 0.0, 0.0);
  f.pole = enu(0.0, 0.0, R);
  return f;
}

cudaError_t mesh_enu(const double* ecef, int nmv, int ncell, const Frame& f, float* vert32,
                     double* cell_enu, float* vert_lo, cudaStream_t s) {
  if (nmv <= 0) return cudaSuccess;
  k_mesh_enu<<<grid_for(nmv, 256), 256, 0, s>>>(ecef, nmv, ncell, f, vert32, cell_enu,
                                                vert_lo);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace hz
