// hz_learn.cu -- learned warm start of the bracketing search.
//
// A small MLP proposes, per (cell, azimuth), the lattice elevation at which
// the bracketing search of mo_lradtopo_horayzon.cpp:525-547 starts; the
// search itself is unchanged and refines every proposal, so the MLP only
// decides where the first ray goes (the reference carries the previous
// azimuth's elevation over, cpp:511).
//
//   * k_raster_*: the mesh rasterised to a height field on a regular grid of
//     the domain's ENU x/y plane (maximum of the triangles covering a texel);
//   * k_features: 32 inputs per (cell, azimuth): terrain elevation angles,
//     seen from the ray origin in the cell's local frame, at 8 geometric
//     distances (~1.5 raster texels .. dist_search) x 4 azimuth offsets
//     around the azimuth (+-1/16, +-3/16 of the sector); fused with the MLP
//     for inference (start lattice index per (cell, azimuth));
//   * MLP 32 -> 64 -> 64 -> 1 (ReLU), weights rounded to BF16, FP32
//     accumulation; training kernels: forward with stored activations,
//     backward per sample, weight-gradient reductions over the batch, Adam.
#include <cuda_bf16.h>

#include <cmath>

#include "hz_internal.h"

namespace hz {

namespace {

constexpr int kIn = kMlpIn, kHid = kMlpHidden;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid,
              kW3 = kB2 + kHid, kB3 = kW3 + kHid;
static_assert(kB3 + 1 == kMlpParams, "parameter layout");

__device__ __forceinline__ float bf16r(float x) {
  return __bfloat162float(__float2bfloat16_rn(x));
}

// Loads the BF16-rounded parameters into shared memory.
__device__ __forceinline__ void load_params(float* __restrict__ w, const float* __restrict__ p) {
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = bf16r(p[i]);
  __syncthreads();
}

// Forward pass of one sample with weights in shared memory.
__device__ __forceinline__ float mlp_eval(const float* __restrict__ w, const float* x) {
  float h1[kHid];
#pragma unroll
  for (int j = 0; j < kHid; j++) h1[j] = w[kB1 + j];
#pragma unroll 4
  for (int i = 0; i < kIn; i++) {
    const float xi = x[i];
#pragma unroll
    for (int j = 0; j < kHid; j++) h1[j] = __fmaf_rn(w[kW1 + i * kHid + j], xi, h1[j]);
  }
#pragma unroll
  for (int j = 0; j < kHid; j++) h1[j] = fmaxf(h1[j], 0.f);
  float y = w[kB3];
#pragma unroll 2
  for (int j = 0; j < kHid; j++) {
    float a = w[kB2 + j];
#pragma unroll
    for (int i = 0; i < kHid; i++) a = __fmaf_rn(w[kW2 + i * kHid + j], h1[i], a);
    y = __fmaf_rn(w[kW3 + j], fmaxf(a, 0.f), y);
  }
  return y;
}

// ---------------------------------------------------------------------------
// Height raster
// ---------------------------------------------------------------------------
__global__ void k_raster_fill(unsigned* __restrict__ z, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = 0u;  // below every ordered float: "no terrain"
}

__global__ void k_raster_tris(const float* __restrict__ vert, const int* __restrict__ vot,
                              int n_tri, RasterDesc R, unsigned* __restrict__ z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tri) return;
  const int i0 = vot[3LL * t], i1 = vot[3LL * t + 1], i2 = vot[3LL * t + 2];
  const float ax = vert[3LL * i0], ay = vert[3LL * i0 + 1], az = vert[3LL * i0 + 2];
  const float bx = vert[3LL * i1], by = vert[3LL * i1 + 1], bz = vert[3LL * i1 + 2];
  const float cx = vert[3LL * i2], cy = vert[3LL * i2 + 1], cz = vert[3LL * i2 + 2];
  const float det = (bx - ax) * (cy - ay) - (cx - ax) * (by - ay);
  if (det == 0.f) return;
  const float idet = 1.f / det;
  const int gx0 = max(0, (int)floorf((fminf(fminf(ax, bx), cx) - R.x0) * R.inv_dx));
  const int gx1 = min(R.nx - 1, (int)ceilf((fmaxf(fmaxf(ax, bx), cx) - R.x0) * R.inv_dx));
  const int gy0 = max(0, (int)floorf((fminf(fminf(ay, by), cy) - R.y0) * R.inv_dx));
  const int gy1 = min(R.ny - 1, (int)ceilf((fmaxf(fmaxf(ay, by), cy) - R.y0) * R.inv_dx));
  const float eps = 1e-4f;
  for (int gy = gy0; gy <= gy1; gy++) {
    const float py = R.y0 + gy * R.dx;
    for (int gx = gx0; gx <= gx1; gx++) {
      const float px = R.x0 + gx * R.dx;
      const float l1 = ((px - ax) * (cy - ay) - (cx - ax) * (py - ay)) * idet;
      const float l2 = ((bx - ax) * (py - ay) - (px - ax) * (by - ay)) * idet;
      const float l0 = 1.f - l1 - l2;
      if (l0 < -eps || l1 < -eps || l2 < -eps) continue;
      const float h = l0 * az + l1 * bz + l2 * cz;
      atomicMax(&z[(long long)gy * R.nx + gx], f2ord(h));
    }
  }
}

__global__ void k_raster_finish(const unsigned* __restrict__ zi, float* __restrict__ zf,
                                long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) zf[i] = zi[i] == 0u ? -INFINITY : ord2f(zi[i]);
}

// Bilinear height; NaN outside the raster or where no triangle covers a corner.
__device__ __forceinline__ float raster_height(const RasterDesc& R, float x, float y) {
  const float fx = (x - R.x0) * R.inv_dx, fy = (y - R.y0) * R.inv_dx;
  const int ix = (int)floorf(fx), iy = (int)floorf(fy);
  if (ix < 0 || iy < 0 || ix + 1 >= R.nx || iy + 1 >= R.ny) return NAN;
  const float ux = fx - ix, uy = fy - iy;
  const float* z = R.z + (long long)iy * R.nx + ix;
  const float z00 = __ldg(z), z01 = __ldg(z + 1), z10 = __ldg(z + R.nx), z11 = __ldg(z + R.nx + 1);
  if (!(z00 > -INFINITY && z01 > -INFINITY && z10 > -INFINITY && z11 > -INFINITY)) return NAN;
  return (1.f - uy) * ((1.f - ux) * z00 + ux * z01) + uy * ((1.f - ux) * z10 + ux * z11);
}

// ---------------------------------------------------------------------------
// Features (+ fused inference)
// ---------------------------------------------------------------------------
constexpr int kLearnBlock = 128;

__global__ void __launch_bounds__(kLearnBlock)
    k_features(LearnParams q, const float* __restrict__ params) {
  extern __shared__ float w[];  // kMlpParams floats when params != nullptr
  if (params) load_params(w, params);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= q.cell_count) return;
  const int cell = q.cell_begin + k;
  // Cell frame (as the search: cpp:694-720), then FP32 for the features.
  const double qx = q.cell_enu[3LL * cell], qy = q.cell_enu[3LL * cell + 1],
               qz = q.cell_enu[3LL * cell + 2];
  double nx = qx - q.centre.x, ny = qy - q.centre.y, nz = qz - q.centre.z;
  double inv = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
  nx *= inv; ny *= inv; nz *= inv;
  const double vx = q.pole.x - qx, vy = q.pole.y - qy, vz = q.pole.z - qz;
  const double dp = vx * nx + vy * ny + vz * nz;
  double ex_ = vx - dp * nx, ey_ = vy - dp * ny, ez_ = vz - dp * nz;
  inv = 1.0 / sqrt(ex_ * ex_ + ey_ * ey_ + ez_ * ez_);
  const float Nx = (float)(ex_ * inv), Ny = (float)(ey_ * inv), Nz = (float)(ez_ * inv);
  const float Ux = (float)nx, Uy = (float)ny, Uz = (float)nz;
  // East = N x U.
  const float Ex = Ny * Uz - Nz * Uy, Ey = Nz * Ux - Nx * Uz, Ez = Nx * Uy - Ny * Ux;
  const float Ox = (float)(qx + nx * q.ray_org_elev);
  const float Oy = (float)(qy + ny * q.ray_org_elev);
  const float Oz = (float)(qz + nz * q.ray_org_elev);
  const float sector = 6.28318530717958647f / (float)q.nhori;
  const float off[4] = {-0.1875f * sector, -0.0625f * sector, 0.0625f * sector,
                        0.1875f * sector};
  // Distances: geometric from ~1.5 texels (the local slopes that set most
  // horizons on rough terrain) to dist_search.
  const float r0 = fminf(fmaxf(1.5f * q.raster.dx, q.dist_search * (1.f / 512.f)),
                         0.5f * q.dist_search);
  const float rstep = __powf(q.dist_search / r0, 1.f / 7.f);
  for (int a = 0; a < q.L_pred; a++) {
    const double2 cs = __ldg(&q.azim_cs[a]);
    float x[kIn];
#pragma unroll
    for (int s = 0; s < 4; s++) {
      float so, co;
      __sincosf(off[s], &so, &co);
      const float c = (float)cs.x * co - (float)cs.y * so;  // cos(theta + off)
      const float sn = (float)cs.y * co + (float)cs.x * so;  // sin(theta + off)
      const float hx = c * Nx + sn * Ex, hy = c * Ny + sn * Ey, hz = c * Nz + sn * Ez;
      float dist = r0;
#pragma unroll
      for (int r = 0; r < 8; r++, dist *= rstep) {
        const float px = Ox + dist * hx, py = Oy + dist * hy;
        const float zt = raster_height(q.raster, px, py);
        float f = -2.f;  // no terrain: -20 deg
        if (zt == zt) {
          const float dx = px - Ox, dy = py - Oy, dz = zt - Oz;
          const float up = dx * Ux + dy * Uy + dz * Uz;
          const float len2 = dx * dx + dy * dy + dz * dz;
          const float hor = sqrtf(fmaxf(len2 - up * up, 1e-6f));
          f = atan2f(up, hor) * (57.29577951308232f / 10.f);
        }
        x[s * 8 + r] = f;
      }
    }
    const long long e = (long long)a * q.ncell + cell;
    if (q.features) {
      float4* dst = reinterpret_cast<float4*>(q.features + e * kIn);
#pragma unroll
      for (int f = 0; f < kIn / 4; f++)
        dst[f] = make_float4(x[4 * f], x[4 * f + 1], x[4 * f + 2], x[4 * f + 3]);
    }
    if (params) {
      // Output y = j / 32 with the horizon h = j * 0.25 deg; the bracket that
      // ends at j = 2k - 1 starts best at lattice elevation k.
      const float y = mlp_eval(w, x);
      const float kf = rintf((y * 32.f + 1.f) * 0.5f);
      const int kk = (int)fminf(fmaxf(kf, (float)kMlpStartMin), (float)kMlpStartMax);
      q.start_m[e] = (int16_t)kk;
    }
  }
}

// ---------------------------------------------------------------------------
// Training
// ---------------------------------------------------------------------------
// Forward with stored post-ReLU activations, per-sample loss gradient, and
// the backward pass to the hidden layers (per sample).
__global__ void __launch_bounds__(128)
    k_mlp_train_fwd_bwd(const float* __restrict__ params, const float* __restrict__ X,
                        const float* __restrict__ T, int n, float* __restrict__ H1,
                        float* __restrict__ H2, float* __restrict__ G1,
                        float* __restrict__ G2, float* __restrict__ G3,
                        float* __restrict__ Y, float* __restrict__ loss) {
  extern __shared__ float w[];
  load_params(w, params);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (b < n) {
    float x[kIn];
#pragma unroll
    for (int i = 0; i < kIn; i++) x[i] = X[(long long)b * kIn + i];
    float h1[kHid];
#pragma unroll
    for (int j = 0; j < kHid; j++) h1[j] = w[kB1 + j];
#pragma unroll 4
    for (int i = 0; i < kIn; i++) {
#pragma unroll
      for (int j = 0; j < kHid; j++) h1[j] = __fmaf_rn(w[kW1 + i * kHid + j], x[i], h1[j]);
    }
#pragma unroll
    for (int j = 0; j < kHid; j++) {
      h1[j] = fmaxf(h1[j], 0.f);
      H1[(long long)b * kHid + j] = h1[j];
    }
    float y = w[kB3];
    for (int j = 0; j < kHid; j++) {
      float a = w[kB2 + j];
#pragma unroll
      for (int i = 0; i < kHid; i++) a = __fmaf_rn(w[kW2 + i * kHid + j], h1[i], a);
      a = fmaxf(a, 0.f);
      H2[(long long)b * kHid + j] = a;
      y = __fmaf_rn(w[kW3 + j], a, y);
    }
    Y[b] = y;
    const float d = y - T[b];
    l = d * d / (float)n;
    const float g = 2.f * d / (float)n;  // dLoss/dy, mean squared error
    G3[b] = g;
    // g2_j = g * W3_j * [h2_j > 0];  g1_i = sum_j W2_ij g2_j * [h1_i > 0]
    float g1[kHid];
#pragma unroll
    for (int i = 0; i < kHid; i++) g1[i] = 0.f;
    for (int j = 0; j < kHid; j++) {
      const float h2 = H2[(long long)b * kHid + j];
      const float g2 = h2 > 0.f ? g * w[kW3 + j] : 0.f;
      G2[(long long)b * kHid + j] = g2;
#pragma unroll
      for (int i = 0; i < kHid; i++) g1[i] = __fmaf_rn(w[kW2 + i * kHid + j], g2, g1[i]);
    }
#pragma unroll
    for (int i = 0; i < kHid; i++) G1[(long long)b * kHid + i] = h1[i] > 0.f ? g1[i] : 0.f;
  }
  // Loss: block reduction, one atomic per block.
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  __shared__ float red[4];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(loss, red[0] + red[1] + red[2] + red[3]);
}

// grad[p * Q + q] += sum_b A[b, p] * B[b, q] over this block's batch chunk
// (A == nullptr: A = 1, the bias gradient). 256 threads, P * Q <= 4096.
constexpr int kRedChunk = 512;
__global__ void __launch_bounds__(256)
    k_outer_reduce(const float* __restrict__ A, int P, const float* __restrict__ B, int Q,
                   int n, float* __restrict__ grad) {
  __shared__ float sa[64][64];
  __shared__ float sb[64][64];
  const int b0 = blockIdx.x * kRedChunk;
  const int nout = P * Q;
  float acc[16];
#pragma unroll
  for (int k = 0; k < 16; k++) acc[k] = 0.f;
  for (int base = b0; base < min(b0 + kRedChunk, n); base += 64) {
    const int m = min(64, n - base);
    for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
      const int r = idx / 64, c = idx % 64;
      sa[r][c] = (r < m && c < P) ? (A ? A[(long long)(base + r) * P + c] : 1.f) : 0.f;
      sb[r][c] = (r < m && c < Q) ? B[(long long)(base + r) * Q + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const int o = threadIdx.x + 256 * k;
      if (o < nout) {
        const int p = o / Q, qq = o % Q;
        float s = acc[k];
        for (int r = 0; r < m; r++) s = __fmaf_rn(sa[r][p], sb[r][qq], s);
        acc[k] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < 16; k++) {
    const int o = threadIdx.x + 256 * k;
    if (o < nout) atomicAdd(&grad[o], acc[k]);
  }
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_mlp_forward(const float* __restrict__ params, const float* __restrict__ X,
                              int n, float* __restrict__ Y) {
  extern __shared__ float w[];
  load_params(w, params);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  float x[kIn];
#pragma unroll
  for (int i = 0; i < kIn; i++) x[i] = X[(long long)b * kIn + i];
  Y[b] = mlp_eval(w, x);
}

}  // namespace

cudaError_t raster_build(const float* vert32, const int* vot, int n_tri, RasterDesc R,
                         unsigned* zbits, float* z, cudaStream_t s) {
  const long long n = (long long)R.nx * R.ny;
  k_raster_fill<<<grid_for(n, 256), 256, 0, s>>>(zbits, n);
  if (n_tri > 0)
    k_raster_tris<<<grid_for(n_tri, 128), 128, 0, s>>>(vert32, vot, n_tri, R, zbits);
  k_raster_finish<<<grid_for(n, 256), 256, 0, s>>>(zbits, z, n);
  note_launches(n_tri > 0 ? 3 : 2);
  return cudaGetLastError();
}

cudaError_t learn_features(const LearnParams& q, const float* params, cudaStream_t s) {
  if (q.cell_count <= 0) return cudaSuccess;
  const size_t smem = params ? sizeof(float) * kMlpParams : 0;
  if (smem > 48 * 1024) return cudaErrorInvalidValue;
  k_features<<<grid_for(q.cell_count, kLearnBlock), kLearnBlock, smem, s>>>(q, params);
  note_launches(1);
  return cudaGetLastError();
}

size_t mlp_train_scratch_floats(int n) { return (size_t)n * (4 * kHid + 2) + 64; }

cudaError_t mlp_train_step(float* params, float* adam_m, float* adam_v, const float* X,
                           const float* T, int n, int step, float lr, float* loss,
                           float* grads, float* scratch, cudaStream_t s) {
  if (n <= 0) return cudaErrorInvalidValue;
  float* H1 = scratch;
  float* H2 = H1 + (size_t)n * kHid;
  float* G1 = H2 + (size_t)n * kHid;
  float* G2 = G1 + (size_t)n * kHid;
  float* G3 = G2 + (size_t)n * kHid;
  float* Y = G3 + n;
  cudaError_t e = cudaMemsetAsync(grads, 0, sizeof(float) * kMlpParams, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  const size_t smem = sizeof(float) * kMlpParams;
  k_mlp_train_fwd_bwd<<<grid_for(n, 128), 128, smem, s>>>(params, X, T, n, H1, H2, G1, G2, G3,
                                                         Y, loss);
  const unsigned chunks = grid_for(n, kRedChunk);
  // dW1 = X^T G1, db1 = 1^T G1, dW2 = H1^T G2, db2 = 1^T G2, dW3 = H2^T G3, db3 = 1^T G3
  k_outer_reduce<<<chunks, 256, 0, s>>>(X, kIn, G1, kHid, n, grads + kW1);
  k_outer_reduce<<<chunks, 256, 0, s>>>(nullptr, 1, G1, kHid, n, grads + kB1);
  k_outer_reduce<<<chunks, 256, 0, s>>>(H1, kHid, G2, kHid, n, grads + kW2);
  k_outer_reduce<<<chunks, 256, 0, s>>>(nullptr, 1, G2, kHid, n, grads + kB2);
  k_outer_reduce<<<chunks, 256, 0, s>>>(H2, kHid, G3, 1, n, grads + kW3);
  k_outer_reduce<<<chunks, 256, 0, s>>>(nullptr, 1, G3, 1, n, grads + kB3);
  note_launches(7);
  if (lr > 0.f) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<grid_for(kMlpParams, 256), 256, 0, s>>>(params, adam_m, adam_v, grads, kMlpParams,
                                                     lr, b1, b2, 1e-8f, c1, c2);
    note_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t mlp_forward(const float* params, const float* X, int n, float* Y, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_mlp_forward<<<grid_for(n, 128), 128, sizeof(float) * kMlpParams, s>>>(params, X, n, Y);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace hz
