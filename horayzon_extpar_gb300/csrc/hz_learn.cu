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
//   * k_features: 32 inputs per (cell, azimuth): the sine of the terrain's
//     elevation angle, seen from the ray origin in the cell's local frame, at
//     8 geometric distances (~1.5 raster texels .. dist_search) x 4 azimuth
//     offsets around the azimuth (+-1/16, +-3/16 of the sector); one thread
//     per (cell, predicted azimuth), fused with the MLP for inference (start
//     lattice index per (cell, azimuth));
//   * MLP 32 -> 64 -> 64 -> 1 (ReLU) on the tensor cores: BF16 inputs,
//     weights and first hidden layer, FP32 accumulation (mma.sync m16n8k16;
//     a warp computes 16 or 32 samples x 64 hidden units per layer), the
//     last layer an FP32 dot product with BF16-rounded weights;
//   * training: one fused kernel per step computes forward, loss, backward
//     and the weight gradients of a batch (the batch reductions X^T G1 and
//     H1^T G2 as tensor-core products over the samples), then Adam.
//
// Rounding points (the FP64 oracle, oracle/mlp_ref.py, restates them): X,
// the weights and biases, and h1 = relu(X W1 + b1) are rounded to BF16; the
// backward pass rounds G2 = dL/da2 and G1 = dL/da1 to BF16 for the products
// G2 W2^T, H1^T G2 and X^T G1; everything else is FP32.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "hz_internal.h"

namespace hz {

namespace {

constexpr int kIn = kMlpIn, kHid = kMlpHidden;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid,
              kW3 = kB2 + kHid, kB3 = kW3 + kHid;
static_assert(kB3 + 1 == kMlpParams, "parameter layout");
static_assert(kIn == 32 && kHid == 64, "the tensor-core tiling assumes 32 -> 64 -> 64 -> 1");

__device__ __forceinline__ float bf16r(float x) {
  return __bfloat162float(__float2bfloat16_rn(x));
}

// ---------------------------------------------------------------------------
// Tensor-core helpers (mma.sync m16n8k16, BF16 in, FP32 accumulate).
// Fragment layouts (groupID g = lane / 4, thread-in-group t = lane % 4):
//   A 16x16 row major: reg0 (row g, cols 2t, 2t+1), reg1 (row g+8, same),
//                      reg2 (row g, cols 2t+8, 2t+9), reg3 (row g+8, same);
//   B 16x8  col major: reg0 (rows 2t, 2t+1, col g), reg1 (rows 2t+8, 2t+9);
//   C 16x8:  c0, c1 (row g, cols 2t, 2t+1), c2, c3 (row g+8, same).
// Two C tiles of adjacent 8-column blocks are, packed to BF16, the A
// fragment of the 16-column k-block they span (the next layer's input).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
      "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Four 8x8 BF16 matrices from shared memory; lanes 8q .. 8q + 7 give the row
// addresses of matrix q (16-byte aligned). .trans delivers the transposed
// fragment: lane gets (row 2t, 2t+1; col g) of the stored matrix.
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

// Row strides (BF16 elements) of the shared tiles: 16-byte aligned rows, and
// the eight row addresses of an 8x8 matrix fall in distinct bank groups.
constexpr int kXStride = kIn + 8;   // 40 (80 bytes)
constexpr int kHStride = kHid + 8;  // 72 (144 bytes)

// Weights in shared memory: the B fragments of W1 (k = input, n = hidden),
// W2 (k = hidden 1, n = hidden 2) and, for training, W2^T (k = hidden 2, n =
// hidden 1), each as [k-block][n-block][lane] pairs of packed BF16; biases
// and W3 as BF16-rounded FP32.
struct __align__(16) MlpWeights {
  uint2 w1f[2 * 8 * 32];
  uint2 w2f[4 * 8 * 32];
  float b1[kHid], b2[kHid], w3[kHid];
  float b3;
};
struct __align__(16) MlpWeightsT {
  uint2 w2tf[4 * 8 * 32];
};

// B fragment (kb, nb) of a row-major K x N matrix W (W[k * ldw + n]), or of
// its transpose when kTrans (B[k][n] = W[n * ldw + k]).
template <bool kTrans>
__device__ __forceinline__ uint2 b_frag(const float* __restrict__ W, int ldw, int kb, int nb,
                                        int lane) {
  const int g = lane >> 2, t = lane & 3;
  const int k0 = kb * 16 + 2 * t, n = nb * 8 + g;
  auto w = [&](int k) { return kTrans ? W[n * ldw + k] : W[k * ldw + n]; };
  return make_uint2(pack_bf16(w(k0), w(k0 + 1)), pack_bf16(w(k0 + 8), w(k0 + 9)));
}

// Packs the parameters (global FP32) into shared memory; all threads of the
// block call it.
__device__ __forceinline__ void load_weights(MlpWeights* S, MlpWeightsT* T,
                                             const float* __restrict__ p) {
  for (int f = threadIdx.x; f < 2 * 8 * 32; f += blockDim.x) {
    const int lane = f & 31, nb = (f >> 5) & 7, kb = f >> 8;
    S->w1f[f] = b_frag<false>(p + kW1, kHid, kb, nb, lane);
  }
  for (int f = threadIdx.x; f < 4 * 8 * 32; f += blockDim.x) {
    const int lane = f & 31, nb = (f >> 5) & 7, kb = f >> 8;
    S->w2f[f] = b_frag<false>(p + kW2, kHid, kb, nb, lane);
    if (T) T->w2tf[f] = b_frag<true>(p + kW2, kHid, kb, nb, lane);
  }
  for (int j = threadIdx.x; j < kHid; j += blockDim.x) {
    S->b1[j] = bf16r(p[kB1 + j]);
    S->b2[j] = bf16r(p[kB2 + j]);
    S->w3[j] = bf16r(p[kW3 + j]);
  }
  if (threadIdx.x == 0) S->b3 = bf16r(p[kB3]);
  __syncthreads();
}

// Forward pass of one 16-row tile whose BF16 inputs are rows row0 ..
// row0 + 15 of Xs (stride kXStride). Returns the second layer's
// pre-activations a2 (C tiles, 8 x 4) and the first layer's BF16 activations
// as A fragments of layer 2 (h1a, 4 k-blocks x 4), and the output y of rows
// g and g + 8 (in every lane of the quad).
struct TileFwd {
  float a2[8][4];
  uint32_t h1a[4][4];
  float y_lo, y_hi;
};

__device__ __forceinline__ void tile_forward(const MlpWeights& W, const __nv_bfloat16* Xs,
                                             int row0, int lane, TileFwd& o) {
  const int t = lane & 3;
  // A fragments of X: matrices (rows 0-7 | 8-15) x (cols 0-7 | 8-15) of each
  // 16-column k-block.
  uint32_t ax[2][4];
  {
    const int q = lane >> 3, r = lane & 7;
    const __nv_bfloat16* base = Xs + (row0 + r + (q & 1) * 8) * kXStride + (q >> 1) * 8;
    ldsm_x4(ax[0], base);
    ldsm_x4(ax[1], base + 16);
  }
  float c1[8][4];
#pragma unroll
  for (int nb = 0; nb < 8; nb++) {
    const float b0 = W.b1[nb * 8 + 2 * t], b1 = W.b1[nb * 8 + 2 * t + 1];
    c1[nb][0] = b0; c1[nb][1] = b1; c1[nb][2] = b0; c1[nb][3] = b1;
  }
#pragma unroll
  for (int kb = 0; kb < 2; kb++)
#pragma unroll
    for (int nb = 0; nb < 8; nb++) mma_bf16(c1[nb], ax[kb], W.w1f[(kb * 8 + nb) * 32 + lane]);
#pragma unroll
  for (int kb = 0; kb < 4; kb++) {
    o.h1a[kb][0] = pack_bf16(fmaxf(c1[2 * kb][0], 0.f), fmaxf(c1[2 * kb][1], 0.f));
    o.h1a[kb][1] = pack_bf16(fmaxf(c1[2 * kb][2], 0.f), fmaxf(c1[2 * kb][3], 0.f));
    o.h1a[kb][2] = pack_bf16(fmaxf(c1[2 * kb + 1][0], 0.f), fmaxf(c1[2 * kb + 1][1], 0.f));
    o.h1a[kb][3] = pack_bf16(fmaxf(c1[2 * kb + 1][2], 0.f), fmaxf(c1[2 * kb + 1][3], 0.f));
  }
#pragma unroll
  for (int nb = 0; nb < 8; nb++) {
    const float b0 = W.b2[nb * 8 + 2 * t], b1 = W.b2[nb * 8 + 2 * t + 1];
    o.a2[nb][0] = b0; o.a2[nb][1] = b1; o.a2[nb][2] = b0; o.a2[nb][3] = b1;
  }
#pragma unroll
  for (int kb = 0; kb < 4; kb++)
#pragma unroll
    for (int nb = 0; nb < 8; nb++) mma_bf16(o.a2[nb], o.h1a[kb], W.w2f[(kb * 8 + nb) * 32 + lane]);
  float lo = 0.f, hi = 0.f;
#pragma unroll
  for (int nb = 0; nb < 8; nb++) {
    const float w0 = W.w3[nb * 8 + 2 * t], w1 = W.w3[nb * 8 + 2 * t + 1];
    lo = __fmaf_rn(w0, fmaxf(o.a2[nb][0], 0.f), lo);
    lo = __fmaf_rn(w1, fmaxf(o.a2[nb][1], 0.f), lo);
    hi = __fmaf_rn(w0, fmaxf(o.a2[nb][2], 0.f), hi);
    hi = __fmaf_rn(w1, fmaxf(o.a2[nb][3], 0.f), hi);
  }
  lo += __shfl_xor_sync(0xffffffffu, lo, 1);
  lo += __shfl_xor_sync(0xffffffffu, lo, 2);
  hi += __shfl_xor_sync(0xffffffffu, hi, 1);
  hi += __shfl_xor_sync(0xffffffffu, hi, 2);
  o.y_lo = lo + W.b3;
  o.y_hi = hi + W.b3;
}

// The 32 samples of a warp (rows 0-31 of its Xs slice, written by the warp's
// lanes): each lane gets the output of its own row. Ys: 32 floats of the warp.
__device__ __forceinline__ float warp_forward32(const MlpWeights& W, const __nv_bfloat16* Xs,
                                                float* Ys, int lane) {
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 2; m++) {
    TileFwd o;
    tile_forward(W, Xs, 16 * m, lane, o);
    if ((lane & 3) == 0) {
      Ys[16 * m + (lane >> 2)] = o.y_lo;
      Ys[16 * m + (lane >> 2) + 8] = o.y_hi;
    }
  }
  __syncwarp();
  return Ys[lane];
}

// One row of 32 FP32 inputs to BF16 in Xs (stride kXStride).
__device__ __forceinline__ void store_row_bf16(__nv_bfloat16* row, const float (&x)[kIn]) {
#pragma unroll
  for (int f = 0; f < kIn; f += 8) {
    uint4 v;
    v.x = pack_bf16(x[f], x[f + 1]);
    v.y = pack_bf16(x[f + 2], x[f + 3]);
    v.z = pack_bf16(x[f + 4], x[f + 5]);
    v.w = pack_bf16(x[f + 6], x[f + 7]);
    *reinterpret_cast<uint4*>(row + f) = v;
  }
}

// ---------------------------------------------------------------------------
// Height raster
// ---------------------------------------------------------------------------
// The raster over the triangle-centre bounds of the BVH build (ordered
// floats: min x, min y, max x, max y) with a margin of 4 texels: square
// texels, as fine as `budget` texels allow. One thread; the descriptor stays
// on the device, so the learned start needs no host readback.
__global__ void k_raster_setup(const unsigned* __restrict__ bounds, int n_tri, long long budget,
                               float4* quad, RasterDesc* __restrict__ out) {
  RasterDesc R;
  R.nx = R.ny = 1;
  R.dx = R.inv_dx = 1.f;
  R.x0 = R.y0 = 0.f;
  if (n_tri > 0) {
    const float x0 = ord2f(bounds[0]), y0 = ord2f(bounds[1]);
    const float x1 = ord2f(bounds[2]), y1 = ord2f(bounds[3]);
    const double ex = fmax(1.0, (double)x1 - x0), ey = fmax(1.0, (double)y1 - y0);
    double dx = sqrt(ex * ey / (0.9 * (double)budget));
    for (int it = 0; it < 200; it++) {
      const long long nx = (long long)ceil(ex / dx) + 8, ny = (long long)ceil(ey / dx) + 8;
      if (nx * ny <= budget) {
        R.nx = (int)nx;
        R.ny = (int)ny;
        break;
      }
      dx *= 1.05;
    }
    R.dx = (float)dx;
    R.inv_dx = (float)(1.0 / dx);
    R.x0 = (float)(x0 - 4.0 * dx);
    R.y0 = (float)(y0 - 4.0 * dx);
  }
  R.quad = quad;
  *out = R;
}

__global__ void k_raster_fill(unsigned* __restrict__ z, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = 0u;  // below every ordered float: "no terrain"
}

__global__ void k_raster_tris(const float* __restrict__ vert, const int* __restrict__ vot,
                              int n_tri, const RasterDesc* __restrict__ Rp,
                              unsigned* __restrict__ z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tri) return;
  const RasterDesc R = *Rp;
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

__device__ __forceinline__ float raster_texel(const unsigned* __restrict__ zi, long long i) {
  const unsigned v = __ldg(zi + i);
  return v == 0u ? -INFINITY : ord2f(v);
}

// The quads of the finished raster; the last row and column, which no
// bilinear sample reads, get -inf neighbours.
__global__ void k_raster_finish(const unsigned* __restrict__ zi, float4* __restrict__ quad,
                                const RasterDesc* __restrict__ Rp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = Rp->nx, ny = Rp->ny;
  if (i >= (long long)nx * ny) return;
  const int ix = (int)(i % nx), iy = (int)(i / nx);
  const bool rx = ix + 1 < nx, ry = iy + 1 < ny;
  quad[i] = make_float4(raster_texel(zi, i), rx ? raster_texel(zi, i + 1) : -INFINITY,
                        ry ? raster_texel(zi, i + nx) : -INFINITY,
                        rx && ry ? raster_texel(zi, i + nx + 1) : -INFINITY);
}

// Bilinear height; NaN outside the raster or where no triangle covers a corner.
__device__ __forceinline__ float raster_height(const RasterDesc& R, float x, float y) {
  const float fx = (x - R.x0) * R.inv_dx, fy = (y - R.y0) * R.inv_dx;
  const int ix = (int)floorf(fx), iy = (int)floorf(fy);
  if (ix < 0 || iy < 0 || ix + 1 >= R.nx || iy + 1 >= R.ny) return NAN;
  const float ux = fx - ix, uy = fy - iy;
  const float4 c = __ldg(R.quad + (long long)iy * R.nx + ix);
  const float z00 = c.x, z01 = c.y, z10 = c.z, z11 = c.w;
  if (!(z00 > -INFINITY && z01 > -INFINITY && z10 > -INFINITY && z11 > -INFINITY)) return NAN;
  return (1.f - uy) * ((1.f - ux) * z00 + ux * z01) + uy * ((1.f - ux) * z10 + ux * z11);
}

// ---------------------------------------------------------------------------
// Features (+ fused inference)
// ---------------------------------------------------------------------------
constexpr int kLearnBlock = 128;
constexpr int kLearnWarps = kLearnBlock / 32;

// One thread per (cell, predicted azimuth q): azimuth a = q * a_stride, items
// ordered azimuth-major so that a warp's 32 samples share the azimuth.
__global__ void __launch_bounds__(kLearnBlock)
    k_features(LearnParams q, const float* __restrict__ params) {
  __shared__ MlpWeights W;
  __shared__ __align__(16) __nv_bfloat16 Xs[kLearnWarps][32 * kXStride];
  __shared__ float Ys[kLearnWarps][32];
  if (params) load_weights(&W, nullptr, params);
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)q.cell_count * q.n_pred;
  const bool valid = k < total;
  const RasterDesc raster = *q.raster;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float x[kIn];
  int cell = 0, a = 0;
  if (valid) {
    const int qa = (int)(k / q.cell_count);
    cell = q.cell_begin + (int)(k - (long long)qa * q.cell_count);
    a = qa * q.a_stride;
    // Local frame of the cell in FP32 (the search's frame is FP64; the
    // features need only its direction to about 1e-6): up U = the sphere
    // normal, north N = the pole direction projected on the tangent plane,
    // east E = N x U; ray origin O 0.2 m (ray_org_elev) above the cell.
    const double qx = q.cell_enu[3LL * cell], qy = q.cell_enu[3LL * cell + 1],
                 qz = q.cell_enu[3LL * cell + 2];
    float ux = (float)(qx - q.centre.x), uy = (float)(qy - q.centre.y),
          uz = (float)(qz - q.centre.z);
    float inv = rsqrtf(ux * ux + uy * uy + uz * uz);
    ux *= inv; uy *= inv; uz *= inv;
    const float vx = (float)(q.pole.x - qx), vy = (float)(q.pole.y - qy),
                vz = (float)(q.pole.z - qz);
    const float dp = vx * ux + vy * uy + vz * uz;
    float nx = vx - dp * ux, ny = vy - dp * uy, nz = vz - dp * uz;
    inv = rsqrtf(nx * nx + ny * ny + nz * nz);
    nx *= inv; ny *= inv; nz *= inv;
    const float ex = ny * uz - nz * uy, ey = nz * ux - nx * uz, ez = nx * uy - ny * ux;
    (void)ez;
    const float elev = (float)q.ray_org_elev;
    const float Ox = (float)qx + ux * elev, Oy = (float)qy + uy * elev, Oz = (float)qz + uz * elev;
    const float sector = 6.28318530717958647f / (float)q.nhori;
    const float off[4] = {-0.1875f * sector, -0.0625f * sector, 0.0625f * sector,
                          0.1875f * sector};
    // Distances: geometric from ~1.5 texels (the local slopes that set most
    // horizons on rough terrain) to dist_search.
    const float r0 = fminf(fmaxf(1.5f * raster.dx, q.dist_search * (1.f / 512.f)),
                           0.5f * q.dist_search);
    const float rstep = __powf(q.dist_search / r0, 1.f / 7.f);
    const double2 cs = __ldg(&q.azim_cs[a]);
#pragma unroll
    for (int s = 0; s < 4; s++) {
      float so, co;
      __sincosf(off[s], &so, &co);
      const float c = (float)cs.x * co - (float)cs.y * so;   // cos(theta + off)
      const float sn = (float)cs.y * co + (float)cs.x * so;  // sin(theta + off)
      const float hx = c * nx + sn * ex, hy = c * ny + sn * ey;
      float dist = r0;
#pragma unroll
      for (int r = 0; r < 8; r++, dist *= rstep) {
        const float dx = dist * hx, dy = dist * hy;
        const float zt = raster_height(raster, Ox + dx, Oy + dy);
        float f = -2.f;  // no terrain
        if (zt == zt) {
          // sin(elevation) of the terrain point seen from O, times 5.
          const float dz = zt - Oz;
          const float up = dx * ux + dy * uy + dz * uz;
          const float len2 = dx * dx + dy * dy + dz * dz;
          f = 5.f * up * rsqrtf(fmaxf(len2, 1e-6f));
        }
        x[s * 8 + r] = f;
      }
    }
    if (q.features) {
      float4* dst = reinterpret_cast<float4*>(q.features + ((long long)a * q.ncell + cell) * kIn);
#pragma unroll
      for (int f = 0; f < kIn / 4; f++)
        dst[f] = make_float4(x[4 * f], x[4 * f + 1], x[4 * f + 2], x[4 * f + 3]);
    }
  } else {
#pragma unroll
    for (int f = 0; f < kIn; f++) x[f] = 0.f;
  }
  if (!params) return;  // block-uniform: no weights were loaded
  // Inference: the warp's 32 samples through the tensor cores.
  store_row_bf16(&Xs[w][lane * kXStride], x);
  const float y = warp_forward32(W, Xs[w], Ys[w], lane);
  if (valid) {
    // Output y = j / 32 with the horizon h = j * 0.25 deg; the bracket that
    // ends at j = 2k - 1 starts best at lattice elevation k.
    const float kf = rintf((y * 32.f + 1.f) * 0.5f);
    const int kk = (int)fminf(fmaxf(kf, (float)kMlpStartMin), (float)kMlpStartMax);
    q.start_m[(long long)a * q.ncell + cell] = (int16_t)kk;
  }
}

// Y[n] = MLP(X[n][32]): a warp per 32 samples.
__global__ void __launch_bounds__(kLearnBlock)
    k_mlp_forward(const float* __restrict__ params, const float* __restrict__ X, int n,
                  float* __restrict__ Y) {
  __shared__ MlpWeights W;
  __shared__ __align__(16) __nv_bfloat16 Xs[kLearnWarps][32 * kXStride];
  __shared__ float Ys[kLearnWarps][32];
  load_weights(&W, nullptr, params);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float x[kIn];
  if (b < n) {
    const float4* src = reinterpret_cast<const float4*>(X + b * kIn);
#pragma unroll
    for (int f = 0; f < kIn / 4; f++) {
      const float4 v = __ldg(src + f);
      x[4 * f] = v.x; x[4 * f + 1] = v.y; x[4 * f + 2] = v.z; x[4 * f + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int f = 0; f < kIn; f++) x[f] = 0.f;
  }
  store_row_bf16(&Xs[w][lane * kXStride], x);
  const float y = warp_forward32(W, Xs[w], Ys[w], lane);
  if (b < n) Y[b] = y;
}

// ---------------------------------------------------------------------------
// Training: forward, loss, backward and weight gradients of a batch in one
// kernel. A block takes chunks of 64 samples (16 per warp); per chunk each
// warp runs its 16-row tile forward and backward on the tensor cores and
// leaves X, H1, G2, G1 (BF16) in shared memory; then the block's warps
// reduce the chunk into their slices of dW2 = H1^T G2 and dW1 = X^T G1
// (tensor-core products with the samples as the k dimension), kept in
// registers across chunks and added to the gradient once per block.
// ---------------------------------------------------------------------------
constexpr int kTrainChunk = 64;

struct __align__(16) TrainTiles {
  __nv_bfloat16 X[kTrainChunk * kXStride];
  __nv_bfloat16 H1[kTrainChunk * kHStride];
  __nv_bfloat16 G2[kTrainChunk * kHStride];
  __nv_bfloat16 G1[kTrainChunk * kHStride];
};

__global__ void __launch_bounds__(kLearnBlock)
    k_mlp_train(const float* __restrict__ params, const float* __restrict__ X,
                const float* __restrict__ T, int n, float* __restrict__ grads,
                float* __restrict__ loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpWeights& W = *reinterpret_cast<MlpWeights*>(smem_raw);
  MlpWeightsT& WT = *reinterpret_cast<MlpWeightsT*>(smem_raw + sizeof(MlpWeights));
  TrainTiles& S = *reinterpret_cast<TrainTiles*>(smem_raw + sizeof(MlpWeights) +
                                                 sizeof(MlpWeightsT));
  load_weights(&W, &WT, params);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const float inv_n = 1.f / (float)n;
  // Accumulators over this block's chunks.
  float dW2[8][4];   // rows 16 w + (g, g + 8) of dW2, all 64 columns
  float dW1[4][4];   // rows 16 (w & 1) + (g, g + 8), columns 32 (w >> 1) .. + 32
  float db1[16], db2[16], dw3[16];  // columns nb * 8 + 2 t (+ 1), rows g and g + 8 summed
  float db3 = 0.f, lsum = 0.f;
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int c = 0; c < 4; c++) dW2[i][c] = 0.f;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int c = 0; c < 4; c++) dW1[i][c] = 0.f;
#pragma unroll
  for (int i = 0; i < 16; i++) { db1[i] = 0.f; db2[i] = 0.f; dw3[i] = 0.f; }

  const int nchunks = (n + kTrainChunk - 1) / kTrainChunk;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int s0 = ch * kTrainChunk + 16 * w;  // first sample of the warp's tile
    // X rows of the tile to BF16 (lane: row lane / 2, half lane % 2).
    {
      const int r = lane >> 1, h = lane & 1;
      const int s = s0 + r;
      float x[16];
      if (s < n) {
        const float4* src = reinterpret_cast<const float4*>(X + (long long)s * kIn + 16 * h);
#pragma unroll
        for (int f = 0; f < 4; f++) {
          const float4 v = __ldg(src + f);
          x[4 * f] = v.x; x[4 * f + 1] = v.y; x[4 * f + 2] = v.z; x[4 * f + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int f = 0; f < 16; f++) x[f] = 0.f;
      }
      __nv_bfloat16* row = &S.X[(16 * w + r) * kXStride + 16 * h];
#pragma unroll
      for (int f = 0; f < 16; f += 8) {
        uint4 v;
        v.x = pack_bf16(x[f], x[f + 1]);
        v.y = pack_bf16(x[f + 2], x[f + 3]);
        v.z = pack_bf16(x[f + 4], x[f + 5]);
        v.w = pack_bf16(x[f + 6], x[f + 7]);
        *reinterpret_cast<uint4*>(row + f) = v;
      }
    }
    __syncwarp();
    TileFwd o;
    tile_forward(W, S.X, 16 * w, lane, o);
    // Loss gradient of rows g and g + 8: dL/dy = 2 (y - t) / n.
    const int sl = s0 + g, sh = s0 + g + 8;
    const float tl = sl < n ? __ldg(T + sl) : 0.f, th = sh < n ? __ldg(T + sh) : 0.f;
    const float dl = sl < n ? o.y_lo - tl : 0.f, dh = sh < n ? o.y_hi - th : 0.f;
    if (t == 0) lsum += dl * dl + dh * dh;
    const float gl = 2.f * dl * inv_n, gh = 2.f * dh * inv_n;
    if (t == 0) db3 += gl + gh;
    // G2 = g W3 [a2 > 0] (FP32 sums, BF16 for the products), dW3 = g h2.
    uint32_t g2a[4][4];
#pragma unroll
    for (int nb = 0; nb < 8; nb++) {
      const float w0 = W.w3[nb * 8 + 2 * t], w1 = W.w3[nb * 8 + 2 * t + 1];
      const float q0 = o.a2[nb][0] > 0.f ? gl * w0 : 0.f;
      const float q1 = o.a2[nb][1] > 0.f ? gl * w1 : 0.f;
      const float q2 = o.a2[nb][2] > 0.f ? gh * w0 : 0.f;
      const float q3 = o.a2[nb][3] > 0.f ? gh * w1 : 0.f;
      db2[2 * nb] += q0 + q2;
      db2[2 * nb + 1] += q1 + q3;
      dw3[2 * nb] += gl * fmaxf(o.a2[nb][0], 0.f) + gh * fmaxf(o.a2[nb][2], 0.f);
      dw3[2 * nb + 1] += gl * fmaxf(o.a2[nb][1], 0.f) + gh * fmaxf(o.a2[nb][3], 0.f);
      const uint32_t plo = pack_bf16(q0, q1), phi = pack_bf16(q2, q3);
      g2a[nb >> 1][(nb & 1) * 2] = plo;
      g2a[nb >> 1][(nb & 1) * 2 + 1] = phi;
      *reinterpret_cast<uint32_t*>(&S.G2[(16 * w + g) * kHStride + nb * 8 + 2 * t]) = plo;
      *reinterpret_cast<uint32_t*>(&S.G2[(16 * w + g + 8) * kHStride + nb * 8 + 2 * t]) = phi;
    }
    // H1 (BF16) of the tile for dW2, from its A fragments.
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
      __nv_bfloat16* r0 = &S.H1[(16 * w + g) * kHStride + kb * 16 + 2 * t];
      __nv_bfloat16* r8 = &S.H1[(16 * w + g + 8) * kHStride + kb * 16 + 2 * t];
      *reinterpret_cast<uint32_t*>(r0) = o.h1a[kb][0];
      *reinterpret_cast<uint32_t*>(r8) = o.h1a[kb][1];
      *reinterpret_cast<uint32_t*>(r0 + 8) = o.h1a[kb][2];
      *reinterpret_cast<uint32_t*>(r8 + 8) = o.h1a[kb][3];
    }
    // G1 = (G2 W2^T) [h1 > 0].
    float c1[8][4];
#pragma unroll
    for (int nb = 0; nb < 8; nb++)
#pragma unroll
      for (int c = 0; c < 4; c++) c1[nb][c] = 0.f;
#pragma unroll
    for (int kb = 0; kb < 4; kb++)
#pragma unroll
      for (int nb = 0; nb < 8; nb++) mma_bf16(c1[nb], g2a[kb], WT.w2tf[(kb * 8 + nb) * 32 + lane]);
#pragma unroll
    for (int nb = 0; nb < 8; nb++) {
      // h1 > 0 from its BF16 A fragment: block nb lies in k-block nb / 2,
      // registers 0 / 1 (rows g / g + 8) for even nb, 2 / 3 for odd nb.
      const uint32_t hlo = o.h1a[nb >> 1][(nb & 1) * 2];
      const uint32_t hhi = o.h1a[nb >> 1][(nb & 1) * 2 + 1];
      // A BF16 value is > 0 iff its sign bit is clear and it is not zero.
      const float q0 = ((hlo & 0xFFFFu) != 0u && !(hlo & 0x8000u)) ? c1[nb][0] : 0.f;
      const float q1 = ((hlo >> 16) != 0u && !(hlo & 0x80000000u)) ? c1[nb][1] : 0.f;
      const float q2 = ((hhi & 0xFFFFu) != 0u && !(hhi & 0x8000u)) ? c1[nb][2] : 0.f;
      const float q3 = ((hhi >> 16) != 0u && !(hhi & 0x80000000u)) ? c1[nb][3] : 0.f;
      db1[2 * nb] += q0 + q2;
      db1[2 * nb + 1] += q1 + q3;
      *reinterpret_cast<uint32_t*>(&S.G1[(16 * w + g) * kHStride + nb * 8 + 2 * t]) =
          pack_bf16(q0, q1);
      *reinterpret_cast<uint32_t*>(&S.G1[(16 * w + g + 8) * kHStride + nb * 8 + 2 * t]) =
          pack_bf16(q2, q3);
    }
    __syncthreads();
    // dW2 rows 16 w .. + 16 (A = H1^T: transposed loads of H1), all columns
    // (B = G2: transposed loads give the col-major fragments, two 8-column
    // blocks per x4 load); k = the chunk's 64 samples.
    {
      const int qm = lane >> 3, r = lane & 7;
#pragma unroll
      for (int kb = 0; kb < 4; kb++) {
        uint32_t a[4];
        // Matrices: (samples kb*16 + 0-7 | 8-15) x (rows 16w + 0-7 | 8-15):
        // q = 0: (s 0-7, i 0-7), 1: (s 0-7, i 8-15), 2: (s 8-15, i 0-7), 3: (s 8-15, i 8-15).
        ldsm_x4_t(a, &S.H1[(kb * 16 + r + (qm >> 1) * 8) * kHStride + 16 * w + (qm & 1) * 8]);
#pragma unroll
        for (int nb = 0; nb < 8; nb += 2) {
          uint32_t b[4];
          // q = 0: (s 0-7, j nb), 1: (s 8-15, j nb), 2: (s 0-7, j nb+1), 3: (s 8-15, j nb+1).
          ldsm_x4_t(b, &S.G2[(kb * 16 + r + (qm & 1) * 8) * kHStride + (nb + (qm >> 1)) * 8]);
          mma_bf16(dW2[nb], a, make_uint2(b[0], b[1]));
          mma_bf16(dW2[nb + 1], a, make_uint2(b[2], b[3]));
        }
      }
      // dW1 rows 16 (w & 1) .. + 16 of the inputs, columns 32 (w >> 1) .. + 32.
      const int i0 = 16 * (w & 1), j0 = 32 * (w >> 1);
#pragma unroll
      for (int kb = 0; kb < 4; kb++) {
        uint32_t a[4];
        ldsm_x4_t(a, &S.X[(kb * 16 + r + (qm >> 1) * 8) * kXStride + i0 + (qm & 1) * 8]);
#pragma unroll
        for (int nb = 0; nb < 4; nb += 2) {
          uint32_t b[4];
          ldsm_x4_t(b, &S.G1[(kb * 16 + r + (qm & 1) * 8) * kHStride + j0 + (nb + (qm >> 1)) * 8]);
          mma_bf16(dW1[nb], a, make_uint2(b[0], b[1]));
          mma_bf16(dW1[nb + 1], a, make_uint2(b[2], b[3]));
        }
      }
    }
    __syncthreads();  // the tiles are rewritten by the next chunk
  }
  // Weight gradients: each warp's slices are its own (no overlap in the block).
#pragma unroll
  for (int nb = 0; nb < 8; nb++) {
    const int i = 16 * w + g, j = nb * 8 + 2 * t;
    atomicAdd(&grads[kW2 + i * kHid + j], dW2[nb][0]);
    atomicAdd(&grads[kW2 + i * kHid + j + 1], dW2[nb][1]);
    atomicAdd(&grads[kW2 + (i + 8) * kHid + j], dW2[nb][2]);
    atomicAdd(&grads[kW2 + (i + 8) * kHid + j + 1], dW2[nb][3]);
  }
#pragma unroll
  for (int nb = 0; nb < 4; nb++) {
    const int i = 16 * (w & 1) + g, j = 32 * (w >> 1) + nb * 8 + 2 * t;
    atomicAdd(&grads[kW1 + i * kHid + j], dW1[nb][0]);
    atomicAdd(&grads[kW1 + i * kHid + j + 1], dW1[nb][1]);
    atomicAdd(&grads[kW1 + (i + 8) * kHid + j], dW1[nb][2]);
    atomicAdd(&grads[kW1 + (i + 8) * kHid + j + 1], dW1[nb][3]);
  }
  // Column sums: reduce over the eight row groups (lanes with the same t).
#pragma unroll
  for (int c = 0; c < 16; c++) {
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
      db1[c] += __shfl_xor_sync(0xffffffffu, db1[c], o);
      db2[c] += __shfl_xor_sync(0xffffffffu, db2[c], o);
      dw3[c] += __shfl_xor_sync(0xffffffffu, dw3[c], o);
    }
  }
  if (g == 0) {
#pragma unroll
    for (int c = 0; c < 16; c++) {
      const int j = (c >> 1) * 8 + 2 * t + (c & 1);
      atomicAdd(&grads[kB1 + j], db1[c]);
      atomicAdd(&grads[kB2 + j], db2[c]);
      atomicAdd(&grads[kW3 + j], dw3[c]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    db3 += __shfl_xor_sync(0xffffffffu, db3, o);
    lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  }
  if (lane == 0) {
    atomicAdd(&grads[kB3], db3);
    atomicAdd(loss, lsum * inv_n);
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

constexpr size_t kTrainSmem = sizeof(MlpWeights) + sizeof(MlpWeightsT) + sizeof(TrainTiles);

}  // namespace

cudaError_t raster_build(const float* vert32, const int* vot, int n_tri, const unsigned* bounds,
                         long long budget, RasterDesc* rdesc, unsigned* zbits, float4* quad,
                         cudaStream_t s) {
  k_raster_setup<<<1, 1, 0, s>>>(bounds, n_tri, budget, quad, rdesc);
  k_raster_fill<<<grid_for(budget, 256), 256, 0, s>>>(zbits, budget);
  if (n_tri > 0)
    k_raster_tris<<<grid_for(n_tri, 128), 128, 0, s>>>(vert32, vot, n_tri, rdesc, zbits);
  k_raster_finish<<<grid_for(budget, 256), 256, 0, s>>>(zbits, quad, rdesc);
  note_launches(n_tri > 0 ? 4 : 3);
  return cudaGetLastError();
}

cudaError_t learn_features(const LearnParams& q, const float* params, cudaStream_t s) {
  const long long total = (long long)q.cell_count * q.n_pred;
  if (total <= 0) return cudaSuccess;
  k_features<<<grid_for(total, kLearnBlock), kLearnBlock, 0, s>>>(q, params);
  note_launches(1);
  return cudaGetLastError();
}

size_t mlp_train_scratch_floats(int n) {
  (void)n;
  return 64;
}

cudaError_t mlp_train_step(float* params, float* adam_m, float* adam_v, const float* X,
                           const float* T, int n, int step, float lr, float* loss,
                           float* grads, float* scratch, cudaStream_t s) {
  (void)scratch;
  if (n <= 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(grads, 0, sizeof(float) * kMlpParams, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  // The kernel's shared memory is above the 48 KB default: raise the limit
  // once per device (the attribute belongs to the device's context).
  static bool attr_set[128] = {};
  if (dev >= 0 && dev < 128 && !attr_set[dev]) {
    e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kTrainSmem);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  // At most two blocks per SM's worth of chunks: each block adds its
  // gradient slices once, so fewer blocks mean fewer atomics.
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long chunks = (n + kTrainChunk - 1) / kTrainChunk;
  const long long blocks = std::min<long long>(chunks, 2LL * (sms > 0 ? sms : 1));
  k_mlp_train<<<(unsigned)blocks, kLearnBlock, kTrainSmem, s>>>(params, X, T, n, grads, loss);
  note_launches(1);
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
  k_mlp_forward<<<grid_for(n, kLearnBlock), kLearnBlock, 0, s>>>(params, X, n, Y);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace hz
