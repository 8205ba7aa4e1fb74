// hz_trace.cu -- per-cell horizon search and SVF, one thread per ICON cell.
//
// Replaces the tbb::parallel_reduce over cells (mo_lradtopo_horayzon.cpp:
// 686-761), terrain_horizon (cpp:490-555) and its Embree occlusion queries
// (cpp:446-460):
//   * the cell frame (sphere normal, north, ray origin) in FP64, cpp:694-722;
//   * the chained bracketing search over L = nhori * refine_factor azimuths
//     with the reference's incremental FP64 Rodrigues rotations (cpp:119-130)
//     and its lattice of elevation steps (2 * 0.25 deg from 0, downward walk
//     bounded by -85 deg), so the tested directions equal the reference's;
//   * each ray as an FP32 any-hit query: conservative slab tests against the
//     BVH2 node boxes and the watertight ray/triangle test of Woop, Benthin &
//     Wald (JCGT 2013) with every operation explicitly rounded, so hit
//     decisions are bit-identical to the CPU oracle's;
//   * clip at 0, sector mean over refine_factor, rad->deg and the SVF sum
//     (cpp:736-754, 333-358) accumulated online per azimuth, in the
//     reference's summation order.
#include "hz_internal.h"

namespace hz {

namespace {

struct Ray {
  float ox, oy, oz;       // origin
  float ix, iy, iz;       // 1 / direction (IEEE)
  float oix, oiy, oiz;    // origin * inverse direction (slab test)
  float pox, poy, poz;    // origin permuted to (kx, ky, kz)
  float Sx, Sy, Sz;       // shear constants
  int kx, ky, kz;
  float tfar;
};

__device__ __forceinline__ float sel3(float x, float y, float z, int k) {
  return k == 0 ? x : (k == 1 ? y : z);
}

__device__ __forceinline__ Ray make_ray(float ox, float oy, float oz, float dx, float dy,
                                        float dz, float tfar) {
  Ray r;
  r.ox = ox; r.oy = oy; r.oz = oz;
  r.ix = __frcp_rn(dx); r.iy = __frcp_rn(dy); r.iz = __frcp_rn(dz);
  r.oix = __fmul_rn(ox, r.ix); r.oiy = __fmul_rn(oy, r.iy); r.oiz = __fmul_rn(oz, r.iz);
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const float dkz = sel3(dx, dy, dz, kz);
  if (dkz < 0.f) { int tmp = kx; kx = ky; ky = tmp; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  r.Sx = __fdiv_rn(sel3(dx, dy, dz, kx), dkz);
  r.Sy = __fdiv_rn(sel3(dx, dy, dz, ky), dkz);
  r.Sz = __frcp_rn(dkz);
  r.pox = sel3(ox, oy, oz, kx);
  r.poy = sel3(ox, oy, oz, ky);
  r.poz = sel3(ox, oy, oz, kz);
  r.tfar = tfar;
  return r;
}

// Woop, Benthin & Wald 2013; hit iff 0 < t <= tfar. Same operation order as
// the oracle (hz_occlusion.h), every operation rounded to nearest.
__device__ __forceinline__ bool tri_hit(const Ray& r, const float4 v0, const float4 v1,
                                        const float4 v2) {
  const float Akx = __fsub_rn(sel3(v0.x, v0.y, v0.z, r.kx), r.pox);
  const float Aky = __fsub_rn(sel3(v0.x, v0.y, v0.z, r.ky), r.poy);
  const float Akz = __fsub_rn(sel3(v0.x, v0.y, v0.z, r.kz), r.poz);
  const float Bkx = __fsub_rn(sel3(v1.x, v1.y, v1.z, r.kx), r.pox);
  const float Bky = __fsub_rn(sel3(v1.x, v1.y, v1.z, r.ky), r.poy);
  const float Bkz = __fsub_rn(sel3(v1.x, v1.y, v1.z, r.kz), r.poz);
  const float Ckx = __fsub_rn(sel3(v2.x, v2.y, v2.z, r.kx), r.pox);
  const float Cky = __fsub_rn(sel3(v2.x, v2.y, v2.z, r.ky), r.poy);
  const float Ckz = __fsub_rn(sel3(v2.x, v2.y, v2.z, r.kz), r.poz);
  const float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
  const float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
  const float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
  const float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
  const float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
  const float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By),
                                    __dmul_rn((double)Cy, (double)Bx)));
    V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy),
                                    __dmul_rn((double)Ay, (double)Cx)));
    W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay),
                                    __dmul_rn((double)By, (double)Ax)));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  const float det = __fadd_rn(__fadd_rn(U, V), W);
  if (det == 0.f) return false;
  const float Az = __fmul_rn(r.Sz, Akz);
  const float Bz = __fmul_rn(r.Sz, Bkz);
  const float Cz = __fmul_rn(r.Sz, Ckz);
  const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
  const float tmax = __fmul_rn(r.tfar, det);
  if (det > 0.f) return T > 0.f && T <= tmax;
  return T < 0.f && T >= tmax;
}

// Conservative slab test: the boxes carry a margin far above the rounding of
// these multiply-adds, so no triangle the watertight test would hit is culled.
__device__ __forceinline__ bool box_hit(const Ray& r, float lx, float hx, float ly, float hy,
                                        float lz, float hz, float& tentry) {
  const float tx0 = __fmaf_rn(lx, r.ix, -r.oix), tx1 = __fmaf_rn(hx, r.ix, -r.oix);
  const float ty0 = __fmaf_rn(ly, r.iy, -r.oiy), ty1 = __fmaf_rn(hy, r.iy, -r.oiy);
  const float tz0 = __fmaf_rn(lz, r.iz, -r.oiz), tz1 = __fmaf_rn(hz, r.iz, -r.oiz);
  const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.f));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  tf = fminf(__fmul_rn(tf, 1.00000072f), r.tfar);
  tentry = tn;
  return tn <= tf;
}

template <bool kCount>
__device__ bool occluded(const Ray& r, const Node* __restrict__ nodes,
                         const Tri* __restrict__ tris, int root,
                         unsigned long long& nvis, unsigned long long& ntest, int* err) {
  if (root == kEmptyRef) return false;
  int stack[kStackDepth];
  int sp = 0;
  int ref = root;
  for (;;) {
    if (ref < 0) {
      const int s = leaf_start(ref), c = leaf_count(ref);
      for (int k = s; k < s + c; k++) {
        if (kCount) ntest++;
        const float4 v0 = __ldg(&tris[k].v0);
        const float4 v1 = __ldg(&tris[k].v1);
        const float4 v2 = __ldg(&tris[k].v2);
        if (tri_hit(r, v0, v1, v2)) return true;
      }
    } else {
      if (kCount) nvis++;
      const Node* nd = nodes + ref;
      const float4 a = __ldg(&nd->a);
      const float4 b = __ldg(&nd->b);
      const float4 c = __ldg(&nd->c);
      const float4 d = __ldg(&nd->d);
      const int c0 = __float_as_int(d.x), c1 = __float_as_int(d.y);
      float t0, t1;
      const bool h0 = box_hit(r, a.x, a.y, a.z, a.w, c.x, c.y, t0);
      const bool h1 = c1 != kEmptyRef && box_hit(r, b.x, b.y, b.z, b.w, c.z, c.w, t1);
      if (h0 && h1) {
        if (sp >= kStackDepth) {
          atomicOr(err, kErrStack);
          return true;
        }
        const bool near0 = t0 <= t1;
        stack[sp++] = near0 ? c1 : c0;
        ref = near0 ? c0 : c1;
        continue;
      }
      if (h0) { ref = c0; continue; }
      if (h1) { ref = c1; continue; }
    }
    if (sp == 0) return false;
    ref = stack[--sp];
  }
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

struct V3 {
  double x, y, z;
};

__device__ __forceinline__ double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ void unit3(V3& a) {
  const double m = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  a.x /= m;
  a.y /= m;
  a.z /= m;
}
// mo_lradtopo_horayzon.cpp:119-130
__device__ __forceinline__ V3 rotate3(V3 v, V3 k, double s, double c) {
  const double term = dot3(k, v) * (1.0 - c);
  V3 r;
  r.x = v.x * c + (k.y * v.z - k.z * v.y) * s + k.x * term;
  r.y = v.y * c + (k.z * v.x - k.x * v.z) * s + k.y * term;
  r.z = v.z * c + (k.x * v.y - k.y * v.x) * s + k.z * term;
  return r;
}

template <bool kCount>
__global__ void __launch_bounds__(128) k_trace_exact(TraceParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long rays = 0, nvis = 0, ntest = 0;
  if (i < p.ncell) {
    const V3 q{p.cell_enu[3LL * i], p.cell_enu[3LL * i + 1], p.cell_enu[3LL * i + 2]};
    V3 normal{q.x - p.centre.x, q.y - p.centre.y, q.z - p.centre.z};
    unit3(normal);
    const V3 v_n{p.pole.x - q.x, p.pole.y - q.y, p.pole.z - q.z};
    const double dp = dot3(v_n, normal);
    V3 north{v_n.x - dp * normal.x, v_n.y - dp * normal.y, v_n.z - dp * normal.z};
    unit3(north);
    const float ox = (float)(q.x + normal.x * p.ray_org_elev);
    const float oy = (float)(q.y + normal.y * p.ray_org_elev);
    const float oz = (float)(q.z + normal.z * p.ray_org_elev);

    const double ha = p.hori_acc;
    V3 dir = rotate3(north, normal, p.shift_sin, p.shift_cos);
    double elev = 0.0, sector = 0.0, svf = 0.0;
    for (int a = 0; a < p.L; a++) {
      V3 axis = cross3(dir, normal);
      unit3(axis);
      bool hit = occluded<kCount>(make_ray(ox, oy, oz, (float)dir.x, (float)dir.y,
                                           (float)dir.z, p.tfar),
                                  p.nodes, p.tris, p.root, nvis, ntest, p.err);
      rays++;
      double h;
      if (hit) {
        // A ray origin enclosed by the mesh would make the reference's upward
        // walk circle forever; stop after one full turn (720 steps).
        int up = 0;
        while (hit && up++ < kMaxUpSteps) {
          elev += (2.0 * ha);
          dir = rotate3(dir, axis, p.elev_sin_2ha, p.elev_cos_2ha);
          hit = occluded<kCount>(make_ray(ox, oy, oz, (float)dir.x, (float)dir.y,
                                          (float)dir.z, p.tfar),
                                 p.nodes, p.tris, p.root, nvis, ntest, p.err);
          rays++;
        }
        h = elev - ha;
      } else {
        while ((!hit) && (elev > p.elev_floor)) {
          elev -= (2.0 * ha);
          dir = rotate3(dir, axis, -p.elev_sin_2ha, p.elev_cos_2ha);
          hit = occluded<kCount>(make_ray(ox, oy, oz, (float)dir.x, (float)dir.y,
                                          (float)dir.z, p.tfar),
                                 p.nodes, p.tris, p.root, nvis, ntest, p.err);
          rays++;
        }
        h = elev + ha;
      }
      dir = rotate3(dir, normal, -p.azim_sin, p.azim_cos);
      if (h < 0.0) h = 0.0;
      sector += h;
      if ((a + 1) % p.refine == 0) {
        const int j = a / p.refine;
        p.horizon[(long long)j * p.ncell + i] = ((sector / kPi) * 180.0) / (double)p.refine;
        sector = 0.0;
      }
      const double s = sin(h);
      if (p.svf_type == 0) svf += (1.0 - s);
      else if (p.svf_type == 1) svf += (1.0 - (s * s));
      else svf += (1.0 - (s * s * s));
    }
    p.skyview[i] = svf / (double)p.L;
  }
  // Warp-aggregated counters.
  rays = warp_sum_u64(rays);
  if (kCount) {
    nvis = warp_sum_u64(nvis);
    ntest = warp_sum_u64(ntest);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&p.counters[0], rays);
    if (kCount) {
      atomicAdd(&p.counters[1], nvis);
      atomicAdd(&p.counters[2], ntest);
    }
  }
}

}  // namespace

cudaError_t trace_exact(const TraceParams& p, bool count_work, cudaStream_t s) {
  if (p.ncell <= 0) return cudaSuccess;
  if (count_work) k_trace_exact<true><<<grid_for(p.ncell, 128), 128, 0, s>>>(p);
  else k_trace_exact<false><<<grid_for(p.ncell, 128), 128, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace hz
