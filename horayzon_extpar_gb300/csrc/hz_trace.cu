// hz_trace.cu -- the horizon search and SVF over all cells, and the ray query.
//
// Replaces the tbb::parallel_reduce over cells (mo_lradtopo_horayzon.cpp:
// 686-761), terrain_horizon (cpp:490-555) and its Embree occlusion queries
// (cpp:446-460). Kernels: k_trace_warp, the persistent search (the default;
// overview further down), with its pre-pass k_cell_frames and epilogue
// k_finish_outputs; k_trace_exact, one thread per cell running the
// reference's loops as written; k_rays, the any-hit query on arbitrary rays;
// and the cell ordering and lattice tables. What they share:
//   * the cell frame (sphere normal, north, ray origin) in FP64, cpp:694-722;
//   * the chained bracketing search over L = nhori * refine_factor azimuths
//     on the reference's lattice of elevation steps (2 * 0.25 deg from 0,
//     downward walk bounded by -85 deg): k_trace_exact with the reference's
//     incremental FP64 Rodrigues rotations (cpp:119-130), the persistent
//     search with each direction in closed form from tabulated lattice
//     angles; both cast the same FP32 rays;
//   * each ray as an FP32 any-hit query: conservative slab tests against the
//     node boxes (binary or 4-wide tree) and the watertight ray/triangle test of Woop, Benthin &
//     Wald (JCGT 2013) with every operation explicitly rounded, so hit
//     decisions are bit-identical to the CPU oracle's;
//   * clip at 0, sector mean over refine_factor, rad->deg and the SVF sum
//     (cpp:736-754, 333-358), in the reference's summation order.
#include <algorithm>

#include "hz_internal.h"

namespace hz {

namespace {

struct Ray {
  float ox, oy, oz;       // origin
  float ix, iy, iz;       // 1 / direction (IEEE)
  float oix, oiy, oiz;    // origin * inverse direction (slab test)
  float pox, poy, poz;    // origin permuted to (kx, ky, kz)
  float plx, ply, plz;    // precise mode: FP32 residual of the origin, permuted
  float Sx, Sy, Sz;       // shear constants
  // Axis order of the shear (kx, ky, kz) and the signs of the inverse
  // direction (n = 1 where negative: near plane = hi), packed in one
  // register: kx | ky << 2 | kz << 4 | nx << 6 | ny << 7 | nz << 8. The
  // persistent search then holds its state in 64 registers without spills.
  unsigned ax;
  __device__ int kx() const { return ax & 3u; }
  __device__ int ky() const { return (ax >> 2) & 3u; }
  __device__ int kz() const { return (ax >> 4) & 3u; }
  __device__ int nx() const { return (ax >> 6) & 1u; }
  __device__ int ny() const { return (ax >> 7) & 1u; }
  __device__ int nz() const { return (ax >> 8) & 1u; }
  float tfar;
};

__device__ __forceinline__ float sel3(float x, float y, float z, int k) {
  return k == 0 ? x : (k == 1 ? y : z);
}

__device__ __forceinline__ Ray make_ray(float ox, float oy, float oz, float dx, float dy,
                                        float dz, float tfar, float lx = 0.f, float ly = 0.f,
                                        float lz = 0.f) {
  Ray r;
  r.ox = ox; r.oy = oy; r.oz = oz;
  r.ix = __frcp_rn(dx); r.iy = __frcp_rn(dy); r.iz = __frcp_rn(dz);
  r.oix = __fmul_rn(ox, r.ix); r.oiy = __fmul_rn(oy, r.iy); r.oiz = __fmul_rn(oz, r.iz);
  const unsigned sx = signbit(r.ix) ? 1u : 0u, sy = signbit(r.iy) ? 1u : 0u,
                 sz = signbit(r.iz) ? 1u : 0u;
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const float dkz = sel3(dx, dy, dz, kz);
  if (dkz < 0.f) { int tmp = kx; kx = ky; ky = tmp; }
  r.ax = (unsigned)kx | ((unsigned)ky << 2) | ((unsigned)kz << 4) | (sx << 6) | (sy << 7) |
         (sz << 8);
  r.Sx = __fdiv_rn(sel3(dx, dy, dz, kx), dkz);
  r.Sy = __fdiv_rn(sel3(dx, dy, dz, ky), dkz);
  r.Sz = __frcp_rn(dkz);
  r.pox = sel3(ox, oy, oz, kx);
  r.poy = sel3(ox, oy, oz, ky);
  r.poz = sel3(ox, oy, oz, kz);
  r.plx = sel3(lx, ly, lz, kx);
  r.ply = sel3(lx, ly, lz, ky);
  r.plz = sel3(lx, ly, lz, kz);
  r.tfar = tfar;
  return r;
}

// FP64 re-evaluation of the three edge functions when one of them is zero
// (rare). Kept out of line so that the common path carries no FP64 work.
__device__ __noinline__ void edge_functions_fp64(float Ax, float Ay, float Bx, float By,
                                                 float Cx, float Cy, float* U, float* V,
                                                 float* W) {
  *U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By),
                                   __dmul_rn((double)Cy, (double)Bx)));
  *V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy),
                                   __dmul_rn((double)Ay, (double)Cx)));
  *W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay),
                                   __dmul_rn((double)By, (double)Ax)));
}

// Woop, Benthin & Wald 2013 on origin-relative vertices A, B, C given in the
// ray's (kx, ky, kz) order; hit iff 0 < t <= tfar. Same operation order as
// the oracle (hz_occlusion.h), every operation rounded to nearest.
__device__ __forceinline__ bool tri_hit_rel(const Ray& r, float Akx, float Aky, float Akz,
                                            float Bkx, float Bky, float Bkz, float Ckx,
                                            float Cky, float Ckz) {
  const float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
  const float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
  const float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
  const float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
  const float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
  const float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.f || V == 0.f || W == 0.f) edge_functions_fp64(Ax, Ay, Bx, By, Cx, Cy, &U, &V, &W);
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

// Reference arithmetic: FP32 vertices minus the FP32 origin in the domain's
// global ENU frame (mo_lradtopo_horayzon.cpp:403-410, 715-720). X, Y, Z are
// the triangle's (kx, ky, kz) axes: (v0, v1, v2) components of each.
__device__ __forceinline__ bool tri_hit(const Ray& r, const float4 X, const float4 Y,
                                        const float4 Z) {
  return tri_hit_rel(r, __fsub_rn(X.x, r.pox), __fsub_rn(Y.x, r.poy), __fsub_rn(Z.x, r.poz),
                     __fsub_rn(X.y, r.pox), __fsub_rn(Y.y, r.poy), __fsub_rn(Z.y, r.poz),
                     __fsub_rn(X.z, r.pox), __fsub_rn(Y.z, r.poy), __fsub_rn(Z.z, r.poz));
}

// Precise arithmetic: vertices and origin as FP32 hi + lo pairs (~48-bit
// FP64 values); the origin-relative vector (hi - o_hi) + (lo - o_lo) is
// accurate to FP32 relative to its own length, i.e. centimetres become
// micrometres for the triangles next to the cell. LX, LY, LZ: the residuals.
__device__ __forceinline__ float rel(float vh, float vl, float oh, float ol) {
  return __fadd_rn(__fsub_rn(vh, oh), __fsub_rn(vl, ol));
}
__device__ __forceinline__ bool tri_hit_hl(const Ray& r, const float4 X, const float4 Y,
                                           const float4 Z, const float4 LX, const float4 LY,
                                           const float4 LZ) {
  return tri_hit_rel(r, rel(X.x, LX.x, r.pox, r.plx), rel(Y.x, LY.x, r.poy, r.ply),
                     rel(Z.x, LZ.x, r.poz, r.plz), rel(X.y, LX.y, r.pox, r.plx),
                     rel(Y.y, LY.y, r.poy, r.ply), rel(Z.y, LZ.y, r.poz, r.plz),
                     rel(X.z, LX.z, r.pox, r.plx), rel(Y.z, LY.z, r.poy, r.ply),
                     rel(Z.z, LZ.z, r.poz, r.plz));
}

// Triangle k's axes in the ray's (kx, ky, kz) order (Tri: one float4 per
// axis), and the same for the precise residuals.
__device__ __forceinline__ void load_tri(const Tri* __restrict__ tris, const Ray& r, int k,
                                         float4& X, float4& Y, float4& Z) {
  const float4* t = reinterpret_cast<const float4*>(tris + k);
  X = __ldg(t + r.kx());
  Y = __ldg(t + r.ky());
  Z = __ldg(t + r.kz());
}

// Conservative slab test: the boxes carry a margin far above the rounding of
// these multiply-adds, so no triangle the watertight test would hit is culled.
// Each axis' near and far plane is chosen by the sign of the inverse
// direction (near = lo where it is positive). For a finite inverse direction
// the entry / exit distances equal the min / max of the two planes'; for an
// infinite one (a zero direction component) they are NaN or infinite, and the
// NaN-skipping fminf / fmaxf then leave the axis unconstrained unless the
// parallel ray lies outside the slab.
__device__ __forceinline__ bool box_hit_nf(const Ray& r, float nx, float fx, float ny, float fy,
                                           float nz, float fz, float& tentry) {
  const float tn = fmaxf(fmaxf(__fmaf_rn(nx, r.ix, -r.oix), __fmaf_rn(ny, r.iy, -r.oiy)),
                         fmaxf(__fmaf_rn(nz, r.iz, -r.oiz), 0.f));
  float tf = fminf(fminf(__fmaf_rn(fx, r.ix, -r.oix), __fmaf_rn(fy, r.iy, -r.oiy)),
                   __fmaf_rn(fz, r.iz, -r.oiz));
  tf = fminf(__fmul_rn(tf, 1.00000072f), r.tfar);
  tentry = tn;
  return tn <= tf;
}

// The same test on a box given as (lo, hi) per axis.
__device__ __forceinline__ bool box_hit(const Ray& r, float lx, float hx, float ly, float hy,
                                        float lz, float hz, float& tentry) {
  return box_hit_nf(r, r.nx() ? hx : lx, r.nx() ? lx : hx, r.ny() ? hy : ly, r.ny() ? ly : hy,
                    r.nz() ? hz : lz, r.nz() ? lz : hz, tentry);
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
        float4 X, Y, Z;
        load_tri(tris, r, k, X, Y, Z);
        if (tri_hit(r, X, Y, Z)) return true;
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
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = p.cell_begin + k;
  unsigned long long rays = 0, nvis = 0, ntest = 0;
  if (k < p.cell_count) {
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

// ---------------------------------------------------------------------------
// Persistent search (the TBB loop over cells, cpp:683-761, with its Embree
// queries). Same search and the same rays as k_trace_exact, restructured for
// the SIMT machine:
//   * persistent blocks take cells from a global counter in the order given
//     by `order` (Hilbert-curve order of the cells); each lane owns one cell at a
//     time and runs its bracketing search as a state machine;
//   * every loop iteration is executed by all 32 lanes of a warp (the loop
//     ends when no lane has work left), so the ballots see the whole warp;
//   * a lane whose ray has finished advances its search (next elevation, next
//     azimuth or next cell) only once at least `advance_min` lanes of the warp
//     are waiting, so the FP64 search code runs for many lanes at once;
//   * the traversal alternates node passes and triangle passes. A node pass
//     visits one BVH node for every lane whose next target is a node; a leaf
//     reached this way is postponed (one per lane) and the lane continues
//     from its stack. A triangle pass runs when at least `leaf_min` lanes hold
//     a postponed leaf, or when no lane has a node left to visit, and tests
//     ONE triangle per such lane. Occlusion is an any-hit query, so the order
//     in which leaves are tested changes no hit decision;
//   * the search state (FP64 frame and sums, lattice index, azimuth, cell,
//     FP32 origin) lives in shared memory; registers hold the ray and its
//     traversal.
// kWide: the 4-wide BVH (Node4); otherwise the binary BVH.
// ---------------------------------------------------------------------------
constexpr int kFlatBlock = 128;
#ifndef HZ_WARP_MIN_BLOCKS
#define HZ_WARP_MIN_BLOCKS 8  // resident blocks per SM the register budget targets
#endif

#ifndef HZ_NODE_STEPS
#define HZ_NODE_STEPS 3  // node visits per lane in one node pass
#endif
#ifndef HZ_TRI_STEPS
#define HZ_TRI_STEPS 2  // triangle tests per lane in one triangle pass
#endif
#ifndef HZ_NODE4_ORDER
#define HZ_NODE4_ORDER 1  // 0: hit children sorted by entry distance; 1: nearest first only
#endif

enum : int { kPhaseStart = 0, kPhaseFirst = 1, kPhaseUp = 2, kPhaseDown = 3, kPhaseDeep = 4 };

// Search-state slot (k_trace_warp) of the triangle that hid the lane's last
// ray, the occluder cache.
constexpr int kOccluder = 10;

// Bracket sentinel of the walk below the clip: no hit found yet.
constexpr int kNoHit = 0x7fff;

// Candidates of the downward step walk from e0 down to the floor (cpp:538):
// the k of the first e_k = e0 - 2 hori_acc - ... - 2 hori_acc <= elev_floor,
// accumulated as the reference does.
__device__ __forceinline__ int deep_walk_count(double e0, const DomainDesc& D) {
  int K = 0;
  double e = e0;
  do {
    e -= D.two_ha;
    K++;
  } while (e > D.elev_floor);
  return K;
}

#ifndef HZ_CHECKED
#define HZ_CHECKED 0  // 1: the search checks its indices and records violations (kErrBounds)
#endif
// What a checked build checks: a node reference against the tree's nodes, a
// leaf's triangle range against its triangles, an output row / cell.
enum : int { kCheckNode = 1, kCheckLeaf = 2, kCheckOutput = 3 };

// In checked builds: records the first failed check (code, index) in err[1],
// err[2] and raises kErrBounds; the caller then skips the access. Without
// HZ_CHECKED every check passes and compiles away.
__device__ __forceinline__ bool check_ok(bool ok, int code, long long index, int* err) {
#if HZ_CHECKED
  if (!ok) {
    if (atomicCAS(err + 1, 0, code) == 0) err[2] = (int)index;
    atomicOr(err, kErrBounds);
  }
  return ok;
#else
  (void)code;
  (void)index;
  (void)err;
  return true;
#endif
}

#ifndef HZ_STACK_TOP
#define HZ_STACK_TOP 1  // 1: the top stack entries live in registers (StackTop)
#endif
// Traversal stack: entries in `stack` (local memory) below a top entry held
// in a register (kEmptyRef when the stack is empty), so that a pop returns at
// once and the reload of the next top overlaps with the node fetch.
// The top entries of a traversal stack held in registers: `a` is the top,
// `b` the entry below it (kRegs == 2 only; empty while `a` is); the rest
// lives in local memory, stack[0, sp). The binary tree pushes and pops once
// per visit and gains from two register entries; the 4-wide tree, which
// pushes up to three children at once, from one (HZ_STACK_TOP 0: none).
struct StackTop {
  int a = kEmptyRef;
  int b = kEmptyRef;
  __device__ void clear() {
    a = kEmptyRef;
    b = kEmptyRef;
  }
};
template <int kRegs>
__device__ __forceinline__ void stk_push(int* stack, int& sp, StackTop& top, int x) {
  if (HZ_STACK_TOP && kRegs == 2) {
    if (top.b != kEmptyRef) stack[sp++] = top.b;
    top.b = top.a;
    top.a = x;
  } else if (HZ_STACK_TOP) {
    if (top.a != kEmptyRef) stack[sp++] = top.a;
    top.a = x;
  } else {
    stack[sp++] = x;
  }
}
template <int kRegs>
__device__ __forceinline__ int stk_pop(int* stack, int& sp, StackTop& top) {
  if (HZ_STACK_TOP && kRegs == 2) {
    const int r = top.a;
    if (top.b != kEmptyRef) {
      top.a = top.b;
      top.b = kEmptyRef;
    } else {
      top.a = sp > 0 ? stack[--sp] : kEmptyRef;
    }
    return r;
  }
  if (HZ_STACK_TOP) {
    const int r = top.a;
    top.a = sp > 0 ? stack[--sp] : kEmptyRef;
    return r;
  }
  return sp > 0 ? stack[--sp] : kEmptyRef;
}
constexpr int kRegsBinary = 2, kRegsWide = 1;

// Visits internal node `ref`: descends into the nearer hit child (pushing the
// other), or pops. Returns false on stack overflow.
__device__ __forceinline__ bool visit_node(const Node* __restrict__ nodes, const Ray& r,
                                           int& ref, int* stack, int& sp, StackTop& top) {
  const Node* nd = nodes + ref;
  const float4 na = __ldg(&nd->a);
  const float4 nb = __ldg(&nd->b);
  const float4 nc = __ldg(&nd->c);
  const float4 ndd = __ldg(&nd->d);
  const int c0 = __float_as_int(ndd.x), c1 = __float_as_int(ndd.y);
  float t0, t1;
  const bool h0 = box_hit(r, na.x, na.y, na.z, na.w, nc.x, nc.y, t0);
  const bool h1 = c1 != kEmptyRef && box_hit(r, nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, t1);
  if (h0 && h1) {
    if (sp >= kStackDepth - 1) return false;
    const bool near0 = t0 <= t1;
    stk_push<kRegsBinary>(stack, sp, top, near0 ? c1 : c0);
    ref = near0 ? c0 : c1;
  } else if (h0) {
    ref = c0;
  } else if (h1) {
    ref = c1;
  } else {
    ref = stk_pop<kRegsBinary>(stack, sp, top);
  }
  return true;
}

// Visits BVH4 node `ref`: continues with the nearest hit child and pushes the
// other hit children, farthest first; pops when no child is hit. Returns false
// on stack overflow.
__device__ __forceinline__ bool visit_node4(const Node4* __restrict__ nodes4, const Ray& r,
                                            int& ref, int* stack, int& sp, StackTop& top) {
  // Planes in node order lo.x, hi.x, lo.y, hi.y, lo.z, hi.z: the near plane
  // of an axis is lo + n (n = 1 for a negative inverse direction).
  const float4* pl = reinterpret_cast<const float4*>(nodes4 + ref);
  const float4 nx = __ldg(pl + r.nx()), fx = __ldg(pl + 1 - r.nx());
  const float4 ny = __ldg(pl + 2 + r.ny()), fy = __ldg(pl + 3 - r.ny());
  const float4 nz = __ldg(pl + 4 + r.nz()), fz = __ldg(pl + 5 - r.nz());
  const int4 ch = __ldg(&nodes4[ref].child);
  float t0, t1, t2, t3;
  int r0 = ch.x, r1 = ch.y, r2 = ch.z, r3 = ch.w;
  if (!(r0 != kEmptyRef && box_hit_nf(r, nx.x, fx.x, ny.x, fy.x, nz.x, fz.x, t0))) t0 = INFINITY;
  if (!(r1 != kEmptyRef && box_hit_nf(r, nx.y, fx.y, ny.y, fy.y, nz.y, fz.y, t1))) t1 = INFINITY;
  if (!(r2 != kEmptyRef && box_hit_nf(r, nx.z, fx.z, ny.z, fy.z, nz.z, fz.z, t2))) t2 = INFINITY;
  if (!(r3 != kEmptyRef && box_hit_nf(r, nx.w, fx.w, ny.w, fy.w, nz.w, fz.w, t3))) t3 = INFINITY;
  auto cx = [](float& ta, int& ra, float& tb, int& rb) {
    const bool sw = tb < ta;
    const float t = sw ? tb : ta;
    const int q = sw ? rb : ra;
    tb = sw ? ta : tb;
    rb = sw ? ra : rb;
    ta = t;
    ra = q;
  };
#if HZ_NODE4_ORDER == 1
  // Nearest hit child first; the others keep their slot order.
  cx(t0, r0, t1, r1);
  cx(t0, r0, t2, r2);
  cx(t0, r0, t3, r3);
#else
  // Sorting network on (t, ref): (0,1) (2,3) (0,2) (1,3) (1,2).
  cx(t0, r0, t1, r1);
  cx(t2, r2, t3, r3);
  cx(t0, r0, t2, r2);
  cx(t1, r1, t3, r3);
  cx(t1, r1, t2, r2);
#endif
  if (t0 == INFINITY) {
    ref = stk_pop<kRegsWide>(stack, sp, top);
    return true;
  }
  const int extra = (t1 != INFINITY) + (t2 != INFINITY) + (t3 != INFINITY);
  if (sp + extra >= kStackDepth4) return false;
  if (t3 != INFINITY) stk_push<kRegsWide>(stack, sp, top, r3);
  if (t2 != INFINITY) stk_push<kRegsWide>(stack, sp, top, r2);
  if (t1 != INFINITY) stk_push<kRegsWide>(stack, sp, top, r1);
  ref = r0;
  return true;
}

// One ray/triangle test of triangle k (kPrecise: hi + lo vertices).
template <bool kPrecise>
__device__ __forceinline__ bool test_tri(const Tri* __restrict__ tris,
                                         const float4* __restrict__ tri_lo, const Ray& r, int k) {
  float4 X, Y, Z;
  load_tri(tris, r, k, X, Y, Z);
  if (kPrecise) {
    const float4* l = tri_lo + 3LL * k;
    return tri_hit_hl(r, X, Y, Z, __ldg(l + r.kx()), __ldg(l + r.ky()), __ldg(l + r.kz()));
  }
  return tri_hit(r, X, Y, Z);
}

// One azimuth's SVF term for sin(h) = s (cpp:333-358).
__device__ __forceinline__ double svf_term(double s, int svf_type) {
  if (svf_type == 0) return 1.0 - s;
  if (svf_type == 1) return 1.0 - (s * s);
  return 1.0 - (s * s * s);
}

// SVF term of a clipped horizon h ~ j * hori_acc: 1 for h = 0 (sin 0 = 0),
// the tabulated term of the lattice value, or computed off the table.
__device__ __forceinline__ double lattice_svf_term(const DomainDesc& D, double h, int j) {
  if (!(h > 0.0)) return 1.0;
  if (j > 0 && j < kSvfTable) return __ldg(&D.svf_lattice[j]);
  return svf_term(sin(h), D.svf_type);
}

// RN(v / pi) without a division, by Markstein's correction for a divisor
// known in advance (P. Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990): y =
// RN(1 / pi) lies within 0.131 ulp of 1 / pi, so for a normal v >= 0
// q0 = RN(v * y) is within 0.206 + 0.5 ulp of v / pi, a faithful quotient;
// its remainder r = v - q0 * pi is then exact in one FMA, and RN(q0 + r * y)
// is the correctly rounded quotient, the value of v / pi. The search's sums
// are 0 or at least 0.25 deg, far from the subnormal range.
__device__ __forceinline__ double div_pi_rn(double v) {
  const double q0 = __dmul_rn(v, kInvPi);
  const double r = __fma_rn(-q0, kPi, v);
  return __fma_rn(r, kInvPi, q0);
}

// The epilogue's SVF term of a clipped horizon v (0, or at least 0.25 deg on
// the lattice v ~ j * hori_acc, j < kSvfTable in practice), with integer and
// FP32 operations where the search's form uses FP64 ones: v > 0 from the
// exponent bits, and j from an FP32 copy of v truncated to its top 20
// mantissa bits (relative error < 2^-20, so |f / hori_acc - j| < 0.01).
__device__ __forceinline__ double finish_svf_term(const DomainDesc& D, double v, float inv_ha) {
  const int hi = __double2hiint(v);
  const int e = (hi >> 20) & 0x7ff;
  if (hi < 0 || e == 0) return 1.0;  // v == 0 (the clip leaves no negatives)
  const int fe = e - 1023 + 127;
  if (fe <= 0 || fe >= 255) return svf_term(sin(v), D.svf_type);
  const float f = __int_as_float((fe << 23) | ((hi & 0xfffff) << 3));
  const int j = __float2int_rn(f * inv_ha);
  if (j > 0 && j < kSvfTable) return __ldg(&D.svf_lattice[j]);
  return svf_term(sin(v), D.svf_type);
}

// Domain of work id g (doms sorted by cell_offset).
__device__ __forceinline__ int domain_of(const DomainDesc* __restrict__ doms, int ndom,
                                         long long g) {
  int lo = 0, hi = ndom - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (doms[mid].cell_offset <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// A warm-start lattice index within [-85, +90] deg.
__device__ __forceinline__ int clamp_start(int m) {
  return m < kMlpStartMin ? kMlpStartMin : (m > kMlpStartMax ? kMlpStartMax : m);
}

// Domain of search item k (doms sorted by item_begin).
__device__ __forceinline__ int domain_of_item(const DomainDesc* __restrict__ doms, int ndom,
                                              long long k) {
  int lo = 0, hi = ndom - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (doms[mid].item_begin <= k) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One step of a search item's bracketing search (mo_lradtopo_horayzon.cpp:
// 490-555, 694-754) on the state `st` (FP64: 0-2 sphere normal U, 3-5
// horizontal direction of the current azimuth, 6 elevation accumulator, 7
// sector sum, 8 SVF sum; integers: domain, cell, azimuth, phase, upward
// steps, lattice index m, work position, end azimuth of the item; FP32 ray
// origin hi and lo). An item is one cell's run over one group of
// consecutive azimuths: all L azimuths (the reference's chain) or, with the
// learned start split into G groups, L / G of them starting at the MLP's
// proposal. Items of a domain are numbered group-major (item = q * cells +
// p), so the 32 items a warp takes are neighbouring cells in the same group.
// North and east are read from the cell frame table at each new azimuth.
// Given the result of the item's last ray (or, in phase kPhaseStart, the
// item number k_new of a new item), it continues the bracket, or closes the
// azimuth (clip, sector mean, SVF) and starts the next one, or finishes the
// item. Returns 1 with the next ray's direction, 0 when the item has
// finished (the state is back in kPhaseStart and needs a new item), -1 when
// k_new is past the last item.
template <bool kPrecise, class S>
__device__ __forceinline__ int search_step(const S& st, const DomainDesc* __restrict__ doms,
                                           int ndom, const int* __restrict__ order, int total,
                                           int k_new, bool last_hit, float3& dir, int& dom_out,
                                           int* err) {
#define SV(k_) st.d(k_)
#define SO(k_) st.f(k_)
  int dom = st.i(0), cell = st.i(1), a = st.i(2), phase = st.i(3), up = st.i(4), m = st.i(5);
  int p = st.i(6);
  bool alive = true;
  bool emit = false;
  while (!emit) {
    if (phase == kPhaseStart) {
      const int k = k_new;
      if (k >= total) {
        alive = false;
        break;
      }
      dom = domain_of_item(doms, ndom, k);
      const DomainDesc& D = doms[dom];
      const long long local = k - D.item_begin;
      const int grp = (int)(local / D.ncell_traced);
      // Cell frame (mo_lradtopo_horayzon.cpp:694-720) from k_cell_frames.
      p = (int)(local - (long long)grp * D.ncell_traced);
      cell = (int)(order[D.k_begin + p] - D.cell_offset);
      const long long nc = D.ncell;
      const double* fr = D.cell_frame + p;
      SV(0) = fr[0]; SV(1) = fr[nc]; SV(2) = fr[2 * nc];
      const float* org = D.cell_origin + p;
      SO(0) = org[0];
      SO(1) = org[nc];
      SO(2) = org[2 * nc];
      if (kPrecise) {
        SO(3) = org[3 * nc];
        SO(4) = org[4 * nc];
        SO(5) = org[5 * nc];
      }
      SV(7) = 0.0; SV(8) = 0.0;
      const int span = D.L / D.groups;
      a = grp * span;
      st.i(7) = a + span;  // end azimuth of the item
      // The first elevation: the reference's 0 (cpp:511), or the learned
      // proposal of the item's first azimuth.
      m = D.start_m ? clamp_start(D.start_m[(long long)a * D.ncell + cell]) : 0;
      SV(6) = (double)m * D.two_ha;
      phase = kPhaseFirst;
    } else {
      // Result of the last ray: continue the bracket or close the azimuth.
      const DomainDesc& D = doms[dom];
      const double ha = D.hori_acc;
      double elev = SV(6);
      if (phase == kPhaseFirst) {
        phase = last_hit ? kPhaseUp : kPhaseDown;
        up = 0;
      }
      bool hit = last_hit;
      if (phase == kPhaseDeep) {
        // Result of probe k = m0 - m of the search for the highest hit below
        // the clip (DomainDesc::deep_walk): bracket (lo missed, hi hit; hi =
        // kNoHit before the first hit), m0 and e0 (SV(6)) the last miss of
        // the step walk, `up` the number K of candidates down to the floor
        // (negative while it is only the estimate -K').
        const int m0 = st.i(9), cur = m0 - m;
        int lo = st.i(8) & 0xffff, hi = st.i(8) >> 16;
        if (last_hit) hi = cur;
        else lo = cur;
        const bool no_hit = hi == kNoHit;
        if (no_hit && up < 0 && 2 * lo >= -up - 2) up = deep_walk_count(elev, D);
        const int K = up < 0 ? -up : up;
        const int next = no_hit ? (lo >= K ? 0 : min(max(1, 2 * lo), K))  // double
                                : (hi - lo > 1 ? (lo + hi) >> 1 : 0);     // bisect
        if (next > 0) {
          m = m0 - next;
          st.i(8) = lo | (hi << 16);
          emit = true;
          break;
        }
        // The walk's stop: the reference's elevation after ks steps of
        // cpp:538, accumulated as it does.
        const int ks = no_hit ? K : hi;
        hit = !no_hit;
        for (int q = 0; q < ks; q++) elev -= D.two_ha;
        m = m0 - ks;
        SV(6) = elev;
        phase = kPhaseDown;
      }
      const bool step_up = phase == kPhaseUp && hit && up < kMaxUpSteps;
      const bool step_dn = phase == kPhaseDown && !hit && elev > D.elev_floor;
      if (step_dn && D.deep_walk && elev <= ha) {
        // Every further candidate e_k = e0 - k 2 hori_acc gives a horizon
        // e_k + hori_acc <= 0, clipped to 0 (cpp:737-741): the walk only
        // decides the elevation carried into the next azimuth, its first
        // hit. Doubling steps then bisection find it in O(log K) rays; where
        // hits are contiguous below that stop (visibility monotone in
        // elevation) it is the step walk's stop.
        // K is estimated here (within one of the count); the exact count,
        // a serial FP64 accumulation, runs only once the doubling comes
        // within two candidates of the floor.
        up = -(int)ceilf((float)(elev - D.elev_floor) / (float)D.two_ha);
        st.i(9) = m;
        st.i(8) = kNoHit << 16;
        phase = kPhaseDeep;
        m--;  // probe k = 1
        emit = true;
        break;
      }
      if (step_up || step_dn) {
        if (step_up) {
          up++;
          m++;
          elev += D.two_ha;
        } else {
          m--;
          elev -= D.two_ha;
        }
        SV(6) = elev;
        emit = true;
        break;
      }
      // cpp:535/546, then the clip / sector / SVF epilogue of cpp:736-754.
      double h = phase == kPhaseUp ? elev - ha : elev + ha;
      const int j = phase == kPhaseUp ? 2 * m - 1 : 2 * m + 1;  // h ~ j * ha
      if (D.raw_j) D.raw_j[(long long)a * D.ncell + cell] = (int16_t)j;
      if (h < 0.0) h = 0.0;
      double sector = SV(7) + h;
      if (D.refine == 1 || (a + 1) % D.refine == 0) {
        // Converted to degrees by k_finish_outputs.
        const int row = D.refine == 1 ? a : a / D.refine;
        if (check_ok(row < D.nhori && cell >= 0 && cell < D.ncell, kCheckOutput,
                     (long long)row * D.ncell + cell, err))
          D.horizon[(long long)row * D.ncell + cell] = sector;
        sector = 0.0;
      }
      // SVF sum (cpp:333-358, 754). With refine_factor 1 the horizon array
      // holds every clipped h, and k_finish_outputs sums the SVF from it in
      // the same order.
      double svf = SV(8);
      if (D.refine != 1) svf = svf + lattice_svf_term(D, h, j);
      a++;
      if (a == st.i(7)) {
        // Divided by L in k_finish_outputs; a split cell's groups leave
        // partial sums, added there in group order.
        if (D.refine != 1) {
          if (D.groups == 1) D.skyview[cell] = svf;
          else D.svf_part[(long long)(a / (D.L / D.groups) - 1) * D.ncell + cell] = svf;
        }
        if (D.done) {
          // Completion time of the domain's last item (batch latency).
          const unsigned long long fin_items = atomicAdd(&D.done[0], 1ull) + 1ull;
          if (fin_items == (unsigned long long)D.ncell_traced * (unsigned long long)D.groups) {
            unsigned long long now;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            D.done[1] = now;
          }
        }
        // The next cell comes from the warp's chunk in the next pass.
        phase = kPhaseStart;
        break;
      }
      SV(7) = sector;
      SV(8) = svf;
      phase = kPhaseFirst;
    }
    // New azimuth: the elevation carries over (cpp:511), or, with the
    // learned start at every azimuth, starts at the proposal; horizontal
    // direction cos(theta_a) N + sin(theta_a) E.
    const int16_t* start_m = doms[dom].start_m;
    if (start_m && doms[dom].start_all) {
      m = clamp_start(start_m[(long long)a * doms[dom].ncell + cell]);
      SV(6) = (double)m * doms[dom].two_ha;
    }
    const double2 cs = __ldg(&doms[dom].azim_cs[a]);
    // North and east from the frame table (once per azimuth).
    const long long nc = doms[dom].ncell;
    const double* fr = doms[dom].cell_frame + p;
    SV(3) = cs.x * fr[3 * nc] + cs.y * fr[6 * nc];
    SV(4) = cs.x * fr[4 * nc] + cs.y * fr[7 * nc];
    SV(5) = cs.x * fr[5 * nc] + cs.y * fr[8 * nc];
    emit = true;
  }
  st.i(3) = phase;
  if (!alive) return -1;
  if (!emit) return 0;
  st.i(0) = dom;
  st.i(1) = cell;
  st.i(2) = a;
  st.i(4) = up;
  st.i(5) = m;
  st.i(6) = p;
  // Direction at lattice elevation m: cos(e_m) h_a + sin(e_m) U.
  const DomainDesc& D = doms[dom];
  double2 ecs;
  if (m >= kElevMin && m < kElevMin + kElevTable) {
    ecs = __ldg(&D.elev_cs[m - kElevMin]);
  } else {
    const double e = (double)m * D.two_ha;
    ecs = make_double2(cos(e), sin(e));
  }
  dir.x = (float)(ecs.x * SV(3) + ecs.y * SV(0));
  dir.y = (float)(ecs.x * SV(4) + ecs.y * SV(1));
  dir.z = (float)(ecs.x * SV(5) + ecs.y * SV(2));
  dom_out = dom;
  return 1;
#undef SV
#undef SO
}

// Search state of one lane in shared memory (k_trace_warp).
struct LaneState {
  double (*sv)[kFlatBlock];
  int (*si)[kFlatBlock];
  float (*so)[kFlatBlock];
  int t;
  __device__ double& d(int f) const { return sv[f][t]; }
  __device__ int& i(int f) const { return si[f][t]; }
  __device__ float& f(int k) const { return so[k][t]; }
};

template <bool kCount, bool kPrecise, bool kWide>
__global__ void __launch_bounds__(kFlatBlock, HZ_WARP_MIN_BLOCKS)
    k_trace_warp(const DomainDesc* __restrict__ doms, int ndom, const int* __restrict__ order,
                 int total, int* __restrict__ work, unsigned long long* __restrict__ counters,
                 int* __restrict__ err, int advance_min, int leaf_min, int chunk) {
  // Per-lane search state (128 bytes; the rest of the SM's L1 caches the
  // tree). FP64: 0-2 sphere normal U, 3-5 horizontal direction of the
  // current azimuth, 6 elevation accumulator, 7 sector sum, 8 SVF sum.
  // Integers: domain, cell, azimuth, phase, upward steps, lattice index m of
  // the current elevation, position of the cell in the work order, end
  // azimuth of the item, the deep walk's bracket and start, and the
  // triangle that hid the lane's last ray (-1: none). FP32 ray origin (hi,
  // and lo in precise mode).
  __shared__ double sv[9][kFlatBlock];
  __shared__ int si[11][kFlatBlock];
  __shared__ float so[kPrecise ? 6 : 3][kFlatBlock];
  __shared__ int wq[2][kFlatBlock / 32];  // per warp: next and end of its chunk of work ids
  constexpr unsigned kFull = 0xffffffffu;
  const int t = threadIdx.x;
  if ((t & 31) == 0) {
    wq[0][t >> 5] = 0;
    wq[1][t >> 5] = 0;
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 10; q++) si[q][t] = 0;
  si[3][t] = kPhaseStart;
  si[kOccluder][t] = -1;

  bool alive = true, need = true, last_hit = false;
  int ref = kEmptyRef, sp = 0;
  StackTop top;
  // Postponed leaf as next triangle << 4 | triangles left (0 = none).
  int pl0 = 0;
  int stack[kWide ? kStackDepth4 : kStackDepth];
  const Node* nodes = nullptr;
  const Node4* nodes4 = nullptr;
  const Tri* tris = nullptr;
  const float4* tri_lo = nullptr;
  int n_tri = 0;  // of the lane's domain (checked builds)
  Ray r;
  unsigned long long rays = 0, nvis = 0, ntest = 0;
#ifdef HZ_DIAG
  // Per-warp loop statistics: iterations, node passes, node lanes, triangle
  // passes, triangle lanes, advance passes, advancing lanes, live lanes,
  // tracing lanes (summed over iterations); warp start / end times.
  unsigned long long dg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  // SM clock cycles the warp spends in the advance, node and triangle
  // sections of its loop.
  unsigned long long cyc[3] = {0, 0, 0};
  long long c_mark = clock64();
  unsigned long long t_start;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
#define HZ_DIAG_SECTION(k_)              \
  do {                                   \
    const long long c_now_ = clock64();  \
    cyc[k_] += c_now_ - c_mark;          \
    c_mark = c_now_;                     \
  } while (0)
#else
#define HZ_DIAG_SECTION(k_) \
  do {                      \
  } while (0)
#endif

  // A leaf target is postponed when the lane holds none and the lane
  // continues from its stack; a ray with neither a target nor a postponed
  // leaf has missed.
  auto settle = [&]() {
    if (ref < 0 && ref != kEmptyRef && pl0 == 0) {
      if (check_ok(leaf_start(ref) >= 0 && leaf_start(ref) + leaf_count(ref) <= n_tri,
                   kCheckLeaf, leaf_start(ref), err))
        pl0 = (leaf_start(ref) << 4) | leaf_count(ref);
      ref = stk_pop<kWide ? kRegsWide : kRegsBinary>(stack, sp, top);
    }
    if (ref == kEmptyRef && pl0 == 0) {
      need = true;
      last_hit = false;
    }
  };

  for (;;) {
    const unsigned live = __ballot_sync(kFull, alive);
    if (live == 0u) break;
    const unsigned waiting = __ballot_sync(kFull, alive && need);
#ifdef HZ_DIAG
    dg[0]++;
    dg[7] += __popc(live);
    dg[8] += __popc(live & ~waiting);
    if (waiting != 0u && (__popc(waiting) >= advance_min || waiting == live)) {
      dg[5]++;
      dg[6] += __popc(waiting);
    }
#endif
    const bool advance = waiting != 0u && (__popc(waiting) >= advance_min || waiting == live);
    // Cells for the lanes that start one: consecutive work ids (curve order)
    // from the warp's chunk, refilled with one atomic of `chunk` ids.
    int k_new = 0;
    if (advance) {
      const unsigned starting = __ballot_sync(kFull, alive && need && si[3][t] == kPhaseStart);
      if (starting != 0u) {
        const int lane = t & 31, w = t >> 5;
        const int nreq = __popc(starting);
        int first = 0, take = 0, nb = 0;
        if (lane == 0) {
          take = min(wq[1][w] - wq[0][w], nreq);
          first = wq[0][w];
          wq[0][w] += take;
          if (take < nreq) {
            // Near the end of the queue (less than one chunk per warp of the
            // launch left) a warp takes only what it needs, so the last
            // cells spread over more warps.
            const int left = total - *(volatile int*)work;
            const bool tail = left < (int)min(2147483647ll, (long long)gridDim.x * (kFlatBlock / 32) * chunk);
            const int grab = tail ? nreq - take : max(chunk, nreq - take);
            nb = atomicAdd(work, grab);
            wq[0][w] = nb + (nreq - take);
            wq[1][w] = nb + grab;
          }
        }
        first = __shfl_sync(kFull, first, 0);
        take = __shfl_sync(kFull, take, 0);
        nb = __shfl_sync(kFull, nb, 0);
        const int rank = __popc(starting & ((1u << lane) - 1u));
        k_new = rank < take ? first + rank : nb + (rank - take);
      }
    }
    if (advance && alive && need) {
      const LaneState st{sv, si, so, t};
      float3 d;
      int dom = 0;
      const int res =
          search_step<kPrecise>(st, doms, ndom, order, total, k_new, last_hit, d, dom, err);
      if (res < 0) {
        alive = false;
      } else if (res > 0) {
        const DomainDesc& D = doms[dom];
        if (kWide) nodes4 = D.nodes4;
        else nodes = D.nodes;
        tris = D.tris;
        n_tri = D.n_tri;
        if (kPrecise) tri_lo = D.tri_lo;
        if (kPrecise)
          r = make_ray(so[0][t], so[1][t], so[2][t], d.x, d.y, d.z, D.tfar,
                       so[kPrecise ? 3 : 0][t], so[kPrecise ? 4 : 0][t], so[kPrecise ? 5 : 0][t]);
        else
          r = make_ray(so[0][t], so[1][t], so[2][t], d.x, d.y, d.z, D.tfar);
        ref = D.root;
        sp = 0;
        top.clear();
        pl0 = 0;
        need = false;
        rays++;
        settle();
        // Occluder cache: an upward step 2 hori_acc above a ray that hit
        // first tests the triangle that hid that ray. The query is any-hit
        // (cpp:446-460), so a hit there is the traversal's answer: the ray
        // ends without touching the tree and the lane takes its next step
        // in the next advance pass. (Taking it at once, in a loop here,
        // measured 26 % slower: the loop costs the kernel registers.)
        const int occ = si[kOccluder][t];
        si[kOccluder][t] = -1;
        if (occ >= 0 && D.occ_cache && si[3][t] == kPhaseUp) {
          if (kCount) ntest++;
          if (test_tri<kPrecise>(tris, tri_lo, r, occ)) {
            si[kOccluder][t] = occ;
            need = true;
            last_hit = true;
          }
        }
      }
    }

    HZ_DIAG_SECTION(0);
    // Node pass.
#ifdef HZ_DIAG
    {
      const unsigned nl = __ballot_sync(kFull, alive && !need && ref >= 0);
      if (nl) {
        dg[1]++;
        dg[2] += __popc(nl);
      }
    }
#endif
#pragma unroll
    for (int step = 0; step < HZ_NODE_STEPS; step++) {
      if (alive && !need && ref >= 0) {
        if (kCount) nvis++;
        if (!check_ok(ref < (n_tri > 1 ? n_tri - 1 : 1), kCheckNode, ref, err)) {
          ref = kEmptyRef;  // the ray ends as if it had hit (the call fails)
          need = true;
          last_hit = true;
        } else if (!(kWide ? visit_node4(nodes4, r, ref, stack, sp, top)
                    : visit_node(nodes, r, ref, stack, sp, top))) {
          atomicOr(err, kErrStack);
          need = true;
          last_hit = true;
        } else {
          settle();
        }
      }
    }
    HZ_DIAG_SECTION(1);
    // Triangle pass.
    const bool has_leaf = alive && !need && pl0 != 0;
    const unsigned pend = __ballot_sync(kFull, has_leaf);
    if (pend != 0u) {
      const unsigned nodes_left = __ballot_sync(kFull, alive && !need && ref >= 0);
#ifdef HZ_DIAG
      if (__popc(pend) >= leaf_min || nodes_left == 0u) {
        dg[3]++;
        dg[4] += __popc(pend);
      }
#endif
      if ((__popc(pend) >= leaf_min || nodes_left == 0u) && has_leaf) {
        // Up to HZ_TRI_STEPS triangles: the rest of a 2-triangle leaf, or
        // the first of the next postponed leaf once settle() has moved it up.
#pragma unroll
        for (int q = 0; q < HZ_TRI_STEPS; q++) {
          if (q > 0 && (need || pl0 == 0)) break;
          if (kCount) ntest++;
          const int k = pl0 >> 4;
          const bool hit = test_tri<kPrecise>(tris, tri_lo, r, k);
          pl0 += (1 << 4) - 1;  // next triangle, one fewer left
          if (hit) {
            need = true;
            last_hit = true;
            si[kOccluder][t] = k;
          } else if ((pl0 & 15) == 0) {
            pl0 = 0;  // leaf done: the slot is free again
            settle();
          }
        }
      }
    }
    HZ_DIAG_SECTION(2);
  }
  rays = warp_sum_u64(rays);
  if (kCount) {
    nvis = warp_sum_u64(nvis);
    ntest = warp_sum_u64(ntest);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&counters[0], rays);
    if (kCount) {
      atomicAdd(&counters[1], nvis);
      atomicAdd(&counters[2], ntest);
    }
#ifdef HZ_DIAG
    for (int q = 0; q < 9; q++) atomicAdd(&counters[3 + q], dg[q]);
    unsigned long long t_end;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_end));
    atomicMin(&counters[12], t_start);  // host clears this word to ~0
    atomicMin(&counters[13], t_end);
    atomicMax(&counters[14], t_end);
    atomicAdd(&counters[15], t_end - t_start);
    for (int q = 0; q < 3; q++) atomicAdd(&counters[16 + q], cyc[q]);
#endif
  }
}
#undef HZ_DIAG_SECTION

// Any-hit query of arbitrary rays, one thread per ray, with the search's own
// ray setup, box tests, traversal steps and watertight triangle test
// (mo_lradtopo_horayzon.cpp:446-460): the binary tree through `occluded`,
// the 4-wide tree through visit_node4 and test_tri.
template <bool kWide>
__global__ void __launch_bounds__(128)
    k_rays(const Node* __restrict__ nodes, const Node4* __restrict__ nodes4,
           const Tri* __restrict__ tris, int root, const float* __restrict__ org,
           const float* __restrict__ dir, int n, float tfar, uint8_t* __restrict__ hit,
           int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Ray r = make_ray(org[3LL * i], org[3LL * i + 1], org[3LL * i + 2], dir[3LL * i],
                         dir[3LL * i + 1], dir[3LL * i + 2], tfar);
  bool h = false;
  if (!kWide) {
    unsigned long long nv = 0, nt = 0;
    h = occluded<false>(r, nodes, tris, root, nv, nt, err);
  } else {
    int stack[kStackDepth4];
    int sp = 0, ref = root;
    StackTop top;
    while (ref != kEmptyRef && !h) {
      if (ref < 0) {
        const int s0 = leaf_start(ref), c = leaf_count(ref);
        for (int k = s0; k < s0 + c && !h; k++) h = test_tri<false>(tris, nullptr, r, k);
        ref = stk_pop<kRegsWide>(stack, sp, top);
      } else if (!visit_node4(nodes4, r, ref, stack, sp, top)) {
        atomicOr(err, kErrStack);
        h = true;
      }
    }
  }
  hit[i] = h ? 1 : 0;
}

// Frame and FP32 ray origin of every traced cell, mo_lradtopo_horayzon.cpp:
// 694-720 (the per-cell kernel's expressions), stored by the cell's position
// in the work order (the search reads them coalesced).
template <bool kPrecise>
__global__ void k_cell_frames(const DomainDesc* __restrict__ doms, int ndom,
                              const int* __restrict__ order, int total) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  const long long g = order[k];
  const DomainDesc& D = doms[domain_of(doms, ndom, g)];
  const int cell = (int)(g - D.cell_offset);
  const long long p = k - D.k_begin;
  const V3 q{D.cell_enu[3LL * cell], D.cell_enu[3LL * cell + 1], D.cell_enu[3LL * cell + 2]};
  V3 normal{q.x - D.centre.x, q.y - D.centre.y, q.z - D.centre.z};
  unit3(normal);
  const V3 v_n{D.pole.x - q.x, D.pole.y - q.y, D.pole.z - q.z};
  const double dp = dot3(v_n, normal);
  V3 north{v_n.x - dp * normal.x, v_n.y - dp * normal.y, v_n.z - dp * normal.z};
  unit3(north);
  const V3 east = cross3(north, normal);
  const double o64x = q.x + normal.x * D.ray_org_elev;
  const double o64y = q.y + normal.y * D.ray_org_elev;
  const double o64z = q.z + normal.z * D.ray_org_elev;
  const long long nc = D.ncell;
  double* fr = D.cell_frame + p;
  fr[0] = normal.x; fr[nc] = normal.y; fr[2 * nc] = normal.z;
  fr[3 * nc] = north.x; fr[4 * nc] = north.y; fr[5 * nc] = north.z;
  fr[6 * nc] = east.x; fr[7 * nc] = east.y; fr[8 * nc] = east.z;
  float* org = D.cell_origin + p;
  const float ox = (float)o64x, oy = (float)o64y, oz = (float)o64z;
  org[0] = ox;
  org[nc] = oy;
  org[2 * nc] = oz;
  if (kPrecise) {
    org[3 * nc] = (float)(o64x - (double)ox);
    org[4 * nc] = (float)(o64y - (double)oy);
    org[5 * nc] = (float)(o64z - (double)oz);
  }
}

// The search's sums to outputs (cpp:736-754): horizon sector sums [rad] ->
// degrees (v / pi * 180, the division by div_pi_rn) and mean over
// refine_factor; SVF sum -> mean over the azimuths. x / 1.0 == x exactly, so
// that division is left out for refine_factor 1 (kRefine1: a separate
// instance, so that no division is evaluated and discarded per value). One
// thread per traced cell in index order (coalesced rows of horizon): thread
// k is the (k - k_begin)-th traced cell of the domain holding position k. A
// thread reads kFinishRows rows before it converts and stores them, so that
// several loads are in flight per thread.
constexpr int kFinishRows = 8;

template <bool kRefine1>
__device__ __forceinline__ void finish_cell(const DomainDesc& D, int cell) {
  const long long nc = D.ncell;
  const int nhori = D.nhori;
  const double refine = (double)D.refine;
  const float inv_ha = (float)(1.0 / D.hori_acc);
  double* col = D.horizon + cell;
  double svf = 0.0;
  for (int j0 = 0; j0 < nhori; j0 += kFinishRows) {
    double v[kFinishRows];
#pragma unroll
    for (int u = 0; u < kFinishRows; u++)
      v[u] = j0 + u < nhori ? col[(long long)(j0 + u) * nc] : 0.0;
#pragma unroll
    for (int u = 0; u < kFinishRows; u++) {
      if (j0 + u >= nhori) break;
      const double deg = __dmul_rn(div_pi_rn(v[u]), 180.0);
      if (kRefine1) {
        // v is the clipped h of azimuth j0 + u; h > 0 lies on the lattice
        // j * hori_acc up to the rounding of the elevation sum.
        svf = svf + finish_svf_term(D, v[u], inv_ha);
        col[(long long)(j0 + u) * nc] = deg;
      } else {
        col[(long long)(j0 + u) * nc] = deg / refine;
      }
    }
  }
  if (!kRefine1) {
    if (D.groups == 1) {
      svf = D.skyview[cell];
    } else {
      svf = D.svf_part[cell];
      for (int q = 1; q < D.groups; q++) svf = svf + D.svf_part[(long long)q * nc + cell];
    }
  }
  D.skyview[cell] = svf / (double)D.L;
}

__global__ void k_finish_outputs(const DomainDesc* __restrict__ doms, int ndom, int total) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  int lo = 0, hi = ndom - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (doms[mid].k_begin <= k) lo = mid;
    else hi = mid - 1;
  }
  const DomainDesc& D = doms[lo];
  const int cell = D.cell_begin + (int)(k - D.k_begin);
  if (D.refine == 1) finish_cell<true>(D, cell);
  else finish_cell<false>(D, cell);
}

// Bounds of the traced cells' horizontal ENU positions (for their curve keys).
__global__ void k_cell_bounds(const double* __restrict__ cell_enu, int begin, int count,
                              unsigned* __restrict__ bounds) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = k < count;
  const float x = valid ? (float)cell_enu[3LL * (begin + k)] : 0.f;
  const float y = valid ? (float)cell_enu[3LL * (begin + k) + 1] : 0.f;
  unsigned b[4] = {valid ? f2ord(x) : 0xFFFFFFFFu, valid ? f2ord(y) : 0xFFFFFFFFu,
                   valid ? f2ord(x) : 0u, valid ? f2ord(y) : 0u};
  block_bounds_atomic<2, 2>(b, bounds);
}

__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x &= 0x0000FFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

#ifndef HZ_CELL_ORDER
#define HZ_CELL_ORDER 1  // order of the work queue: 0 Morton (Z) curve, 1 Hilbert curve
#endif

// Index of (x, y) in [0, 2^16)^2 along the Hilbert curve (the classic
// quadrant-by-quadrant construction, rotating / reflecting each sub-square).
__device__ __forceinline__ uint32_t hilbert16(uint32_t x, uint32_t y) {
  uint32_t d = 0;
  for (uint32_t s = 1u << 15; s > 0; s >>= 1) {
    const uint32_t rx = (x & s) ? 1u : 0u;
    const uint32_t ry = (y & s) ? 1u : 0u;
    d += s * s * ((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = 65535u - x;
        y = 65535u - y;
      }
      const uint32_t t = x;
      x = y;
      y = t;
    }
  }
  return d;
}

// Cells of a border vertex (a vertex with a -2 entry in cells_of_vertex, the
// reference's border, functions.py:58-97): the edge row, whose searches look
// out over the void and cost several times an inner cell's.
__global__ void k_mark_border(const int* __restrict__ cov, int nv, int ncell,
                              uint8_t* __restrict__ border) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  bool edge = false;
#pragma unroll
  for (int j = 0; j < 6; j++) edge |= cov[(long long)nv * j + v] == -2;
  if (!edge) return;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const int c = cov[(long long)nv * j + v];
    if (c >= 0 && c < ncell) border[c] = 1;
  }
}

// Queue key of a cell: its Hilbert index (or Morton) shifted right by one,
// with the top bit set for cells off the border, so that the border cells,
// the longest searches, are queued first (longest job first: the search's
// last wave then holds no border cell).
__global__ void k_cell_keys(const double* __restrict__ cell_enu, int begin, int count,
                            int id_offset, const unsigned* __restrict__ bounds,
                            const uint8_t* __restrict__ border,
                            uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float mnx = ord2f(bounds[0]), mny = ord2f(bounds[1]);
  const float ex = ord2f(bounds[2]) - mnx, ey = ord2f(bounds[3]) - mny;
  const float x = (float)cell_enu[3LL * (begin + k)];
  const float y = (float)cell_enu[3LL * (begin + k) + 1];
  const float fx = ex > 0.f ? (x - mnx) * (65535.0f / ex) : 0.f;
  const float fy = ey > 0.f ? (y - mny) * (65535.0f / ey) : 0.f;
  const uint32_t qx = fx <= 0.f ? 0u : (fx >= 65535.0f ? 65535u : (uint32_t)fx);
  const uint32_t qy = fy <= 0.f ? 0u : (fy >= 65535.0f ? 65535u : (uint32_t)fy);
#if HZ_CELL_ORDER == 1
  const uint32_t key = hilbert16(qx, qy);
#else
  const uint32_t key = spread16(qx) | (spread16(qy) << 1);
#endif
  const bool first = border != nullptr && border[begin + k] != 0;
  keys[k] = (key >> 1) | (first ? 0u : 0x80000000u);
  vals[k] = id_offset + begin + k;
}

// Lattice tables: azimuths theta_a = shift + a * 2 pi / L (cpp:653-668),
// elevations m * 2 * hori_acc (cpp:527, 538) and the SVF term of
// sin(j * hori_acc) for clipped horizons on the lattice (cpp:333-358).
__global__ void k_trace_tables(double2* __restrict__ azim_cs, double2* __restrict__ elev_cs,
                               double* __restrict__ svf_lattice, int L, double shift,
                               double hori_acc, int svf_type) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < L) {
    const double th = shift + (double)i * ((2.0 * kPi) / (double)L);
    azim_cs[i] = make_double2(cos(th), sin(th));
  }
  if (i < kElevTable) {
    const double e = (double)(kElevMin + i) * (2.0 * hori_acc);
    elev_cs[i] = make_double2(cos(e), sin(e));
  }
  if (i < kSvfTable) svf_lattice[i] = svf_term(sin((double)i * hori_acc), svf_type);
}

__global__ void k_init_cell_bounds(unsigned* b, int* work) {
  b[0] = 0xFFFFFFFFu;
  b[1] = 0xFFFFFFFFu;
  b[2] = 0u;
  b[3] = 0u;
  *work = 0;
}

}  // namespace

cudaError_t trace_tables(double2* azim_cs, double2* elev_cs, double* svf_lattice, int L,
                         double shift, double hori_acc, int svf_type, cudaStream_t s) {
  const int n = L > kSvfTable ? L : kSvfTable;
  k_trace_tables<<<grid_for(n, 256), 256, 0, s>>>(azim_cs, elev_cs, svf_lattice, L, shift,
                                                  hori_acc, svf_type);
  note_launches(1);
  return cudaGetLastError();
}

size_t cell_order_scratch_bytes(long long n) {
  if (n < 1) n = 1;
  return 4 * sizeof(uint32_t) * (size_t)n + (size_t)n + radix_scratch_u32(n) + 64 + 6 * 256;
}

cudaError_t cell_order(const double* cell_enu, const int* cov, int nv, int ncell, int begin,
                       int count, int id_offset, int32_t* order, void* scratch,
                       unsigned* bounds, int* work, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  char* base = (char*)scratch;
  auto take = [&](size_t bytes) {
    char* q = base;
    base += (bytes + 255) & ~size_t(255);
    return (void*)q;
  };
  uint32_t* keys = (uint32_t*)take(sizeof(uint32_t) * count);
  uint32_t* keys_alt = (uint32_t*)take(sizeof(uint32_t) * count);
  int32_t* vals_alt = (int32_t*)take(sizeof(int32_t) * count);
  void* sort_scratch = take(radix_scratch_u32(count));
  uint8_t* border = nullptr;
  if (cov != nullptr && nv > 0 && ncell > 0) {
    border = (uint8_t*)take((size_t)ncell);
    cudaError_t e = cudaMemsetAsync(border, 0, (size_t)ncell, s);
    if (e != cudaSuccess) return e;
    k_mark_border<<<grid_for(nv, 256), 256, 0, s>>>(cov, nv, ncell, border);
    note_launches(1);
  }
  k_init_cell_bounds<<<1, 1, 0, s>>>(bounds, work);
  k_cell_bounds<<<grid_for(count, 256), 256, 0, s>>>(cell_enu, begin, count, bounds);
  k_cell_keys<<<grid_for(count, 256), 256, 0, s>>>(cell_enu, begin, count, id_offset, bounds,
                                                   border, keys, order);
  note_launches(3);
  return radix_sort_pairs(keys, order, keys_alt, vals_alt, count, 32, sort_scratch, s);
}

#ifndef HZ_CARVEOUT
#define HZ_CARVEOUT 1  // 1: ask for the smallest shared-memory carveout that holds the blocks
#endif

// Shared memory is carved out of the SM's 256 KB of L1: ask for just what
// HZ_WARP_MIN_BLOCKS resident blocks need, so the rest caches the tree.
template <typename K>
void prefer_l1(K kernel) {
#if HZ_CARVEOUT
  cudaFuncAttributes fa;
  int dev = 0, smem_sm = 0, reserved = 0;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) !=
          cudaSuccess ||
      smem_sm <= 0) {
    (void)cudaGetLastError();
    return;
  }
  const long long need = (long long)HZ_WARP_MIN_BLOCKS * ((long long)fa.sharedSizeBytes + reserved);
  const int pct = (int)std::min<long long>(100, (need * 100 + smem_sm - 1) / smem_sm);
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct) !=
      cudaSuccess)
    (void)cudaGetLastError();
#else
  (void)kernel;
#endif
}

// One persistent launch: as many blocks as fit on the device at once, at
// most one block per kFlatBlock work items.
template <typename... P, typename... A>
cudaError_t launch_persistent(void (*kernel)(P...), int total, cudaStream_t s, A... args) {
  int dev = 0, sms = 0, per_sm = 0;
  prefer_l1(kernel);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kFlatBlock, 0);
  long long blocks = (long long)sms * (per_sm > 0 ? per_sm : 1);
  const long long needed = ((long long)total + kFlatBlock - 1) / kFlatBlock;
  if (blocks > needed) blocks = needed;
  kernel<<<(unsigned)blocks, kFlatBlock, 0, s>>>(args...);
  note_launches(1);
  return cudaGetLastError();
}

template <bool kCount, bool kPrecise>
cudaError_t launch_variant(const DomainDesc* doms, int ndom, const int32_t* order, int total,
                           int* work, unsigned long long* counters, int* err, int advance_min,
                           int leaf_min, int chunk, int variant, cudaStream_t s) {
  if (variant == kTraceWide)
    return launch_persistent(k_trace_warp<kCount, kPrecise, true>, total, s, doms, ndom, order,
                             total, work, counters, err, advance_min, leaf_min, chunk);
  return launch_persistent(k_trace_warp<kCount, kPrecise, false>, total, s, doms, ndom, order,
                           total, work, counters, err, advance_min, leaf_min, chunk);
}

static cudaError_t launch_search(const DomainDesc* doms, int ndom, const int32_t* order,
                                 int total, int* work, unsigned long long* counters, int* err,
                                 const TraceKnobs& k, bool count_work, bool precise,
                                 cudaStream_t s);

cudaError_t trace_flat(const DomainDesc* doms, int ndom, const int32_t* order, int total,
                       int total_items, int* work, unsigned long long* counters, int* err,
                       const TraceKnobs& k, bool count_work, bool precise, cudaStream_t s) {
  if (total <= 0 || ndom <= 0) return cudaSuccess;
  if (precise) k_cell_frames<true><<<grid_for(total, 256), 256, 0, s>>>(doms, ndom, order, total);
  else k_cell_frames<false><<<grid_for(total, 256), 256, 0, s>>>(doms, ndom, order, total);
  note_launches(1);
  cudaError_t e = launch_search(doms, ndom, order, total_items, work, counters, err, k,
                                count_work, precise, s);
  if (e != cudaSuccess) return e;
  k_finish_outputs<<<grid_for(total, 256), 256, 0, s>>>(doms, ndom, total);
  note_launches(1);
  return cudaGetLastError();
}

static cudaError_t launch_search(const DomainDesc* doms, int ndom, const int32_t* order,
                                 int total, int* work, unsigned long long* counters, int* err,
                                 const TraceKnobs& k, bool count_work, bool precise,
                                 cudaStream_t s) {
  const int c = k.chunk >= 1 ? k.chunk : kDefaultChunk;
  if (precise)
    return count_work ? launch_variant<true, true>(doms, ndom, order, total, work, counters,
                                                   err, k.advance_min, k.leaf_min, c, k.variant,
                                                   s)
                      : launch_variant<false, true>(doms, ndom, order, total, work, counters,
                                                    err, k.advance_min, k.leaf_min, c, k.variant,
                                                    s);
  return count_work ? launch_variant<true, false>(doms, ndom, order, total, work, counters, err,
                                                  k.advance_min, k.leaf_min, c, k.variant, s)
                    : launch_variant<false, false>(doms, ndom, order, total, work, counters,
                                                   err, k.advance_min, k.leaf_min, c, k.variant,
                                                   s);
}

cudaError_t trace_rays(const Node* nodes, const Node4* nodes4, const Tri* tris, int root,
                       const float* org, const float* dir, int n_ray, float tfar, bool wide,
                       uint8_t* hit, int* err, cudaStream_t s) {
  if (n_ray <= 0) return cudaSuccess;
  if (wide)
    k_rays<true><<<grid_for(n_ray, 128), 128, 0, s>>>(nodes, nodes4, tris, root, org, dir,
                                                      n_ray, tfar, hit, err);
  else
    k_rays<false><<<grid_for(n_ray, 128), 128, 0, s>>>(nodes, nodes4, tris, root, org, dir,
                                                       n_ray, tfar, hit, err);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t trace_exact(const TraceParams& p, bool count_work, cudaStream_t s) {
  if (p.cell_count <= 0) return cudaSuccess;
  if (count_work) k_trace_exact<true><<<grid_for(p.cell_count, 128), 128, 0, s>>>(p);
  else k_trace_exact<false><<<grid_for(p.cell_count, 128), 128, 0, s>>>(p);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace hz
