// hz_bvh.cu -- linear BVH over the FP32 mesh, built on the device.
//
// Replaces Embree's rtcCommitScene (mo_lradtopo_horayzon.cpp:395-432):
//   1. k_tri_bounds: triangle boxes; centre range of the boxes in x, y and
//      the largest |coordinate| (box margin), reduced with ordered atomics;
//   2. k_morton: 2 x 16-bit Morton keys of the box centres in the horizontal
//      plane (the terrain is a height field, so x/y carry the locality);
//   3. stable radix sort of (key, triangle) pairs;
//   4. k_karras: binary radix tree (Karras, HPG 2012) with index tie-break;
//      subtrees of <= leaf_max triangles (1..8, default kLeafMax) become
//      leaves;
//   5. k_gather: 48-byte triangle records in leaf order;
//   6. k_refit: bottom-up boxes with one atomic arrival counter per node;
//   7. optionally k_treelet: treelet restructuring (Karras & Aila, "Fast
//      parallel construction of high-quality bounding volume hierarchies",
//      HPG 2013) with treelets of 5 leaves, bottom-up like the refit;
//   8. optionally k_collapse4: the 4-wide tree used by the wide traversal.
// Child boxes carry a margin of 2^-20 x the largest coordinate so that box
// culling never hides a triangle the watertight test would report. The tree
// has the same topology as the CPU oracle's (same keys, same splits).
#include "hz_internal.h"

namespace hz {

namespace {

__device__ __forceinline__ uint32_t part1by1(uint32_t x) {
  x &= 0x0000FFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__device__ __forceinline__ float3 load_vert(const float* __restrict__ v, int i) {
  return make_float3(v[3LL * i], v[3LL * i + 1], v[3LL * i + 2]);
}

__global__ void k_init_bounds(unsigned* b) {
  b[0] = 0xFFFFFFFFu;  // min cx
  b[1] = 0xFFFFFFFFu;  // min cy
  b[2] = 0u;           // max cx
  b[3] = 0u;           // max cy
  b[4] = 0u;           // max |coord|
}

__global__ void k_tri_bounds(const float* __restrict__ vert, const int* __restrict__ vot,
                             int n, float2* __restrict__ cxy, unsigned* __restrict__ bounds) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  float cx = 0.f, cy = 0.f, m = 0.f;
  bool valid = t < n;
  if (valid) {
    float3 a = load_vert(vert, vot[3LL * t]);
    float3 b = load_vert(vert, vot[3LL * t + 1]);
    float3 c = load_vert(vert, vot[3LL * t + 2]);
    float lx = fminf(fminf(a.x, b.x), c.x), hx = fmaxf(fmaxf(a.x, b.x), c.x);
    float ly = fminf(fminf(a.y, b.y), c.y), hy = fmaxf(fmaxf(a.y, b.y), c.y);
    cx = __fmul_rn(__fadd_rn(lx, hx), 0.5f);
    cy = __fmul_rn(__fadd_rn(ly, hy), 0.5f);
    cxy[t] = make_float2(cx, cy);
    m = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(b.x))),
              fmaxf(fmaxf(fabsf(b.y), fabsf(b.z)),
                    fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z))));
  }
  // Block-level reduction, then one atomic per value and block.
  unsigned b[5] = {valid ? f2ord(cx) : 0xFFFFFFFFu, valid ? f2ord(cy) : 0xFFFFFFFFu,
                   valid ? f2ord(cx) : 0u, valid ? f2ord(cy) : 0u, valid ? f2ord(m) : 0u};
  block_bounds_atomic<2, 3>(b, bounds);
}

__global__ void k_morton(const float2* __restrict__ cxy, int n,
                         const unsigned* __restrict__ bounds, uint32_t* __restrict__ keys,
                         int32_t* __restrict__ vals) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float mnx = ord2f(bounds[0]), mny = ord2f(bounds[1]);
  const float mxx = ord2f(bounds[2]), mxy = ord2f(bounds[3]);
  const float ex = __fsub_rn(mxx, mnx), ey = __fsub_rn(mxy, mny);
  const float sx = ex > 0.f ? __fdiv_rn(65535.0f, ex) : 0.f;
  const float sy = ey > 0.f ? __fdiv_rn(65535.0f, ey) : 0.f;
  const float2 c = cxy[t];
  const float fx = __fmul_rn(__fsub_rn(c.x, mnx), sx);
  const float fy = __fmul_rn(__fsub_rn(c.y, mny), sy);
  const uint32_t qx = fx <= 0.f ? 0u : (fx >= 65535.0f ? 65535u : (uint32_t)fx);
  const uint32_t qy = fy <= 0.f ? 0u : (fy >= 65535.0f ? 65535u : (uint32_t)fy);
  keys[t] = part1by1(qx) | (part1by1(qy) << 1);
  vals[t] = t;
}

__device__ __forceinline__ int delta(const uint32_t* __restrict__ keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = keys[i], b = keys[j];
  if (a != b) return __clz(a ^ b);
  return 32 + __clz((uint32_t)(i ^ j));
}

__global__ void k_karras(const uint32_t* __restrict__ keys, int n, Node* __restrict__ nodes,
                         int* __restrict__ parent, int* __restrict__ nsize,
                         int* __restrict__ counter, int leaf_max) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + (d < 0 ? d : 0);
  const int first = min(i, j), last = max(i, j);
  const int nl = gamma - first + 1, nr = last - gamma;
  const int c0 = nl <= leaf_max ? leaf_ref(first, nl) : gamma;
  const int c1 = nr <= leaf_max ? leaf_ref(gamma + 1, nr) : gamma + 1;
  nsize[i] = last - first + 1;
  counter[i] = 0;
  nodes[i].d = make_float4(__int_as_float(c0), __int_as_float(c1), 0.f, 0.f);
  if (last - first + 1 > leaf_max) {  // live node: its internal children are live
    if (c0 >= 0) parent[c0] = (i << 1) | 0;
    if (c1 >= 0) parent[c1] = (i << 1) | 1;
  }
}

__global__ void k_gather(const float* __restrict__ vert, const int* __restrict__ vot,
                         const int32_t* __restrict__ order, int n, Tri* __restrict__ tris,
                         const float* __restrict__ vert_lo, float4* __restrict__ tri_lo) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int t = order[s];
  const int i0 = vot[3LL * t], i1 = vot[3LL * t + 1], i2 = vot[3LL * t + 2];
  const float3 a = load_vert(vert, i0);
  const float3 b = load_vert(vert, i1);
  const float3 c = load_vert(vert, i2);
  Tri r;
  r.x = make_float4(a.x, b.x, c.x, __int_as_float(t));
  r.y = make_float4(a.y, b.y, c.y, 0.f);
  r.z = make_float4(a.z, b.z, c.z, 0.f);
  tris[s] = r;
  if (tri_lo) {  // the residuals in the same per-axis layout
    const float3 la = load_vert(vert_lo, i0);
    const float3 lb = load_vert(vert_lo, i1);
    const float3 lc = load_vert(vert_lo, i2);
    tri_lo[3LL * s + 0] = make_float4(la.x, lb.x, lc.x, 0.f);
    tri_lo[3LL * s + 1] = make_float4(la.y, lb.y, lc.y, 0.f);
    tri_lo[3LL * s + 2] = make_float4(la.z, lb.z, lc.z, 0.f);
  }
}

struct Box {
  float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ Box leaf_box(const Tri* __restrict__ tris, int ref, float pad) {
  const int s = leaf_start(ref), c = leaf_count(ref);
  Box b = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int k = s; k < s + c; k++) {
    const Tri t = tris[k];
    b.lx = fminf(fminf(b.lx, t.x.x), fminf(t.x.y, t.x.z));
    b.hx = fmaxf(fmaxf(b.hx, t.x.x), fmaxf(t.x.y, t.x.z));
    b.ly = fminf(fminf(b.ly, t.y.x), fminf(t.y.y, t.y.z));
    b.hy = fmaxf(fmaxf(b.hy, t.y.x), fmaxf(t.y.y, t.y.z));
    b.lz = fminf(fminf(b.lz, t.z.x), fminf(t.z.y, t.z.z));
    b.hz = fmaxf(fmaxf(b.hz, t.z.x), fmaxf(t.z.y, t.z.z));
  }
  b.lx = __fsub_rn(b.lx, pad); b.ly = __fsub_rn(b.ly, pad); b.lz = __fsub_rn(b.lz, pad);
  b.hx = __fadd_rn(b.hx, pad); b.hy = __fadd_rn(b.hy, pad); b.hz = __fadd_rn(b.hz, pad);
  return b;
}

__device__ __forceinline__ void store_child_box(Node* node, int side, const Box& b) {
  float* base = reinterpret_cast<float*>(node);
  // a / b: (lo.x, hi.x, lo.y, hi.y) of child 0 / 1; c: (lo.z, hi.z) per child.
  __stcg(reinterpret_cast<float4*>(base + 4 * side), make_float4(b.lx, b.hx, b.ly, b.hy));
  __stcg(reinterpret_cast<float2*>(base + 8 + 2 * side), make_float2(b.lz, b.hz));
}

__device__ __forceinline__ Box union_of_children(const Node* node) {
  const float* base = reinterpret_cast<const float*>(node);
  const float4 a = __ldcg(reinterpret_cast<const float4*>(base));
  const float4 b = __ldcg(reinterpret_cast<const float4*>(base + 4));
  const float4 c = __ldcg(reinterpret_cast<const float4*>(base + 8));
  Box u;
  u.lx = fminf(a.x, b.x); u.hx = fmaxf(a.y, b.y);
  u.ly = fminf(a.z, b.z); u.hy = fmaxf(a.w, b.w);
  u.lz = fminf(c.x, c.z); u.hz = fmaxf(c.y, c.w);
  return u;
}

__global__ void k_refit(Node* __restrict__ nodes, const Tri* __restrict__ tris, int n,
                        const int* __restrict__ parent, const int* __restrict__ nsize,
                        int* __restrict__ counter, const unsigned* __restrict__ bounds,
                        int leaf_max) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1 || nsize[i] <= leaf_max) return;
  const float pad = __fmul_rn(ord2f(bounds[4]), 9.5367431640625e-07f);
  const float4 d = nodes[i].d;
  const int c0 = __float_as_int(d.x), c1 = __float_as_int(d.y);
  int arrivals = 0;
  if (c0 < 0) { store_child_box(&nodes[i], 0, leaf_box(tris, c0, pad)); arrivals++; }
  if (c1 < 0) { store_child_box(&nodes[i], 1, leaf_box(tris, c1, pad)); arrivals++; }
  if (arrivals == 0) return;
  __threadfence();
  int old = atomicAdd(&counter[i], arrivals);
  if (old + arrivals != 2) return;
  int node = i;
  while (node != 0) {
    __threadfence();
    const Box u = union_of_children(&nodes[node]);
    const int p = parent[node];
    store_child_box(&nodes[p >> 1], p & 1, u);
    __threadfence();
    old = atomicAdd(&counter[p >> 1], 1);
    if (old + 1 != 2) return;
    node = p >> 1;
  }
}

// ---------------------------------------------------------------------------
// Treelet restructuring. Each live node R, once both of its subtrees are
// done, forms a treelet of up to kTreelet leaves: its two children, then
// repeatedly the treelet leaf with the largest cost area that is an internal
// node replaced by its two children. Dynamic programming over the subsets of
// the leaves finds the binary topology of least cost
//   C(node) = kCi * A(node) + C(left) + C(right),  C(leaf) = kCt * count * A(leaf)
// (A: the cost area below), the treelet's internal nodes are rewired to it
// (same node indices, the leaves untouched) and C(R) is kept for R's
// ancestors. Box tests stay conservative (every box is the union of the
// original padded leaf boxes), so the searches' results do not change.
// Cost area: (dx + dy) dz + 0.1 dx dy -- the projected area for the near-
// horizontal rays of the search plus a share of the footprint (ray origins
// lie on the terrain inside it).
// ---------------------------------------------------------------------------
constexpr int kTreelet = 5;
constexpr float kCi = 1.2f, kCt = 1.0f;

__device__ __forceinline__ float cost_area(const Box& b) {
  const float dx = b.hx - b.lx, dy = b.hy - b.ly, dz = b.hz - b.lz;
  if (!(dx >= 0.f)) return 0.f;  // empty
  return (dx + dy) * dz + 0.1f * dx * dy;
}
__device__ __forceinline__ Box box_union(const Box& a, const Box& b) {
  return Box{fminf(a.lx, b.lx), fminf(a.ly, b.ly), fminf(a.lz, b.lz),
             fmaxf(a.hx, b.hx), fmaxf(a.hy, b.hy), fmaxf(a.hz, b.hz)};
}
// Child `side` of node: reference and box (coherent loads: other threads of
// the same launch wrote them).
__device__ __forceinline__ void load_child(const Node* node, int side, int& ref, Box& b) {
  const float* base = reinterpret_cast<const float*>(node);
  const float4 xy = __ldcg(reinterpret_cast<const float4*>(base + 4 * side));
  const float2 z = __ldcg(reinterpret_cast<const float2*>(base + 8 + 2 * side));
  const float2 d = __ldcg(reinterpret_cast<const float2*>(base + 12));
  ref = __float_as_int(side ? d.y : d.x);
  b = Box{xy.x, xy.z, z.x, xy.y, xy.w, z.y};
}
__device__ __forceinline__ void store_node(Node* node, int r0, const Box& b0, int r1,
                                           const Box& b1) {
  __stcg(&node->a, make_float4(b0.lx, b0.hx, b0.ly, b0.hy));
  __stcg(&node->b, make_float4(b1.lx, b1.hx, b1.ly, b1.hy));
  __stcg(&node->c, make_float4(b0.lz, b0.hz, b1.lz, b1.hz));
  __stcg(&node->d, make_float4(__int_as_float(r0), __int_as_float(r1), 0.f, 0.f));
}

// Restructures the treelet rooted at live node R and stores C(R).
__device__ void treelet_at(Node* nodes, int R, int* parent, int* nsize, float* cost,
                           int leaf_max) {
  int lref[kTreelet];
  Box lbox[kTreelet];
  float lcost[kTreelet];
  int pool[kTreelet - 1];
  int nl = 0, np = 0;
  pool[np++] = R;
  for (int side = 0; side < 2; side++) {
    int r;
    Box b;
    load_child(nodes + R, side, r, b);
    if (r == kEmptyRef) continue;
    lref[nl] = r;
    lbox[nl] = b;
    nl++;
  }
  while (nl < kTreelet) {
    int best = -1;
    float ba = -1.f;
    for (int k = 0; k < nl; k++)
      if (lref[k] >= 0) {
        const float a = cost_area(lbox[k]);
        if (a > ba) {
          ba = a;
          best = k;
        }
      }
    if (best < 0) break;
    const int X = lref[best];
    pool[np++] = X;
    load_child(nodes + X, 0, lref[best], lbox[best]);
    load_child(nodes + X, 1, lref[nl], lbox[nl]);
    nl++;
  }
  for (int k = 0; k < nl; k++)
    lcost[k] = lref[k] >= 0 ? __ldcg(cost + lref[k])
                            : kCt * (float)leaf_count(lref[k]) * cost_area(lbox[k]);
  if (nl < 3) {
    const Box u = nl == 2 ? box_union(lbox[0], lbox[1]) : lbox[0];
    __stcg(cost + R, kCi * cost_area(u) + lcost[0] + (nl == 2 ? lcost[1] : 0.f));
    return;
  }
  constexpr int kSets = 1 << kTreelet;
  float copt[kSets];
  Box ubox[kSets];
  unsigned char bestp[kSets];
  const int full = (1 << nl) - 1;
  for (int st = 1; st <= full; st++) {
    const int low = __ffs(st) - 1;
    if ((st & (st - 1)) == 0) {
      copt[st] = lcost[low];
      ubox[st] = lbox[low];
      continue;
    }
    ubox[st] = box_union(ubox[st & (st - 1)], lbox[low]);
    // Partitions (p, st ^ p) with p holding the lowest member of st.
    const int lowbit = st & -st;
    float c = INFINITY;
    int bp = 0;
    for (int p = (st - 1) & st; p; p = (p - 1) & st) {
      if (!(p & lowbit)) continue;
      const float cp = copt[p] + copt[st ^ p];
      if (cp < c) {
        c = cp;
        bp = p;
      }
    }
    copt[st] = kCi * cost_area(ubox[st]) + c;
    bestp[st] = (unsigned char)bp;
  }
  // Rewire: node pool[k] takes the k-th internal subset in depth-first order.
  int qs[kTreelet], qn[kTreelet], qh = 0, used = 1;
  qs[qh] = full;
  qn[qh] = R;
  qh++;
  while (qh > 0) {
    qh--;
    const int st = qs[qh], node = qn[qh];
    const int part[2] = {bestp[st], st ^ bestp[st]};
    int ref[2];
    for (int side = 0; side < 2; side++) {
      const int q = part[side];
      if ((q & (q - 1)) == 0) {
        ref[side] = lref[__ffs(q) - 1];
        if (ref[side] >= 0) parent[ref[side]] = (node << 1) | side;
      } else {
        const int nd = pool[used++];
        ref[side] = nd;
        parent[nd] = (node << 1) | side;
        nsize[nd] = max(nsize[nd], leaf_max + 1);  // live (k_collapse4)
        __stcg(cost + nd, copt[q]);
        qs[qh] = q;
        qn[qh] = nd;
        qh++;
      }
    }
    store_node(nodes + node, ref[0], ubox[part[0]], ref[1], ubox[part[1]]);
  }
  __stcg(cost + R, copt[full]);
}

// Bottom-up over the live nodes (arrival counters as in k_refit, which left
// them at 2: cleared before this launch).
__global__ void k_treelet(Node* __restrict__ nodes, int n, int* __restrict__ parent,
                          int* __restrict__ nsize, int* __restrict__ counter,
                          float* __restrict__ cost, int leaf_max) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1 || nsize[i] <= leaf_max) return;
  const float4 d = nodes[i].d;
  const int arrivals = (__float_as_int(d.x) < 0) + (__float_as_int(d.y) < 0);
  if (arrivals == 0) return;
  __threadfence();
  int old = atomicAdd(&counter[i], arrivals);
  if (old + arrivals != 2) return;
  int node = i;
  for (;;) {
    __threadfence();
    treelet_at(nodes, node, parent, nsize, cost, leaf_max);
    if (node == 0) return;
    const int p = __ldcg(parent + node) >> 1;
    __threadfence();
    old = atomicAdd(&counter[p], 1);
    if (old + 1 != 2) return;
    node = p;
  }
}

// n_tri <= leaf_max: one node, child 0 = leaf of all triangles, child 1 empty.
__global__ void k_small_root(Node* nodes, const Tri* __restrict__ tris, int n,
                             const unsigned* __restrict__ bounds) {
  const float pad = __fmul_rn(ord2f(bounds[4]), 9.5367431640625e-07f);
  const Box b = leaf_box(tris, leaf_ref(0, n), pad);
  Node r;
  r.a = make_float4(b.lx, b.hx, b.ly, b.hy);
  r.b = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
  r.c = make_float4(b.lz, b.hz, INFINITY, -INFINITY);
  r.d = make_float4(__int_as_float(leaf_ref(0, n)), __int_as_float(kEmptyRef), 0.f, 0.f);
  nodes[0] = r;
}

// BVH4 node i from BVH2 node i: a leaf child stays, an internal child is
// replaced by its two children (with the boxes that child stores for them).
// Only live BVH2 nodes (ranges of more than leaf_max triangles, or the single
// root of a small tree) are converted.
__global__ void k_collapse4(const Node* __restrict__ nodes, int n_nodes,
                            const int* __restrict__ nsize, int leaf_max,
                            Node4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes || (nsize && nsize[i] <= leaf_max)) return;
  float lo[3][4], hi[3][4];
  int ch[4];
  int k = 0;
  auto put = [&](int ref, float lx, float hx, float ly, float hy, float lz, float hz) {
    ch[k] = ref;
    lo[0][k] = lx; hi[0][k] = hx;
    lo[1][k] = ly; hi[1][k] = hy;
    lo[2][k] = lz; hi[2][k] = hz;
    k++;
  };
  const Node n = nodes[i];
  const int c[2] = {__float_as_int(n.d.x), __float_as_int(n.d.y)};
  for (int side = 0; side < 2; side++) {
    const int r = c[side];
    if (r == kEmptyRef) continue;
    if (r < 0) {
      const float4 xy = side ? n.b : n.a;
      put(r, xy.x, xy.y, xy.z, xy.w, side ? n.c.z : n.c.x, side ? n.c.w : n.c.y);
    } else {
      const Node m = nodes[r];
      const int g0 = __float_as_int(m.d.x), g1 = __float_as_int(m.d.y);
      put(g0, m.a.x, m.a.y, m.a.z, m.a.w, m.c.x, m.c.y);
      if (g1 != kEmptyRef) put(g1, m.b.x, m.b.y, m.b.z, m.b.w, m.c.z, m.c.w);
    }
  }
  while (k < 4) put(kEmptyRef, INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY);
  Node4 q;
  q.lox = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
  q.hix = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
  q.loy = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
  q.hiy = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
  q.loz = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
  q.hiz = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
  q.child = make_int4(ch[0], ch[1], ch[2], ch[3]);
  q.pad = make_int4(0, 0, 0, 0);
  out[i] = q;
}

}  // namespace

size_t bvh_scratch_bytes(long long n) {
  if (n < 1) n = 1;
  size_t b = 0;
  b += 4 * sizeof(uint32_t) * (size_t)n;  // keys, vals, keys_alt, vals_alt
  b += sizeof(float2) * (size_t)n;
  b += 3 * sizeof(int) * (size_t)n;       // parent, nsize, counter
  b += sizeof(float) * (size_t)n;         // cost (treelets)
  b += 64;                                // bounds
  b += radix_scratch_u32(n);
  return b + 8 * 256;                     // alignment slack
}

cudaError_t bvh_build(const float* vert32, const int* vot, int n, Node* nodes, Tri* tris,
                      const BvhScratch& sc, cudaStream_t s, const float* vert_lo,
                      float4* tri_lo, Node4* nodes4, int leaf_max, bool treelets) {
  if (leaf_max < 1 || leaf_max > 8) leaf_max = kLeafMax;
  if (n <= 0) return cudaSuccess;
  k_init_bounds<<<1, 1, 0, s>>>(sc.bounds);
  k_tri_bounds<<<grid_for(n, 256), 256, 0, s>>>(vert32, vot, n, sc.cxy, sc.bounds);
  k_morton<<<grid_for(n, 256), 256, 0, s>>>(sc.cxy, n, sc.bounds, sc.keys, sc.vals);
  note_launches(3);
  cudaError_t e = radix_sort_pairs(sc.keys, sc.vals, sc.keys_alt, sc.vals_alt, n, 32,
                                   sc.sort_scratch, s);
  if (e != cudaSuccess) return e;
  k_gather<<<grid_for(n, 256), 256, 0, s>>>(vert32, vot, sc.vals, n, tris, vert_lo,
                                            vert_lo ? tri_lo : nullptr);
  if (n <= leaf_max) {
    k_small_root<<<1, 1, 0, s>>>(nodes, tris, n, sc.bounds);
    note_launches(2);
    if (nodes4) {
      k_collapse4<<<1, 32, 0, s>>>(nodes, 1, nullptr, leaf_max, nodes4);
      note_launches(1);
    }
    return cudaGetLastError();
  }
  note_launches(3);
  k_karras<<<grid_for(n - 1, 256), 256, 0, s>>>(sc.keys, n, nodes, sc.parent, sc.nsize,
                                                sc.counter, leaf_max);
  k_refit<<<grid_for(n - 1, 256), 256, 0, s>>>(nodes, tris, n, sc.parent, sc.nsize,
                                               sc.counter, sc.bounds, leaf_max);
  if (treelets && sc.cost) {
    cudaError_t e = cudaMemsetAsync(sc.counter, 0, sizeof(int) * (size_t)(n - 1), s);
    if (e != cudaSuccess) return e;
    k_treelet<<<grid_for(n - 1, 256), 256, 0, s>>>(nodes, n, sc.parent, sc.nsize, sc.counter,
                                                   sc.cost, leaf_max);
    note_launches(1);
  }
  if (nodes4) {
    k_collapse4<<<grid_for(n - 1, 256), 256, 0, s>>>(nodes, n - 1, sc.nsize, leaf_max,
                                                     nodes4);
    note_launches(1);
  }
  return cudaGetLastError();
}

}  // namespace hz
