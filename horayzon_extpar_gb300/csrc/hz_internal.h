// hz_internal.h -- launch functions shared between the library's translation
// units (mesh, sort, BVH, trace, API). Every function enqueues work on the
// given stream and returns the launch status; nothing here synchronises.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hz_common.cuh"

namespace hz {

// Kernel-launch accounting of the calling thread (reported in hz_stats).
void note_launches(int n);
// Sets the calling thread's message returned by hz_last_error().
void set_last_error(const char* msg);

// ---- hz_scan_sort.cu -------------------------------------------------------
// Exclusive prefix sum of n values; total to *d_total (device). `partials`
// needs scan_partials(n) elements.
long long scan_partials(long long n);
cudaError_t scan_exclusive_u64(const unsigned long long* in, unsigned long long* out,
                               long long n, unsigned long long* d_total,
                               unsigned long long* partials, cudaStream_t s);
cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n,
                               uint32_t* d_total, uint32_t* partials, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits.
// Scratch sizes from radix_scratch_u32(n). Result ends in (keys, vals).
size_t radix_scratch_u32(long long n);
cudaError_t radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_alt,
                             int32_t* vals_alt, long long n, int bits, void* scratch,
                             cudaStream_t s);

// ---- hz_mesh.cu -------------------------------------------------------------
// mo_lradtopo_horayzon.cpp:228-317: per ICON vertex, the triangle count in the
// low 32 bits and the appended-vertex count (grid_type 1) in the high 32 bits.
cudaError_t mesh_count(const int* cov, int nv, int ncell, int grid_type,
                       unsigned long long* packed, int* err, cudaStream_t s);
// Emission at the scanned offsets. Appended vertices go to add_{lon,lat,h}.
cudaError_t mesh_emit(const double* clon, const double* clat, const double* hsurf,
                      const double* vlon, const double* vlat, const int* cov, int nv,
                      int ncell, int grid_type, const unsigned long long* offsets,
                      int* vot, double* add_lon, double* add_lat, double* add_h,
                      cudaStream_t s);
// cpp:158-169 for all mesh vertices (cells first, then appended vertices) and
// per-block partial sums of the cell ECEF coordinates (cpp:624-631).
int ecef_blocks(int ncell);
cudaError_t mesh_ecef(const double* clon, const double* clat, const double* hsurf,
                      const double* add_lon, const double* add_lat, const double* add_h,
                      int ncell, int nadd, double* ecef, double* block_sums,
                      double* d_origin_sum, cudaStream_t s);
// cpp:624-644: the domain's ENU frame from the sum of the cells' ECEF
// coordinates (host, glibc; the one definition every entry point uses).
Frame enu_frame_from_sum(double xo, double yo, double zo);
// cpp:178-201: FP32 ENU of every mesh vertex, FP64 ENU of every cell.
// vert_lo (optional, 3 per mesh vertex): FP64 value minus its FP32 rounding.
cudaError_t mesh_enu(const double* ecef, int nmv, int ncell, const Frame& f,
                     float* vert32, double* cell_enu, float* vert_lo, cudaStream_t s);

// ---- hz_bvh.cu --------------------------------------------------------------
struct BvhScratch {
  uint32_t* keys;       // n
  int32_t* vals;        // n
  uint32_t* keys_alt;   // n
  int32_t* vals_alt;    // n
  float2* cxy;          // n triangle-box centres (x, y)
  int* parent;          // n (node -> parent << 1 | side)
  int* nsize;           // n (range size per internal node)
  int* counter;         // n (refit arrivals)
  float* cost;          // n (treelet costs; optional)
  unsigned* bounds;     // 5: min cx, min cy, max cx, max cy, max |coord| (ordered)
  void* sort_scratch;   // radix_scratch_u32(n)
};
size_t bvh_scratch_bytes(long long n_tri);
// Builds nodes[n_tri - 1] (or one node when n_tri <= leaf_max) and tris[n_tri];
// leaves hold at most leaf_max triangles (1..8; other values: kLeafMax);
// the root is node 0. n_tri == 0 leaves the tree empty.
// With vert_lo, also writes tri_lo[3 * n_tri]: the FP32 residuals of v0, v1,
// v2 per triangle in leaf order (precise mode). With nodes4 (same length as
// nodes), also the BVH4 collapse of the tree (root 0).
// treelets: restructure the binary tree by treelets (k_treelet; needs
// sc.cost) before the collapse.
cudaError_t bvh_build(const float* vert32, const int* vot, int n_tri, Node* nodes,
                      Tri* tris, const BvhScratch& sc, cudaStream_t s,
                      const float* vert_lo = nullptr, float4* tri_lo = nullptr,
                      Node4* nodes4 = nullptr, int leaf_max = kLeafMax,
                      bool treelets = false);

// ---- hz_trace.cu ------------------------------------------------------------
struct TraceParams {
  const double* cell_enu;   // [3 * ncell] FP64 ENU of cell centres
  int ncell;                // row stride of horizon
  int cell_begin, cell_count;  // cells traced: [cell_begin, cell_begin + cell_count)
  const Node* nodes;
  const Tri* tris;
  int root;                 // 0, or kEmptyRef for an empty mesh
  double3 centre, pole;     // Earth centre / North Pole in ENU
  double ray_org_elev;
  float tfar;               // (float)dist_search, cpp:587
  int nhori, refine, L, svf_type;
  double hori_acc, elev_floor;
  double azim_sin, azim_cos, elev_sin_2ha, elev_cos_2ha, shift_sin, shift_cos;
  double* horizon;          // [nhori * ncell] degrees
  double* skyview;          // [ncell]
  unsigned long long* counters;  // [0] rays, [1] node visits, [2] triangle tests
  int* err;
};

// Lattice tables of the persistent search (trace_tables): azim_cs [L] cos,
// sin of azimuth shift + a * 360 deg / L; elev_cs [kElevTable] cos, sin of
// m * 0.5 deg, m = kElevMin + i; svf_lattice [kSvfTable] the SVF term
// 1 - sin(j * 0.25 deg)^(svf_type + 1) of a clipped horizon on the lattice.
constexpr int kElevMin = -256;
constexpr int kElevTable = 1280;
constexpr int kSvfTable = 2560;

// Fills the lattice tables (device FP64 sin/cos); shift is the reference's
// azimuth shift (cpp:662-668).
cudaError_t trace_tables(double2* azim_cs, double2* elev_cs, double* svf_lattice, int L,
                         double shift, double hori_acc, int svf_type, cudaStream_t s);
// One thread per cell, nested loops as in the reference (simple; kept as the
// second implementation the flattened kernel is tested against).
// Any-hit flags (hit[i] = 1) of n_ray rays (org, dir: float3 on the device)
// against a tree built by bvh_build; wide: the 4-wide tree (nodes4), else
// the binary one. One thread per ray.
cudaError_t trace_rays(const Node* nodes, const Node4* nodes4, const Tri* tris, int root,
                       const float* org, const float* dir, int n_ray, float tfar, bool wide,
                       uint8_t* hit, int* err, cudaStream_t s);
cudaError_t trace_exact(const TraceParams& p, bool count_work, cudaStream_t s);
// Hilbert-curve order of cells [begin, begin + count) into order[count]; also resets
// the work counter used by trace_flat.
// Work ids are id_offset + cell.
size_t cell_order_scratch_bytes(long long n);
// With cov (device cells_of_vertex, nv vertices, ncell cells of the domain)
// the cells of border vertices come first.
cudaError_t cell_order(const double* cell_enu, const int* cov, int nv, int ncell, int begin,
                       int count, int id_offset, int32_t* order, void* scratch,
                       unsigned* bounds, int* work, cudaStream_t s);

// One domain of the persistent search (device-resident array).
struct DomainDesc {
  const double* cell_enu;     // [3 * ncell] FP64 ENU of cell centres
  // Per traced cell, indexed by its position p = k - k_begin in `order`
  // (k_cell_frames): [9][ncell] sphere normal, north, east; [6][ncell] FP32
  // ray origin and, in precise mode, its residual.
  double* cell_frame;
  float* cell_origin;
  long long k_begin;          // position in `order` of this domain's first work id
  int cell_begin;             // first traced cell (cells cell_begin .. + ncell_traced)
  const Node* nodes;
  const Node4* nodes4;        // BVH4 collapse of nodes (wide traversal only)
  const Tri* tris;
  const float4* tri_lo;       // precise mode: [3 * n_tri] FP32 vertex residuals
  double* horizon;            // [nhori * ncell] degrees (the search leaves the sector
                              // sums in radians; k_finish_outputs converts them)
  double* skyview;            // [ncell] (the search leaves the sums over azimuths)
  const double2* azim_cs;     // lattice tables (trace_tables)
  const double2* elev_cs;
  const double* svf_lattice;
  unsigned long long* done;   // optional: [0] finished items, [1] globaltimer at the last
  const int16_t* start_m;     // optional learned start lattice index [L][ncell]
  int start_all;              // 1: learned start at every azimuth; 0: at each item's first
  // Search items per traced cell: 1 = the reference's chain over all L
  // azimuths; G > 1 = G groups of L / G consecutive azimuths (a multiple of
  // refine), each starting at the learned proposal of its first azimuth.
  int groups;
  long long item_begin;       // first search item of this domain (items: groups x cells)
  double* svf_part;           // groups > 1 and refine > 1: [groups][ncell] SVF sums
  // 1: below the clip (a downward walk at elevation <= hori_acc, whose
  // further candidates all give a clipped horizon) the walk's stop is found
  // by doubling and bisection instead of one step per ray.
  int deep_walk;
  // 1: an upward step first tests the triangle that hid the step below
  // (k_trace_warp's occluder cache; same results, fewer traversals).
  int occ_cache;
  int16_t* raw_j;             // optional output: unclipped horizon j (h = j * 0.25 deg)
  double3 centre, pole;       // Earth centre / North Pole in ENU
  double ray_org_elev, hori_acc, elev_floor;
  double two_ha;              // 2 * hori_acc (exact): one elevation step
  long long cell_offset;      // work id of cell 0 of this domain
  int root, ncell, ncell_traced, nhori, refine, L, svf_type;
  int n_tri;                  // triangles of the tree (nodes: max(1, n_tri - 1))
  float tfar;
};

// Persistent flattened search (same rays and results as trace_exact) over
// `total` work ids from `order`; a work id is cell_offset + cell of its
// domain, and `doms` is sorted by cell_offset. Three launches: the cell
// frames of every traced cell (FP64, coalesced), the search, and the
// conversion of the accumulated sums into degrees and SVF.
// precise: every domain carries tri_lo and rays use hi + lo vertices/origin.
// k.variant: the BVH the search traverses (kTrace*); k.advance_min /
// k.leaf_min: lanes of a warp that must be waiting before the search state
// advances / holding a postponed leaf before a triangle pass runs; k.chunk:
// consecutive work ids a warp claims at a time.
enum : int {
  kTraceWide = 0,   // 4-wide BVH (DomainDesc::nodes4)
  kTraceBinary = 1  // binary BVH (DomainDesc::nodes)
};
// Counter words of the search: 0 rays, 1 node visits, 2 triangle tests; with
// -DHZ_DIAG, 3.. per-warp loop statistics (printed to stderr by the host).
constexpr int kCounterWords = 20;
constexpr int kDefaultAdvanceMin = 16;
// A triangle pass as soon as one lane of the warp holds a postponed leaf:
// measured fastest on every benchmarked configuration (1.2-2 % against 12).
constexpr int kDefaultLeafMin = 1;
constexpr int kDefaultChunk = 32;
struct TraceKnobs {
  int advance_min;  // 1..32
  int leaf_min;     // 1..32
  int chunk;        // work ids a warp claims per atomic (< 1: kDefaultChunk)
  int variant;      // kTrace*
};
// `total` traced cells (frames, epilogue) and `total_items` search items
// (the sum of groups x traced cells over the domains).
cudaError_t trace_flat(const DomainDesc* doms, int ndom, const int32_t* order, int total,
                       int total_items, int* work, unsigned long long* counters, int* err,
                       const TraceKnobs& k, bool count_work, bool precise, cudaStream_t s);

// ---- hz_static.cu -----------------------------------------------------------
// Forgets the cached device address of the no-allocation entry point's
// static array on `device` (-1: all devices).
void static_forget_device(int device);

// ---- hz_hostcopy.cu ---------------------------------------------------------
// Copies between device memory and caller host buffers: page-locked buffers
// by cudaMemcpyAsync (asynchronous), pageable ones through two page-locked
// chunks with multi-threaded host copies (returns when the data has arrived).
struct Staging;
cudaError_t staging_create(Staging** out);
void staging_destroy(Staging* st);
cudaError_t copy_to_host(Staging* st, void* dst, const void* src_dev, size_t bytes,
                         cudaStream_t s);
cudaError_t copy_from_host(Staging* st, void* dst_dev, const void* src, size_t bytes,
                           cudaStream_t s);

// ---- hz_learn.cu ------------------------------------------------------------
constexpr int kMlpIn = 32;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden +
                           kMlpHidden + kMlpHidden + 1;  // 6337
constexpr int kMlpStartMin = -170;  // -85 deg
constexpr int kMlpStartMax = 180;   // +90 deg

// Height field of a domain on a regular grid of its ENU x/y plane.
struct RasterDesc {
  float x0, y0, dx, inv_dx;
  int nx, ny;
  // [ny][nx]: the heights of texel (ix, iy) and of its neighbours (ix + 1,
  // iy), (ix, iy + 1), (ix + 1, iy + 1), so that a bilinear sample is one
  // 16-byte load; -inf where no triangle covers a texel.
  const float4* quad;
};

struct LearnParams {
  const double* cell_enu;
  double3 centre, pole;
  double ray_org_elev;
  int ncell, cell_begin, cell_count, nhori, L;
  int n_pred, a_stride;  // azimuths q * a_stride, q < n_pred, get features / predictions
  float dist_search;
  const double2* azim_cs;
  const RasterDesc* raster;  // device (raster_build)
  float* features;   // optional [L][ncell][32]
  int16_t* start_m;  // with params: learned start lattice index [L][ncell]
};

// The height raster of a domain: descriptor (sized from the BVH build's
// triangle-centre bounds, at most `budget` texels) to *rdesc on the device,
// then the maximum height of the covering triangles per texel, as the quads
// of RasterDesc::quad.
cudaError_t raster_build(const float* vert32, const int* vot, int n_tri, const unsigned* bounds,
                         long long budget, RasterDesc* rdesc, unsigned* zbits, float4* quad,
                         cudaStream_t s);
// Features of every traced (cell, azimuth); with params (FP32, kMlpParams,
// device) also the MLP's start index.
cudaError_t learn_features(const LearnParams& q, const float* params, cudaStream_t s);
size_t mlp_train_scratch_floats(int n);
// One step on n samples: gradients to grads[kMlpParams]; with lr > 0 an Adam
// update of params (step counts from 1).
cudaError_t mlp_train_step(float* params, float* adam_m, float* adam_v, const float* X,
                           const float* T, int n, int step, float lr, float* loss,
                           float* grads, float* scratch, cudaStream_t s);
cudaError_t mlp_forward(const float* params, const float* X, int n, float* Y, cudaStream_t s);

}  // namespace hz
