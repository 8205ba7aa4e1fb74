// hz_static.cu -- hz_horizon_svf_device_static: the horizon / SVF computation
// for callers that cannot allocate GPU memory.
//
// Some callers must not call cudaMalloc: a host model whose GPU memory is
// entirely owned by another allocator (a framework's caching pool, or an
// application that reserves the whole device up front), or a time-stepping
// code sharing the GPU that cannot afford the device-wide synchronisation
// cudaMalloc/cudaFree imply. This entry point allocates nothing: the caller
// passes device inputs and outputs, and all intermediate data (mesh, frames,
// BVH, work counters) lives in one file-scope __device__ array of
// kStaticScratchBytes, which every GPU that loads the library keeps until the
// process exits.
//
// Host code cannot use the array's name as a device address (it names a
// host-side shadow), so on the first call on each device, with that device
// current, cudaGetSymbolAddress resolves the device address and the address
// is kept; hz_release_workspace(device) forgets it (call it after a
// cudaDeviceReset). The function itself cannot run inside a stream capture:
// it reads results back to the host and waits for its stream mid-call. All
// calls share the array, so GPU work of two calls must never overlap: the
// entry point holds a process-wide lock and, on every return after its first
// queued operation (success or failure), waits for its stream. Values left
// from the previous call are never read: every counter and flag that must
// start at zero is cleared on the stream at the start of the call. Failures
// are reported through hz_last_error() like the other entry points.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/horayzon_gb300.h"
#include "hz_internal.h"

namespace hz {
namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;  // 64 MiB per device

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_addr[128] = {};  // device address of g_static_scratch, per device
// Failure text goes to the message hz_last_error() returns.
int static_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
  char buf[320];
  if (e != cudaSuccess)
    snprintf(buf, sizeof(buf), "%s: %s", msg, cudaGetErrorString(e));
  else
    snprintf(buf, sizeof(buf), "%s", msg);
  set_last_error(buf);
  return code;
}

#define HZ_STATIC_CUDA(call, what)                         \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return static_fail(HZ_ERR_CUDA, what, e_); \
  } while (0)

// Bump layout inside the static array (base == nullptr: size only).
struct Layout {
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += sizeof(T) * (n ? n : 1);
    return p;
  }
};

struct StaticBuffers {
  unsigned long long *packed, *offsets, *scan_partials, *totals;
  int* vot;
  double *add_lon, *add_lat, *add_h, *ecef, *block_sums, *origin_sum, *cell_enu, *cell_frame;
  float* cell_origin;
  float* vert32;
  Node* nodes;
  Tri* tris;
  BvhScratch bvh;
  int32_t* order;
  void* order_scratch;
  unsigned* cell_bounds;
  int* work;
  double2 *azim_cs, *elev_cs;
  double* svf_lattice;
  DomainDesc* dom;
  unsigned long long* counters;
  int* err;
};

StaticBuffers lay_out(Layout& L, long long ncell, long long nvert, long long max_tri,
                      long long num_azimuths) {
  StaticBuffers b;
  std::memset(&b, 0, sizeof(b));
  const long long max_mv = ncell + nvert;
  const long long nt = max_tri > 0 ? max_tri : 1;
  b.packed = L.take<unsigned long long>(nvert);
  b.offsets = L.take<unsigned long long>(nvert);
  b.scan_partials = L.take<unsigned long long>(scan_partials(nvert));
  b.totals = L.take<unsigned long long>(4);
  b.vot = L.take<int>(3 * max_tri);
  b.add_lon = L.take<double>(nvert);
  b.add_lat = L.take<double>(nvert);
  b.add_h = L.take<double>(nvert);
  b.ecef = L.take<double>(3 * max_mv);
  b.block_sums = L.take<double>(3 * (size_t)ecef_blocks((int)max_mv));
  b.origin_sum = L.take<double>(4);
  b.vert32 = L.take<float>(3 * max_mv);
  b.cell_enu = L.take<double>(3 * ncell);
  b.cell_frame = L.take<double>(9 * ncell);
  b.cell_origin = L.take<float>(6 * ncell);
  b.nodes = L.take<Node>(nt > 1 ? nt - 1 : 1);
  b.tris = L.take<Tri>(nt);
  b.bvh.keys = L.take<uint32_t>(nt);
  b.bvh.vals = L.take<int32_t>(nt);
  b.bvh.keys_alt = L.take<uint32_t>(nt);
  b.bvh.vals_alt = L.take<int32_t>(nt);
  b.bvh.cxy = L.take<float2>(nt);
  b.bvh.parent = L.take<int>(nt);
  b.bvh.nsize = L.take<int>(nt);
  b.bvh.counter = L.take<int>(nt);
  b.bvh.bounds = L.take<unsigned>(16);
  b.bvh.sort_scratch = L.take<char>(radix_scratch_u32(nt));
  b.order = L.take<int32_t>(ncell);
  b.order_scratch = L.take<char>(cell_order_scratch_bytes(ncell));
  b.cell_bounds = L.take<unsigned>(8);
  b.work = L.take<int>(4);
  b.azim_cs = L.take<double2>(num_azimuths);
  b.elev_cs = L.take<double2>(kElevTable);
  b.svf_lattice = L.take<double>(kSvfTable);
  b.dom = L.take<DomainDesc>(1);
  b.counters = L.take<unsigned long long>(kCounterWords);
  b.err = L.take<int>(4);
  return b;
}

inline double deg2rad_s(double a) { return ((a / 180.0) * kPi); }

}  // namespace

// Forgets the cached device address of the array on `device` (-1: all): a
// device reset reloads the module and may place the array elsewhere, so the
// next call resolves the address again.
void static_forget_device(int device) {
  std::lock_guard<std::mutex> lock(g_static_mu);
  for (int d = 0; d < 128; d++)
    if (device < 0 || d == device) g_static_addr[d] = nullptr;
}

}  // namespace hz

using namespace hz;

extern "C" int hz_horizon_svf_device_static(
    const double* clon, const double* clat, const double* hsurf, const double* vlon,
    const double* vlat, const int32_t* cells_of_vertex, double* horizon, double* skyview,
    int num_cell, int num_vertex, int num_hori, int grid_type, double dist_search,
    double ray_org_elev, int refine_factor, int svf_type, void* stream) {
  set_last_error("");
  // Argument checks of horizon_svf.pyx:91-103.
  if (num_cell < 1 || num_vertex < 0) return static_fail(HZ_ERR_VALUE, "invalid array sizes");
  if ((num_hori < 4) || (num_hori > 1440))
    return static_fail(HZ_ERR_VALUE, "'num_hori' must be in the range [4, 1440]");
  if ((grid_type < 0) || (grid_type > 1))
    return static_fail(HZ_ERR_VALUE, "'grid_type' must be in the range [0, 1]");
  if (!(dist_search >= 1000.0) || !(dist_search <= 500000.0))
    return static_fail(HZ_ERR_VALUE, "'dist_search' must be in the range [1'000, 500'000] km");
  if (!(ray_org_elev >= 0.1))
    return static_fail(HZ_ERR_TYPE, "Minimal allowed value for 'ray_org_elev' is 0.1 m");
  if ((refine_factor < 1) || (refine_factor > 50))
    return static_fail(HZ_ERR_VALUE, "'refine_factor' must be in the range [1, 50]");
  if ((svf_type < 0) || (svf_type > 2))
    return static_fail(HZ_ERR_VALUE, "'svf_type' must be in the range [0, 2]");

  const long long max_tri = (long long)(grid_type == 0 ? 4 : 6) * num_vertex;
  Layout dry{nullptr};
  const long long num_azimuths = (long long)num_hori * refine_factor;
  lay_out(dry, num_cell, num_vertex, max_tri, num_azimuths);
  if (dry.off > kStaticScratchBytes) {
    char buf[320];
    snprintf(buf, sizeof(buf),
             "domain needs %zu bytes of scratch, above the fixed %zu-byte static array "
             "(about 90,000 cells with grid_type 1, 120,000 with grid_type 0, at one "
             "vertex per two cells); use hz_horizon_svf_device",
             dry.off, kStaticScratchBytes);
    set_last_error(buf);
    return HZ_ERR_VALUE;
  }

  std::lock_guard<std::mutex> lock(g_static_mu);
  int dev = 0;
  HZ_STATIC_CUDA(cudaGetDevice(&dev), "cudaGetDevice failed");
  if (dev < 0 || dev >= 128) return static_fail(HZ_ERR_VALUE, "unsupported device ordinal");
  if (!g_static_addr[dev]) {
    void* ptr = nullptr;
    HZ_STATIC_CUDA(cudaGetSymbolAddress(&ptr, g_static_scratch),
                   "cudaGetSymbolAddress of the static scratch failed");
    g_static_addr[dev] = ptr;
  }
  cudaStream_t s = (cudaStream_t)stream;
  Layout lay{(char*)g_static_addr[dev]};
  const StaticBuffers b = lay_out(lay, num_cell, num_vertex, max_tri, num_azimuths);
  // From the first queued operation on, every return waits for the stream
  // (still under the lock), so that no work of a failed call can overlap the
  // next call's use of the array.
  struct DrainOnReturn {
    cudaStream_t s;
    ~DrainOnReturn() { (void)cudaStreamSynchronize(s); }
  } drain{s};

  // Cleared every call: the array keeps the previous call's contents.
  HZ_STATIC_CUDA(cudaMemsetAsync(b.err, 0, 4 * sizeof(int), s), "clearing error word");
  HZ_STATIC_CUDA(cudaMemsetAsync(b.counters, 0, kCounterWords * sizeof(unsigned long long), s),
                 "clearing counters");

  // Mesh (mo_lradtopo_horayzon.cpp:228-317).
  unsigned long long totals = 0;
  int err = 0;
  HZ_STATIC_CUDA(mesh_count(cells_of_vertex, num_vertex, num_cell, grid_type, b.packed, b.err, s),
                 "mesh count");
  if (num_vertex > 0) {
    HZ_STATIC_CUDA(scan_exclusive_u64(b.packed, b.offsets, num_vertex, b.totals, b.scan_partials,
                                      s), "mesh scan");
    HZ_STATIC_CUDA(cudaMemcpyAsync(&totals, b.totals, sizeof(totals), cudaMemcpyDeviceToHost, s),
                   "reading mesh totals");
  }
  HZ_STATIC_CUDA(cudaMemcpyAsync(&err, b.err, sizeof(int), cudaMemcpyDeviceToHost, s),
                 "reading error word");
  HZ_STATIC_CUDA(cudaStreamSynchronize(s), "mesh count");
  if (err & kErrBadIndex)
    return static_fail(HZ_ERR_INDEX, "Indices of 'cells_of_vertex' out of range");
  const int n_tri = (int)(totals & 0xFFFFFFFFull);
  const int nadd = (int)(totals >> 32);
  const int nmv = num_cell + nadd;
  HZ_STATIC_CUDA(mesh_emit(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_vertex, num_cell,
                           grid_type, b.offsets, b.vot, b.add_lon, b.add_lat, b.add_h, s),
                 "mesh emission");

  // Frames (cpp:611-644).
  double sum[3] = {0.0, 0.0, 0.0};
  HZ_STATIC_CUDA(mesh_ecef(clon, clat, hsurf, b.add_lon, b.add_lat, b.add_h, num_cell, nadd,
                           b.ecef, b.block_sums, b.origin_sum, s), "ECEF");
  HZ_STATIC_CUDA(cudaMemcpyAsync(sum, b.origin_sum, sizeof(sum), cudaMemcpyDeviceToHost, s),
                 "reading the ECEF sum");
  HZ_STATIC_CUDA(cudaStreamSynchronize(s), "ECEF");
  const Frame fr = enu_frame_from_sum(sum[0], sum[1], sum[2]);
  HZ_STATIC_CUDA(mesh_enu(b.ecef, nmv, num_cell, fr, b.vert32, b.cell_enu, nullptr, s), "ENU");

  // BVH and search (cpp:395-432, 651-761).
  HZ_STATIC_CUDA(bvh_build(b.vert32, b.vot, n_tri, b.nodes, b.tris, b.bvh, s), "BVH build");
  const int L = num_hori * refine_factor;
  double azim_shift = 0.0;
  if (refine_factor != 1)
    azim_shift = -(deg2rad_s(360.0) / (2.0 * num_hori)) + (deg2rad_s(360.0) / (2.0 * (double)L));
  DomainDesc D;
  std::memset(&D, 0, sizeof(D));
  D.cell_enu = b.cell_enu;
  D.cell_frame = b.cell_frame;
  D.cell_origin = b.cell_origin;
  D.nodes = b.nodes;
  D.tris = b.tris;
  D.horizon = horizon;
  D.skyview = skyview;
  D.azim_cs = b.azim_cs;
  D.elev_cs = b.elev_cs;
  D.svf_lattice = b.svf_lattice;
  D.centre = fr.centre;
  D.pole = fr.pole;
  D.ray_org_elev = ray_org_elev;
  D.hori_acc = deg2rad_s(0.25);
  D.two_ha = 2.0 * D.hori_acc;
  D.elev_floor = deg2rad_s(-85.0);
  D.cell_offset = 0;
  D.groups = 1;
  D.item_begin = 0;
  D.occ_cache = 1;
  D.root = n_tri > 0 ? 0 : kEmptyRef;
  D.n_tri = n_tri;
  D.ncell = num_cell;
  D.ncell_traced = num_cell;
  D.nhori = num_hori;
  D.refine = refine_factor;
  D.L = L;
  D.svf_type = svf_type;
  D.tfar = (float)dist_search;
  // Pageable source: the copy has finished with `D` when the call returns.
  HZ_STATIC_CUDA(cudaMemcpyAsync(b.dom, &D, sizeof(D), cudaMemcpyHostToDevice, s),
                 "search descriptor");
  HZ_STATIC_CUDA(cell_order(b.cell_enu, nullptr, 0, num_cell, 0, num_cell, 0, b.order,
                            b.order_scratch, b.cell_bounds,
                            b.work, s), "cell order");
  HZ_STATIC_CUDA(trace_tables(b.azim_cs, b.elev_cs, b.svf_lattice, L, azim_shift, D.hori_acc,
                              D.svf_type, s), "lattice tables");
  const TraceKnobs knobs{kDefaultAdvanceMin, kDefaultLeafMin, kDefaultChunk, kTraceBinary};
  HZ_STATIC_CUDA(trace_flat(b.dom, 1, b.order, num_cell, num_cell, b.work, b.counters, b.err,
                            knobs, false, false, s), "horizon search");
  HZ_STATIC_CUDA(cudaMemcpyAsync(&err, b.err, sizeof(int), cudaMemcpyDeviceToHost, s),
                 "reading error word");
  HZ_STATIC_CUDA(cudaStreamSynchronize(s), "horizon search");
  if (err & kErrStack) return static_fail(HZ_ERR_INTERNAL, "BVH traversal stack overflow");
  if (err & kErrBounds) return static_fail(HZ_ERR_INTERNAL, "bounds check failed in the search");
  return HZ_OK;
}
