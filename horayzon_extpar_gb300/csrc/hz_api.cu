// hz_api.cu -- the C ABI (include/horayzon_gb300.h) and the per-device engine
// that runs mesh assembly, geodetic frames, LBVH build and horizon search.
//
// Pipeline of one call (mo_lradtopo_horayzon.cpp:562-785):
//   mesh_count -> scan -> [read totals, check indices] -> mesh_emit ->
//   mesh_ecef -> [read cell ECEF sum] -> frame on the host (glibc, same
//   expressions as cpp:624-644) -> mesh_enu -> bvh_build -> trace -> counters.
// Device memory comes from one grow-only arena per device, carved per call.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <mutex>
#include <string>

#include "../../include/horayzon_gb300.h"
#include "hz_internal.h"

namespace hz {
namespace {

thread_local std::string g_last_error;
thread_local long long g_launches = 0;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define HZ_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(HZ_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
  } while (0)

inline double deg2rad(double a) { return ((a / 180.0) * kPi); }
inline double rad2deg(double a) { return ((a / kPi) * 180.0); }

// Bump allocator over the arena; with base == nullptr it only measures.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base((char*)b) {}
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += sizeof(T) * (n ? n : 1);
    return p;
  }
};

struct Sizes {
  long long ncell, nvert, nhori;
  long long max_tri, max_mv;
  bool host_io;
};

struct Buffers {
  // host-entry staging of inputs/outputs
  double *clon, *clat, *hsurf, *vlon, *vlat;
  int* cov;
  double *horizon, *skyview;
  // mesh
  unsigned long long *packed, *offsets, *scan_partials, *totals;
  int* vot;
  double *add_lon, *add_lat, *add_h;
  double *ecef, *block_sums, *origin_sum;
  float* vert32;
  double* cell_enu;
  // BVH
  Node* nodes;
  Tri* tris;
  BvhScratch bvh;
  // cell order of the persistent search
  int32_t* order;
  void* order_scratch;
  unsigned* cell_bounds;
  int* work;
  double2 *azim_cs, *elev_cs;
  double* sin_lattice;
  // misc
  unsigned long long* counters;  // rays, node visits, triangle tests
  int* err;
};

Buffers carve(Carver& c, const Sizes& s) {
  Buffers b;
  std::memset(&b, 0, sizeof(b));
  if (s.host_io) {
    b.clon = c.take<double>(s.ncell);
    b.clat = c.take<double>(s.ncell);
    b.hsurf = c.take<double>(s.ncell);
    b.vlon = c.take<double>(s.nvert);
    b.vlat = c.take<double>(s.nvert);
    b.cov = c.take<int>(6 * s.nvert);
    b.horizon = c.take<double>(s.nhori * s.ncell);
    b.skyview = c.take<double>(s.ncell);
  }
  b.packed = c.take<unsigned long long>(s.nvert);
  b.offsets = c.take<unsigned long long>(s.nvert);
  b.scan_partials = c.take<unsigned long long>(scan_partials(s.nvert));
  b.totals = c.take<unsigned long long>(4);
  b.vot = c.take<int>(3 * s.max_tri);
  b.add_lon = c.take<double>(s.nvert);
  b.add_lat = c.take<double>(s.nvert);
  b.add_h = c.take<double>(s.nvert);
  b.ecef = c.take<double>(3 * s.max_mv);
  b.block_sums = c.take<double>(3 * (size_t)ecef_blocks((int)s.max_mv));
  b.origin_sum = c.take<double>(4);
  b.vert32 = c.take<float>(3 * s.max_mv);
  b.cell_enu = c.take<double>(3 * s.ncell);
  long long nn = s.max_tri > 1 ? s.max_tri - 1 : 1;
  b.nodes = c.take<Node>(nn);
  b.tris = c.take<Tri>(s.max_tri);
  long long nt = s.max_tri > 0 ? s.max_tri : 1;
  b.bvh.keys = c.take<uint32_t>(nt);
  b.bvh.vals = c.take<int32_t>(nt);
  b.bvh.keys_alt = c.take<uint32_t>(nt);
  b.bvh.vals_alt = c.take<int32_t>(nt);
  b.bvh.cxy = c.take<float2>(nt);
  b.bvh.parent = c.take<int>(nt);
  b.bvh.nsize = c.take<int>(nt);
  b.bvh.counter = c.take<int>(nt);
  b.bvh.bounds = c.take<unsigned>(16);
  b.bvh.sort_scratch = c.take<char>(radix_scratch_u32(nt));
  b.order = c.take<int32_t>(s.ncell);
  b.order_scratch = c.take<char>(cell_order_scratch_bytes(s.ncell));
  b.cell_bounds = c.take<unsigned>(8);
  b.work = c.take<int>(4);
  b.azim_cs = c.take<double2>(s.nhori * 50);  // L <= num_hori * max refine_factor
  b.elev_cs = c.take<double2>(kElevTable);
  b.sin_lattice = c.take<double>(kSinTable);
  b.counters = c.take<unsigned long long>(4);
  b.err = c.take<int>(4);
  return b;
}

struct Engine {
  int device = -1;
  std::mutex mu;
  void* arena = nullptr;
  size_t cap = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  unsigned long long* pinned = nullptr;  // small readbacks

  int init(int dev) {
    device = dev;
    HZ_CUDA(cudaSetDevice(dev));
    HZ_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto& e : ev) HZ_CUDA(cudaEventCreate(&e));
    HZ_CUDA(cudaMallocHost((void**)&pinned, 64 * sizeof(unsigned long long)));
    return HZ_OK;
  }

  int reserve(size_t bytes, cudaStream_t s) {
    if (bytes <= cap) return HZ_OK;
    HZ_CUDA(cudaStreamSynchronize(s));
    if (arena) HZ_CUDA(cudaFree(arena));
    arena = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&arena, want);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      arena = nullptr;
      return fail(HZ_ERR_CUDA, "cudaMalloc of %zu bytes failed: %s", want,
                  cudaGetErrorString(e));
    }
    cap = want;
    return HZ_OK;
  }

  void release() {
    if (arena) cudaFree(arena);
    arena = nullptr;
    cap = 0;
  }
};

std::mutex g_engines_mu;
Engine* g_engines[128] = {};

int get_engine(int device, Engine** out) {
  int dev = device;
  if (dev < 0) HZ_CUDA(cudaGetDevice(&dev));
  int count = 0;
  HZ_CUDA(cudaGetDeviceCount(&count));
  if (dev >= count || dev >= 128) return fail(HZ_ERR_VALUE, "invalid CUDA device %d", dev);
  std::lock_guard<std::mutex> lock(g_engines_mu);
  if (!g_engines[dev]) {
    Engine* e = new Engine();
    int rc = e->init(dev);
    if (rc != HZ_OK) {
      delete e;
      return rc;
    }
    g_engines[dev] = e;
  }
  *out = g_engines[dev];
  return HZ_OK;
}

// horizon_svf.pyx:79-103 (array-length checks are the callers': the C ABI
// receives lengths, not arrays).
int validate(int num_cell, int num_vertex, int num_hori, int grid_type, double dist_search,
             double ray_org_elev, int refine_factor, int svf_type) {
  if (num_cell < 1) return fail(HZ_ERR_VALUE, "'num_cell' must be at least 1");
  if (num_vertex < 0) return fail(HZ_ERR_VALUE, "'num_vertex' must not be negative");
  if ((num_hori < 4) || (num_hori > 1440))
    return fail(HZ_ERR_VALUE, "'num_hori' must be in the range [4, 1440]");
  if ((grid_type < 0) || (grid_type > 1))
    return fail(HZ_ERR_VALUE, "'grid_type' must be in the range [0, 1]");
  if (!(dist_search >= 1000.0) || !(dist_search <= 500000.0))
    return fail(HZ_ERR_VALUE, "'dist_search' must be in the range [1'000, 500'000] km");
  if (!(ray_org_elev >= 0.1))
    return fail(HZ_ERR_TYPE, "Minimal allowed value for 'ray_org_elev' is 0.1 m");
  if ((refine_factor < 1) || (refine_factor > 50))
    return fail(HZ_ERR_VALUE, "'refine_factor' must be in the range [1, 50]");
  if ((svf_type < 0) || (svf_type > 2))
    return fail(HZ_ERR_VALUE, "'svf_type' must be in the range [0, 2]");
  if ((long long)num_hori * (long long)num_cell > (1LL << 40))
    return fail(HZ_ERR_VALUE, "output too large");
  if (num_vertex > (1 << 27))
    return fail(HZ_ERR_VALUE, "'num_vertex' above the supported maximum of 2^27");
  return HZ_OK;
}

// mo_lradtopo_horayzon.cpp:624-644 on the host, from the device sum of the
// cells' ECEF coordinates.
Frame make_frame(double xo, double yo, double zo) {
  const double R = kEarthRadius;
  Frame f;
  double radius = sqrt(xo * xo + yo * yo + zo * zo);
  double lon_o = atan2(yo, xo);
  double lat_o = asin(zo / radius);
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
    double dx = x - f.xe, dy = y - f.ye, dz = z - f.ze;
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

struct Problem {
  const double *clon, *clat, *hsurf, *vlon, *vlat;
  const int* cov;
  double *horizon, *skyview;
  int ncell, nvert, nhori, grid_type;
  double dist_search, ray_org_elev;
  int refine, svf_type;
};

enum class Stop { kMesh, kEnu, kFull };

// Runs the pipeline on device pointers in `pr`. With stop != kFull it ends
// after the mesh (or ENU) stage and leaves results in `b`.
int run_pipeline(Engine& E, const Problem& pr, const Buffers& b, cudaStream_t s,
                 const hz_options& opt, hz_stats* st, Stop stop, int* n_tri_out,
                 int* n_mv_out) {
  auto t0 = std::chrono::steady_clock::now();
  g_launches = 0;
  HZ_CUDA(cudaMemsetAsync(b.err, 0, 4 * sizeof(int), s));
  HZ_CUDA(cudaMemsetAsync(b.counters, 0, 4 * sizeof(unsigned long long), s));
  HZ_CUDA(cudaEventRecord(E.ev[0], s));

  // ---- mesh (cpp:228-317) ----
  HZ_CUDA(mesh_count(pr.cov, pr.nvert, pr.ncell, pr.grid_type, b.packed, b.err, s));
  if (pr.nvert > 0) {
    HZ_CUDA(scan_exclusive_u64(b.packed, b.offsets, pr.nvert, b.totals, b.scan_partials, s));
    HZ_CUDA(cudaMemcpyAsync(E.pinned, b.totals, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, s));
  } else {
    E.pinned[0] = 0;
  }
  HZ_CUDA(cudaMemcpyAsync(E.pinned + 1, b.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  const int err0 = (int)(E.pinned[1] & 0xFFFFFFFFull);
  if (err0 & kErrBadIndex) return fail(HZ_ERR_INDEX, "Indices of 'cells_of_vertex' out of range");
  const unsigned long long tot = E.pinned[0];
  const int n_tri = (int)(tot & 0xFFFFFFFFull);
  const int nadd = (int)(tot >> 32);
  const int nmv = pr.ncell + nadd;
  *n_tri_out = n_tri;
  *n_mv_out = nmv;
  if (opt.verbose) {
    printf("Build triangle mesh from ICON grid cell circumcenters%s\n",
           pr.grid_type == 0 ? "\n (non-unique triangulation)"
                             : " and vertices\n (unique triangulation)");
    printf("Number of triangles in mesh: %d\n", n_tri);
  }
  HZ_CUDA(mesh_emit(pr.clon, pr.clat, pr.hsurf, pr.vlon, pr.vlat, pr.cov, pr.nvert, pr.ncell,
                    pr.grid_type, b.offsets, b.vot, b.add_lon, b.add_lat, b.add_h, s));
  if (stop == Stop::kMesh) return HZ_OK;

  // ---- frames (cpp:611-644) ----
  HZ_CUDA(mesh_ecef(pr.clon, pr.clat, pr.hsurf, b.add_lon, b.add_lat, b.add_h, pr.ncell, nadd,
                    b.ecef, b.block_sums, b.origin_sum, s));
  HZ_CUDA(cudaMemcpyAsync(E.pinned + 2, b.origin_sum, 3 * sizeof(double),
                          cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  double so[3];
  std::memcpy(so, E.pinned + 2, sizeof(so));
  const Frame fr = make_frame(so[0], so[1], so[2]);
  if (opt.verbose) {
    double radius = sqrt(so[0] * so[0] + so[1] * so[1] + so[2] * so[2]);
    printf("Origin of ENU coordinate system: %.4f deg lat, %.4f deg lon\n",
           rad2deg(asin(so[2] / radius)), rad2deg(atan2(so[1], so[0])));
  }
  HZ_CUDA(mesh_enu(b.ecef, nmv, pr.ncell, fr, b.vert32, b.cell_enu, s));
  HZ_CUDA(cudaEventRecord(E.ev[1], s));
  if (stop == Stop::kEnu) return HZ_OK;

  // ---- BVH (cpp:395-432) ----
  HZ_CUDA(bvh_build(b.vert32, b.vot, n_tri, b.nodes, b.tris, b.bvh, s));
  HZ_CUDA(cudaEventRecord(E.ev[2], s));

  // ---- horizon + SVF (cpp:651-761) ----
  TraceParams p;
  std::memset(&p, 0, sizeof(p));
  p.cell_enu = b.cell_enu;
  p.ncell = pr.ncell;
  p.cell_begin = 0;
  p.cell_count = pr.ncell;
  if (opt.cell_count > 0) {
    if (opt.cell_begin < 0 || (long long)opt.cell_begin + opt.cell_count > pr.ncell)
      return fail(HZ_ERR_VALUE, "cell range [%d, %d) outside [0, %d)", opt.cell_begin,
                  opt.cell_begin + opt.cell_count, pr.ncell);
    p.cell_begin = opt.cell_begin;
    p.cell_count = opt.cell_count;
  }
  p.nodes = b.nodes;
  p.tris = b.tris;
  p.root = n_tri > 0 ? 0 : kEmptyRef;
  p.centre = fr.centre;
  p.pole = fr.pole;
  p.ray_org_elev = pr.ray_org_elev;
  p.tfar = (float)pr.dist_search;
  p.nhori = pr.nhori;
  p.refine = pr.refine;
  p.L = pr.nhori * pr.refine;
  p.svf_type = pr.svf_type;
  p.hori_acc = deg2rad(0.25);
  p.elev_floor = deg2rad(opt.elev_floor_deg);
  p.azim_sin = sin(deg2rad(360.0) / (double)p.L);
  p.azim_cos = cos(deg2rad(360.0) / (double)p.L);
  p.elev_sin_2ha = sin(2.0 * p.hori_acc);
  p.elev_cos_2ha = cos(2.0 * p.hori_acc);
  double azim_shift = 0.0;
  if (pr.refine != 1)
    azim_shift = -(deg2rad(360.0) / (2.0 * pr.nhori)) + (deg2rad(360.0) / (2.0 * (double)p.L));
  p.shift_sin = sin(-azim_shift);
  p.shift_cos = cos(-azim_shift);
  p.horizon = pr.horizon;
  p.skyview = pr.skyview;
  p.counters = b.counters;
  p.err = b.err;
  if (opt.kernel == HZ_KERNEL_PER_CELL) {
    HZ_CUDA(trace_exact(p, opt.count_work != 0, s));
  } else {
    const int adv = opt.advance_min >= 1 && opt.advance_min <= 32 ? opt.advance_min : 16;
    HZ_CUDA(trace_tables(b.azim_cs, b.elev_cs, b.sin_lattice, p.L, azim_shift, p.hori_acc, s));
    p.azim_cs = b.azim_cs;
    p.elev_cs = b.elev_cs;
    p.sin_lattice = b.sin_lattice;
    HZ_CUDA(cell_order(b.cell_enu, p.cell_begin, p.cell_count, b.order, b.order_scratch,
                       b.cell_bounds, b.work, s));
    HZ_CUDA(trace_flat(p, b.order, b.work, adv, opt.count_work != 0, s));
  }
  HZ_CUDA(cudaEventRecord(E.ev[3], s));

  HZ_CUDA(cudaMemcpyAsync(E.pinned + 8, b.counters, 3 * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaMemcpyAsync(E.pinned + 12, b.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  const int err1 = (int)(E.pinned[12] & 0xFFFFFFFFull);
  if (err1 & kErrStack) return fail(HZ_ERR_INTERNAL, "BVH traversal stack overflow");
  if (st) {
    st->kernel_launches = g_launches;
    st->num_rays = (int64_t)E.pinned[8];
    st->node_visits = (int64_t)E.pinned[9];
    st->tri_tests = (int64_t)E.pinned[10];
    st->n_tri = n_tri;
    st->n_mesh_vert = nmv;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, E.ev[0], E.ev[1]);
    st->ms_mesh = ms;
    cudaEventElapsedTime(&ms, E.ev[1], E.ev[2]);
    st->ms_bvh = ms;
    cudaEventElapsedTime(&ms, E.ev[2], E.ev[3]);
    st->ms_trace = ms;
  }
  if (opt.verbose) {
    printf("Number of rays shot: %lld\n", (long long)E.pinned[8]);
    printf("Average number of rays per cell and azimuth sector: %.2f\n",
           (double)E.pinned[8] / ((double)pr.ncell * (double)pr.nhori));
  }
  (void)t0;
  return HZ_OK;
}

hz_options resolve(const hz_options* opt) {
  hz_options o;
  hz_default_options(&o);
  if (opt) {
    // Accept older, shorter option structs.
    size_t n = opt->size > 0 && (size_t)opt->size < sizeof(o) ? (size_t)opt->size : sizeof(o);
    std::memcpy(&o, opt, n);
    o.size = sizeof(o);
  }
  return o;
}

}  // namespace

void note_launches(int n) { g_launches += n; }

void set_last_error(const char* msg) { g_last_error = msg; }

}  // namespace hz

using namespace hz;

extern "C" {

void hz_default_options(hz_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->size = sizeof(hz_options);
  opt->device = -1;
  opt->elev_floor_deg = -85.0;
}

const char* hz_last_error(void) { return g_last_error.c_str(); }

int hz_version(void) { return HZ_VERSION; }

int hz_release_workspace(int device) {
  std::lock_guard<std::mutex> lock(g_engines_mu);
  for (int d = 0; d < 128; d++) {
    if ((device < 0 || d == device) && g_engines[d]) {
      std::lock_guard<std::mutex> l2(g_engines[d]->mu);
      cudaSetDevice(d);
      g_engines[d]->release();
    }
  }
  return HZ_OK;
}

int hz_horizon_svf_device(const double* clon, const double* clat, const double* hsurf,
                          const double* vlon, const double* vlat,
                          const int32_t* cells_of_vertex, double* horizon, double* skyview,
                          int num_cell, int num_vertex, int num_hori, int grid_type,
                          double dist_search, double ray_org_elev, int refine_factor,
                          int svf_type, void* stream, const hz_options* opt_in,
                          hz_stats* stats) {
  g_last_error.clear();
  auto t0 = std::chrono::steady_clock::now();
  hz_options opt = resolve(opt_in);
  int rc = validate(num_cell, num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
                    refine_factor, svf_type);
  if (rc) return rc;
  Engine* E = nullptr;
  rc = get_engine(opt.device, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  HZ_CUDA(cudaSetDevice(E->device));
  cudaStream_t s = (cudaStream_t)stream;
  Sizes sz{num_cell, num_vertex, num_hori,
           (long long)(grid_type == 0 ? 4 : 6) * num_vertex,
           (long long)num_cell + num_vertex, false};
  Carver dry(nullptr);
  carve(dry, sz);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  Buffers b = carve(c, sz);
  Problem pr{clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon, skyview,
             num_cell, num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
             refine_factor, svf_type};
  if (stats) std::memset(stats, 0, sizeof(*stats));
  int ntri = 0, nmv = 0;
  rc = run_pipeline(*E, pr, b, s, opt, stats, Stop::kFull, &ntri, &nmv);
  if (rc) return rc;
  if (stats)
    stats->ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return HZ_OK;
}

int hz_horizon_svf(const double* clon, const double* clat, const double* hsurf,
                   const double* vlon, const double* vlat, const int32_t* cells_of_vertex,
                   double* horizon, double* skyview, int num_cell, int num_vertex,
                   int num_hori, int grid_type, double dist_search, double ray_org_elev,
                   int refine_factor, int svf_type, const hz_options* opt_in,
                   hz_stats* stats) {
  g_last_error.clear();
  auto t0 = std::chrono::steady_clock::now();
  hz_options opt = resolve(opt_in);
  int rc = validate(num_cell, num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
                    refine_factor, svf_type);
  if (rc) return rc;
  if (!clon || !clat || !hsurf || !horizon || !skyview ||
      (num_vertex > 0 && (!vlon || !vlat || !cells_of_vertex)))
    return fail(HZ_ERR_VALUE, "null array pointer");
  Engine* E = nullptr;
  rc = get_engine(opt.device, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  HZ_CUDA(cudaSetDevice(E->device));
  cudaStream_t s = E->stream;
  Sizes sz{num_cell, num_vertex, num_hori,
           (long long)(grid_type == 0 ? 4 : 6) * num_vertex,
           (long long)num_cell + num_vertex, true};
  Carver dry(nullptr);
  carve(dry, sz);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  Buffers b = carve(c, sz);
  const size_t nc = (size_t)num_cell, nv = (size_t)num_vertex;
  HZ_CUDA(cudaEventRecord(E->ev[4], s));
  HZ_CUDA(cudaMemcpyAsync(b.clon, clon, nc * 8, cudaMemcpyHostToDevice, s));
  HZ_CUDA(cudaMemcpyAsync(b.clat, clat, nc * 8, cudaMemcpyHostToDevice, s));
  HZ_CUDA(cudaMemcpyAsync(b.hsurf, hsurf, nc * 8, cudaMemcpyHostToDevice, s));
  if (nv) {
    HZ_CUDA(cudaMemcpyAsync(b.vlon, vlon, nv * 8, cudaMemcpyHostToDevice, s));
    HZ_CUDA(cudaMemcpyAsync(b.vlat, vlat, nv * 8, cudaMemcpyHostToDevice, s));
    HZ_CUDA(cudaMemcpyAsync(b.cov, cells_of_vertex, nv * 6 * 4, cudaMemcpyHostToDevice, s));
  }
  HZ_CUDA(cudaEventRecord(E->ev[5], s));
  Problem pr{b.clon, b.clat, b.hsurf, b.vlon, b.vlat, b.cov, b.horizon, b.skyview,
             num_cell, num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
             refine_factor, svf_type};
  if (stats) std::memset(stats, 0, sizeof(*stats));
  int ntri = 0, nmv = 0;
  rc = run_pipeline(*E, pr, b, s, opt, stats, Stop::kFull, &ntri, &nmv);
  if (rc) return rc;
  HZ_CUDA(cudaEventRecord(E->ev[6], s));
  if (opt.cell_count > 0) {
    // Only the traced columns: the caller's other entries stay untouched.
    const size_t c0 = (size_t)opt.cell_begin, cn = (size_t)opt.cell_count;
    HZ_CUDA(cudaMemcpy2DAsync(horizon + c0, nc * 8, b.horizon + c0, nc * 8, cn * 8,
                              (size_t)num_hori, cudaMemcpyDeviceToHost, s));
    HZ_CUDA(cudaMemcpyAsync(skyview + c0, b.skyview + c0, cn * 8, cudaMemcpyDeviceToHost, s));
  } else {
    HZ_CUDA(cudaMemcpyAsync(horizon, b.horizon, (size_t)num_hori * nc * 8,
                            cudaMemcpyDeviceToHost, s));
    HZ_CUDA(cudaMemcpyAsync(skyview, b.skyview, nc * 8, cudaMemcpyDeviceToHost, s));
  }
  HZ_CUDA(cudaEventRecord(E->ev[7], s));
  HZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, E->ev[4], E->ev[5]);
    stats->ms_h2d = ms;
    cudaEventElapsedTime(&ms, E->ev[6], E->ev[7]);
    stats->ms_d2h = ms;
    stats->ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return HZ_OK;
}

void horizon_svf_comp(double* clon, double* clat, double* hsurf, double* vlon, double* vlat,
                      int* cells_of_vertex, double* horizon, double* skyview, int num_cell,
                      int num_vertex, int num_hori, int grid_type, double dist_search,
                      double ray_org_elev, int refine_factor, int svf_type) {
  hz_options opt;
  hz_default_options(&opt);
  const char* v = getenv("HZ_VERBOSE");
  opt.verbose = v && v[0] == '1';
  int rc = hz_horizon_svf(clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon, skyview,
                          num_cell, num_vertex, num_hori, grid_type, dist_search,
                          ray_org_elev, refine_factor, svf_type, &opt, nullptr);
  if (rc != HZ_OK) {
    fprintf(stderr, "horizon_svf_comp: %s\n", hz_last_error());
    if (horizon && skyview && num_cell > 0 && num_hori > 0) {
      for (long long k = 0; k < (long long)num_hori * num_cell; k++) horizon[k] = NAN;
      for (int k = 0; k < num_cell; k++) skyview[k] = NAN;
    }
  }
}

static int mesh_host_common(const double* clon, const double* clat, const double* hsurf,
                            const double* vlon, const double* vlat, const int32_t* cov,
                            int num_cell, int num_vertex, int grid_type, int device,
                            bool want_enu, double* mesh_lon, double* mesh_lat,
                            double* mesh_h, float* enu32, int cap_vert, int32_t* vot,
                            int cap_tri, int* n_mesh_vert, int* n_tri) {
  g_last_error.clear();
  if (num_cell < 1 || num_vertex < 0 || grid_type < 0 || grid_type > 1)
    return fail(HZ_ERR_VALUE, "invalid mesh arguments");
  Engine* E = nullptr;
  int rc = get_engine(device, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  HZ_CUDA(cudaSetDevice(E->device));
  cudaStream_t s = E->stream;
  Sizes sz{num_cell, num_vertex, 4, (long long)(grid_type == 0 ? 4 : 6) * num_vertex,
           (long long)num_cell + num_vertex, true};
  Carver dry(nullptr);
  carve(dry, sz);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  Buffers b = carve(c, sz);
  const size_t nc = (size_t)num_cell, nv = (size_t)num_vertex;
  HZ_CUDA(cudaMemcpyAsync(b.clon, clon, nc * 8, cudaMemcpyHostToDevice, s));
  HZ_CUDA(cudaMemcpyAsync(b.clat, clat, nc * 8, cudaMemcpyHostToDevice, s));
  HZ_CUDA(cudaMemcpyAsync(b.hsurf, hsurf, nc * 8, cudaMemcpyHostToDevice, s));
  if (nv) {
    HZ_CUDA(cudaMemcpyAsync(b.vlon, vlon, nv * 8, cudaMemcpyHostToDevice, s));
    HZ_CUDA(cudaMemcpyAsync(b.vlat, vlat, nv * 8, cudaMemcpyHostToDevice, s));
    HZ_CUDA(cudaMemcpyAsync(b.cov, cov, nv * 6 * 4, cudaMemcpyHostToDevice, s));
  }
  Problem pr{b.clon, b.clat, b.hsurf, b.vlon, b.vlat, b.cov, b.horizon, b.skyview,
             num_cell, num_vertex, 4, grid_type, 1e4, 1.0, 1, 0};
  hz_options opt;
  hz_default_options(&opt);
  int ntri = 0, nmv = 0;
  rc = run_pipeline(*E, pr, b, s, opt, nullptr, want_enu ? Stop::kEnu : Stop::kMesh, &ntri,
                    &nmv);
  if (rc) return rc;
  if (nmv > cap_vert || ntri > cap_tri)
    return fail(HZ_ERR_VALUE, "output capacity too small (%d vertices, %d triangles)", nmv,
                ntri);
  if (want_enu) {
    HZ_CUDA(cudaMemcpyAsync(enu32, b.vert32, (size_t)nmv * 3 * 4, cudaMemcpyDeviceToHost, s));
  } else {
    HZ_CUDA(cudaMemcpyAsync(mesh_lon, b.clon, nc * 8, cudaMemcpyDeviceToHost, s));
    HZ_CUDA(cudaMemcpyAsync(mesh_lat, b.clat, nc * 8, cudaMemcpyDeviceToHost, s));
    HZ_CUDA(cudaMemcpyAsync(mesh_h, b.hsurf, nc * 8, cudaMemcpyDeviceToHost, s));
    const size_t na = (size_t)(nmv - num_cell);
    if (na) {
      HZ_CUDA(cudaMemcpyAsync(mesh_lon + nc, b.add_lon, na * 8, cudaMemcpyDeviceToHost, s));
      HZ_CUDA(cudaMemcpyAsync(mesh_lat + nc, b.add_lat, na * 8, cudaMemcpyDeviceToHost, s));
      HZ_CUDA(cudaMemcpyAsync(mesh_h + nc, b.add_h, na * 8, cudaMemcpyDeviceToHost, s));
    }
  }
  if (ntri)
    HZ_CUDA(cudaMemcpyAsync(vot, b.vot, (size_t)ntri * 3 * 4, cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  *n_mesh_vert = nmv;
  *n_tri = ntri;
  return HZ_OK;
}

int hz_build_mesh(const double* clon, const double* clat, const double* hsurf,
                  const double* vlon, const double* vlat, const int32_t* cells_of_vertex,
                  int num_cell, int num_vertex, int grid_type, double* mesh_lon,
                  double* mesh_lat, double* mesh_h, int cap_vert, int32_t* vertex_of_triangle,
                  int cap_tri, int* n_mesh_vert, int* n_tri, int device) {
  return mesh_host_common(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_cell,
                          num_vertex, grid_type, device, false, mesh_lon, mesh_lat, mesh_h,
                          nullptr, cap_vert, vertex_of_triangle, cap_tri, n_mesh_vert, n_tri);
}

int hz_mesh_enu32(const double* clon, const double* clat, const double* hsurf,
                  const double* vlon, const double* vlat, const int32_t* cells_of_vertex,
                  int num_cell, int num_vertex, int grid_type, float* enu32, int cap_vert,
                  int32_t* vertex_of_triangle, int cap_tri, int* n_mesh_vert, int* n_tri,
                  int device) {
  return mesh_host_common(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_cell,
                          num_vertex, grid_type, device, true, nullptr, nullptr, nullptr,
                          enu32, cap_vert, vertex_of_triangle, cap_tri, n_mesh_vert, n_tri);
}

}  // extern "C"
