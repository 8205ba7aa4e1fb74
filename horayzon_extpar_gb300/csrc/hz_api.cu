// hz_api.cu -- the C ABI (include/horayzon_gb300.h) and the per-device engine
// that runs mesh assembly, geodetic frames, LBVH build and horizon search for
// one domain or a batch of domains.
//
// Pipeline of one call over n domains (mo_lradtopo_horayzon.cpp:562-785 per
// domain):
//   mesh_count + scan for every domain -> [read totals, check indices] ->
//   mesh_emit + mesh_ecef for every domain -> [read cell ECEF sums] -> ENU
//   frames on the host (glibc, same expressions as cpp:624-644) -> mesh_enu +
//   bvh_build + lattice tables + cell order (Hilbert curve) for every domain
//   -> cell-frame pre-pass, ONE persistent search launch over all cells of
//   all domains, epilogue -> counters. The part after the host frames is
//   captured into a CUDA graph kept on the engine (Capture).
// Device memory comes from one grow-only arena per device, carved per call.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/horayzon_gb300.h"
#include "hz_internal.h"

namespace hz {
namespace {

thread_local std::string g_last_error;
thread_local long long g_launches = 0;
// Progress lines of the current call (the reference's std::cout lines).
thread_local std::string g_log;

void log_line(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_log += buf;
}
// NVTX range of the current phase of a call (host side, as enqueued), for
// profilers that show NVTX; a no-op without one attached.
struct PhaseRange {
  bool open = false;
  void next(const char* name) {
    if (open) nvtxRangePop();
    nvtxRangePushA(name);
    open = true;
  }
  ~PhaseRange() {
    if (open) nvtxRangePop();
  }
};

const char* kRule =
    "-------------------------------------------------------------------------------\n";

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

// One domain's problem: arrays (device pointers once staged) and arguments.
struct Problem {
  const double *clon, *clat, *hsurf, *vlon, *vlat;
  const int* cov;
  double *horizon, *skyview;
  int ncell, nvert, nhori, grid_type;
  double dist_search, ray_org_elev;
  int refine, svf_type;
  int cell_begin, cell_count;  // traced range
  int groups;                  // search items per traced cell (DomainDesc::groups)
};

// Device buffers of one domain.
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
  float* vert_lo;    // precise mode only
  float4* tri_lo;    // precise mode only
  // learned warm start only
  unsigned* rz_bits;
  float4* rz;          // raster quads (RasterDesc::quad)
  long long raster_budget;
  RasterDesc* rdesc;   // device descriptor of the raster
  int16_t* start_m;
  double* svf_part;    // split learned start with refine_factor > 1: [groups][ncell]
  double* cell_enu;
  double* cell_frame;  // [9][ncell] (persistent search)
  float* cell_origin;  // [6][ncell]
  // BVH
  Node* nodes;
  Node4* nodes4;     // wide traversal only
  Tri* tris;
  BvhScratch bvh;
  // search
  void* order_scratch;
  unsigned* cell_bounds;
  double2 *azim_cs, *elev_cs;
  double* svf_lattice;
  int* err;
};

// Traversal loop of the persistent search selected by hz_options.kernel.
int trace_variant(const hz_options& opt) {
  // HZ_KERNEL_PER_CELL runs single domains only; batches fall back to the
  // persistent search on the binary BVH it builds.
  return opt.kernel == HZ_KERNEL_PERSISTENT ? kTraceWide : kTraceBinary;
}

Buffers carve_domain(Carver& c, long long ncell, long long nvert, long long nhori,
                     int grid_type, bool host_io, bool precise = false, bool learned = false,
                     long long L = 0, bool wide = false, long long svf_part_len = 0) {
  Buffers b;
  std::memset(&b, 0, sizeof(b));
  const long long max_tri = (grid_type == 0 ? 4 : 6) * nvert;
  const long long max_mv = ncell + nvert;
  if (host_io) {
    b.clon = c.take<double>(ncell);
    b.clat = c.take<double>(ncell);
    b.hsurf = c.take<double>(ncell);
    b.vlon = c.take<double>(nvert);
    b.vlat = c.take<double>(nvert);
    b.cov = c.take<int>(6 * nvert);
    b.horizon = c.take<double>(nhori * ncell);
    b.skyview = c.take<double>(ncell);
  }
  b.packed = c.take<unsigned long long>(nvert);
  b.offsets = c.take<unsigned long long>(nvert);
  b.scan_partials = c.take<unsigned long long>(scan_partials(nvert));
  b.totals = c.take<unsigned long long>(4);
  b.vot = c.take<int>(3 * max_tri);
  b.add_lon = c.take<double>(nvert);
  b.add_lat = c.take<double>(nvert);
  b.add_h = c.take<double>(nvert);
  b.ecef = c.take<double>(3 * max_mv);
  b.block_sums = c.take<double>(3 * (size_t)ecef_blocks((int)max_mv));
  b.origin_sum = c.take<double>(4);
  b.vert32 = c.take<float>(3 * max_mv);
  b.cell_enu = c.take<double>(3 * ncell);
  b.cell_frame = c.take<double>(9 * ncell);
  b.cell_origin = c.take<float>(6 * ncell);
  const long long nt = max_tri > 0 ? max_tri : 1;
  b.nodes = c.take<Node>(nt > 1 ? nt - 1 : 1);
  if (wide) b.nodes4 = c.take<Node4>(nt > 1 ? nt - 1 : 1);
  b.tris = c.take<Tri>(nt);
  if (precise) {
    b.vert_lo = c.take<float>(3 * max_mv);
    b.tri_lo = c.take<float4>(3 * nt);
  }
  if (learned) {
    b.raster_budget = max_mv + max_mv / 10 + 4096;
    b.rz_bits = c.take<unsigned>(b.raster_budget);
    b.rz = c.take<float4>(b.raster_budget);
    b.rdesc = c.take<RasterDesc>(1);
    b.start_m = c.take<int16_t>(L * ncell);
  }
  if (svf_part_len > 0) b.svf_part = c.take<double>(svf_part_len);
  b.bvh.keys = c.take<uint32_t>(nt);
  b.bvh.vals = c.take<int32_t>(nt);
  b.bvh.keys_alt = c.take<uint32_t>(nt);
  b.bvh.vals_alt = c.take<int32_t>(nt);
  b.bvh.cxy = c.take<float2>(nt);
  b.bvh.parent = c.take<int>(nt);
  b.bvh.nsize = c.take<int>(nt);
  b.bvh.counter = c.take<int>(nt);
  b.bvh.cost = c.take<float>(nt);
  b.bvh.bounds = c.take<unsigned>(16);
  b.bvh.sort_scratch = c.take<char>(radix_scratch_u32(nt));
  b.order_scratch = c.take<char>(cell_order_scratch_bytes(ncell));
  b.cell_bounds = c.take<unsigned>(8);
  b.azim_cs = c.take<double2>(nhori * 50);  // L <= num_hori * max refine_factor
  b.elev_cs = c.take<double2>(kElevTable);
  b.svf_lattice = c.take<double>(kSvfTable);
  b.err = c.take<int>(4);
  return b;
}

// Device buffers shared by the domains of one call.
struct BatchBuffers {
  DomainDesc* doms;
  int32_t* order;                 // all work ids
  int* work;
  unsigned long long* counters;   // rays, node visits, triangle tests
  unsigned long long* done;       // per domain: finished cells, completion time
  unsigned long long* t0;         // globaltimer at the start of the search
  int* err;
  float* mlp;                     // learned warm start parameters (device copy)
};

BatchBuffers carve_batch(Carver& c, int n, long long total_cells) {
  BatchBuffers b;
  b.mlp = c.take<float>(kMlpParams);
  b.doms = c.take<DomainDesc>(n);
  b.order = c.take<int32_t>(total_cells);
  b.work = c.take<int>(4);
  b.counters = c.take<unsigned long long>(kCounterWords);
  b.done = c.take<unsigned long long>(2 * (size_t)n);
  b.t0 = c.take<unsigned long long>(2);
  b.err = c.take<int>(4);
  return b;
}

// Stream capture of a stretch of a call into a CUDA graph. Inactive: the
// work is launched directly. An early return inside the stretch ends the
// capture and drops the partial graph.
// The capture runs on the engine's own stream (the caller's may be the
// legacy default stream, which cannot be captured); the graph is launched on
// the caller's stream.
struct Capture {
  cudaStream_t s;       // captured
  cudaStream_t launch;  // the graph's stream
  bool active;
  bool capturing = false;
  Capture(cudaStream_t st, cudaStream_t call, bool on) : s(st), launch(call), active(on) {}
  cudaError_t begin() {
    if (!active) return cudaSuccess;
    const cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    capturing = e == cudaSuccess;
    return e;
  }
  // A timing event: recorded as a node of the graph while capturing, else on
  // the caller's stream, which then carries the work.
  cudaError_t record(cudaEvent_t ev) {
    return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                     : cudaEventRecord(ev, launch);
  }
  // Ends the capture, updates the cached executable graph in place (or
  // instantiates it when the shape changed) and launches it.
  cudaError_t end_and_launch(cudaGraphExec_t* exec) {
    if (!capturing) return cudaSuccess;
    capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess) return e;
    if (*exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(*exec, g, &info) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
      }
    }
    if (!*exec) e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return e;
    return cudaGraphLaunch(*exec, launch);
  }
  ~Capture() {
    if (capturing) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
    }
  }
};

struct Engine {
  int device = -1;
  cudaGraphExec_t graph = nullptr;  // the last captured call (Capture)
  std::mutex mu;
  void* arena = nullptr;
  size_t cap = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  static constexpr int kSide = 8;        // streams the per-domain builds of a batch spread over
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kSide] = {};
  unsigned long long* pinned = nullptr;  // readbacks and descriptor staging
  size_t pinned_words = 0;
  Staging* staging = nullptr;            // pageable caller buffers (host entries)

  int init(int dev) {
    device = dev;
    HZ_CUDA(cudaSetDevice(dev));
    HZ_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (auto& e : ev) HZ_CUDA(cudaEventCreate(&e));
    for (int k = 0; k < kSide; k++) {
      HZ_CUDA(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking));
      HZ_CUDA(cudaEventCreateWithFlags(&join_ev[k], cudaEventDisableTiming));
    }
    HZ_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    HZ_CUDA(staging_create(&staging));
    return reserve_pinned(4096);
  }

  int reserve_pinned(size_t words) {
    if (words <= pinned_words) return HZ_OK;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    pinned_words = 0;
    HZ_CUDA(cudaMallocHost((void**)&pinned, words * sizeof(unsigned long long)));
    pinned_words = words;
    return HZ_OK;
  }

  int reserve(size_t bytes, cudaStream_t s) {
    if (bytes <= cap) return HZ_OK;
    // Failure injection for tests of the error path (no GPU fault involved):
    // HZ_INJECT_ALLOC_FAILURE=1 makes every growth of the workspace fail.
    const char* inject = getenv("HZ_INJECT_ALLOC_FAILURE");
    if (inject && inject[0] == '1')
      return fail(HZ_ERR_CUDA, "cudaMalloc of %zu bytes failed: injected failure", bytes);
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
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    if (arena) cudaFree(arena);
    arena = nullptr;
    cap = 0;
  }
};

// The per-domain work of a loop spread over the engine's side streams
// (domain d on side[d % k]) behind an event recorded on s; s then waits for
// all of them. Inside a stream capture these become fork and join edges of
// the graph. With one domain the work stays on s.
struct Fork {
  Engine& E;
  cudaStream_t s;
  int used;
  Fork(Engine& e, cudaStream_t st, int n)
      : E(e), s(st), used(n > 1 ? std::min(n, Engine::kSide) : 0) {}
  cudaError_t begin() {
    if (!used) return cudaSuccess;
    cudaError_t e = cudaEventRecord(E.fork_ev, s);
    for (int k = 0; k < used && e == cudaSuccess; k++) e = cudaStreamWaitEvent(E.side[k], E.fork_ev, 0);
    return e;
  }
  cudaStream_t on(int d) const { return used ? E.side[d % used] : s; }
  cudaError_t end() {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < used && e == cudaSuccess; k++) {
      e = cudaEventRecord(E.join_ev[k], E.side[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, E.join_ev[k], 0);
    }
    return e;
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

__global__ void k_stamp(unsigned long long* t) {
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  *t = now;
}

enum class Stop { kMesh, kEnu, kFull };

struct RunOut {
  std::vector<int> n_tri, n_mv;
  std::vector<double> latency_ms;
  std::vector<double> origin_lat, origin_lon;  // ENU origin per domain [deg]
};

// Resident threads of the current device (SMs x min(threads per SM, 1024)).
int resident_lanes(long long* lanes) {
  int dev = 0, sms = 0, threads = 0;
  HZ_CUDA(cudaGetDevice(&dev));
  HZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  HZ_CUDA(cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
  *lanes = (long long)sms * std::min(threads, 1024);
  return HZ_OK;
}

// Searches of more items than this many times the resident lanes queue the
// border cells of each domain first (run_batch).
constexpr long long kBorderFirstWaves = 4;

// Runs the pipeline for n domains whose arrays are device pointers in pr[].
// With stop != kFull it ends after the mesh (or ENU) stage and leaves the
// results in b[].
int run_batch(Engine& E, const Problem* pr, const Buffers* b, int n, const BatchBuffers& bb,
              cudaStream_t s, const hz_options& opt, hz_stats* st, Stop stop, RunOut* out) {
  g_launches = 0;
  g_log.clear();
  out->n_tri.assign(n, 0);
  out->n_mv.assign(n, 0);
  out->latency_ms.assign(n, 0.0);
  out->origin_lat.assign(n, 0.0);
  out->origin_lon.assign(n, 0.0);
  // Pinned layout (64-bit words): 0-63 counters and flags; 64 + [0, n) mesh
  // totals; 64 + [n, 2n) error words; 64 + [2n, 5n) cell ECEF sums; the
  // search descriptors from word 64 + 5n + 8.
  const size_t desc_words = (sizeof(DomainDesc) * (size_t)n + 7) / 8;
  int rc = E.reserve_pinned(64 + 5 * (size_t)n + 8 + desc_words);
  if (rc) return rc;
  unsigned long long* pin = E.pinned;
  for (int d = 0; d < n; d++) HZ_CUDA(cudaMemsetAsync(b[d].err, 0, 4 * sizeof(int), s));
  HZ_CUDA(cudaMemsetAsync(bb.err, 0, 4 * sizeof(int), s));
  HZ_CUDA(cudaMemsetAsync(bb.counters, 0, kCounterWords * sizeof(unsigned long long), s));
#ifdef HZ_DIAG
  HZ_CUDA(cudaMemsetAsync(bb.counters + 12, 0xFF, 2 * sizeof(unsigned long long), s));
#endif
  HZ_CUDA(cudaMemsetAsync(bb.done, 0, 2 * sizeof(unsigned long long) * (size_t)n, s));
  PhaseRange phase;
  phase.next("hz: mesh");
  HZ_CUDA(cudaEventRecord(E.ev[0], s));

  // ---- mesh (cpp:228-317) ----
  unsigned long long* pin_tot = pin + 64;
  unsigned long long* pin_err = pin + 64 + n;
  {
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int d = 0; d < n; d++) {
      const Problem& P = pr[d];
      const cudaStream_t sd = fk.on(d);
      HZ_CUDA(mesh_count(P.cov, P.nvert, P.ncell, P.grid_type, b[d].packed, b[d].err, sd));
      if (P.nvert > 0) {
        HZ_CUDA(scan_exclusive_u64(b[d].packed, b[d].offsets, P.nvert, b[d].totals,
                                   b[d].scan_partials, sd));
        HZ_CUDA(cudaMemcpyAsync(pin_tot + d, b[d].totals, sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, sd));
      }
      HZ_CUDA(cudaMemcpyAsync(pin_err + d, b[d].err, sizeof(int), cudaMemcpyDeviceToHost, sd));
    }
    HZ_CUDA(fk.end());
  }
  HZ_CUDA(cudaStreamSynchronize(s));
  std::vector<int> nadd(n);
  for (int d = 0; d < n; d++) {
    if ((int)(pin_err[d] & 0xFFFFFFFFull) & kErrBadIndex)
      return fail(HZ_ERR_INDEX, "Indices of 'cells_of_vertex' out of range%s",
                  n > 1 ? " (batch domain)" : "");
    const unsigned long long tot = pr[d].nvert > 0 ? pin_tot[d] : 0ull;
    out->n_tri[d] = (int)(tot & 0xFFFFFFFFull);
    nadd[d] = (int)(tot >> 32);
    // Leaf references and postponed leaves keep a triangle index in 27 bits.
    if (out->n_tri[d] >= (1 << 27))
      return fail(HZ_ERR_VALUE, "mesh of %d triangles exceeds 2^27 per domain", out->n_tri[d]);
    out->n_mv[d] = pr[d].ncell + nadd[d];
  }
  {
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int d = 0; d < n; d++) {
      const Problem& P = pr[d];
      HZ_CUDA(mesh_emit(P.clon, P.clat, P.hsurf, P.vlon, P.vlat, P.cov, P.nvert, P.ncell,
                        P.grid_type, b[d].offsets, b[d].vot, b[d].add_lon, b[d].add_lat,
                        b[d].add_h, fk.on(d)));
    }
    HZ_CUDA(fk.end());
  }
  if (stop == Stop::kMesh) return HZ_OK;

  // ---- frames (cpp:611-644) ----
  double* sums = reinterpret_cast<double*>(pin + 64 + 2 * n);
  {
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int d = 0; d < n; d++) {
      const Problem& P = pr[d];
      HZ_CUDA(mesh_ecef(P.clon, P.clat, P.hsurf, b[d].add_lon, b[d].add_lat, b[d].add_h,
                        P.ncell, nadd[d], b[d].ecef, b[d].block_sums, b[d].origin_sum,
                        fk.on(d)));
      HZ_CUDA(cudaMemcpyAsync(sums + 3 * d, b[d].origin_sum, 3 * sizeof(double),
                              cudaMemcpyDeviceToHost, fk.on(d)));
    }
    HZ_CUDA(fk.end());
  }
  HZ_CUDA(cudaStreamSynchronize(s));
  std::vector<Frame> frames(n);
  for (int d = 0; d < n; d++) {
    frames[d] = enu_frame_from_sum(sums[3 * d], sums[3 * d + 1], sums[3 * d + 2]);
    const double* so = sums + 3 * d;
    const double radius = sqrt(so[0] * so[0] + so[1] * so[1] + so[2] * so[2]);
    out->origin_lat[d] = rad2deg(asin(so[2] / radius));
    out->origin_lon[d] = rad2deg(atan2(so[1], so[0]));
  }

  // From here to the readback the host waits for nothing: the work is
  // captured into a CUDA graph, kept on the engine and updated in place for
  // the next call of the same shape, and launched as one unit. The learned
  // start's parameters are copied before (a pageable host source).
  if (stop == Stop::kFull && b[0].rz != nullptr && opt.mlp_params)
    HZ_CUDA(cudaMemcpyAsync(bb.mlp, opt.mlp_params, sizeof(float) * kMlpParams,
                            cudaMemcpyHostToDevice, s));
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  HZ_CUDA(cudaStreamIsCapturing(s, &cap_status));
  Capture cap(E.stream, s, stop == Stop::kFull && !opt.direct_launch &&
                     opt.kernel != HZ_KERNEL_PER_CELL &&
                     cap_status == cudaStreamCaptureStatusNone);
  HZ_CUDA(cap.begin());
  const cudaStream_t s_call = s;
  if (cap.capturing) s = cap.s;
  {
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int d = 0; d < n; d++)
      HZ_CUDA(mesh_enu(b[d].ecef, out->n_mv[d], pr[d].ncell, frames[d], b[d].vert32,
                       b[d].cell_enu, b[d].vert_lo, fk.on(d)));
    HZ_CUDA(fk.end());
  }
  HZ_CUDA(cap.record(E.ev[1]));
  phase.next("hz: bvh");
  if (stop == Stop::kEnu) return HZ_OK;

  // ---- BVH (cpp:395-432) ----
  {
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int d = 0; d < n; d++) {
      HZ_CUDA(bvh_build(b[d].vert32, b[d].vot, out->n_tri[d], b[d].nodes, b[d].tris, b[d].bvh,
                        fk.on(d), b[d].vert_lo, b[d].tri_lo, b[d].nodes4, opt.leaf_size,
                        opt.bvh_treelets != 0));
    }
    HZ_CUDA(fk.end());
  }
  HZ_CUDA(cap.record(E.ev[2]));
  phase.next("hz: search");

  // ---- horizon + SVF (cpp:651-761) ----
  const double hori_acc = deg2rad(0.25);
  const double elev_floor = deg2rad(opt.elev_floor_deg);
  std::vector<double> shift(n);
  for (int d = 0; d < n; d++) {
    const int L = pr[d].nhori * pr[d].refine;
    shift[d] = 0.0;
    if (pr[d].refine != 1)
      shift[d] = -(deg2rad(360.0) / (2.0 * pr[d].nhori)) + (deg2rad(360.0) / (2.0 * (double)L));
  }
  if (opt.kernel == HZ_KERNEL_PER_CELL && n == 1) {
    const Problem& P = pr[0];
    TraceParams p;
    std::memset(&p, 0, sizeof(p));
    p.cell_enu = b[0].cell_enu;
    p.ncell = P.ncell;
    p.cell_begin = P.cell_begin;
    p.cell_count = P.cell_count;
    p.nodes = b[0].nodes;
    p.tris = b[0].tris;
    p.root = out->n_tri[0] > 0 ? 0 : kEmptyRef;
    p.centre = frames[0].centre;
    p.pole = frames[0].pole;
    p.ray_org_elev = P.ray_org_elev;
    p.tfar = (float)P.dist_search;
    p.nhori = P.nhori;
    p.refine = P.refine;
    p.L = P.nhori * P.refine;
    p.svf_type = P.svf_type;
    p.hori_acc = hori_acc;
    p.elev_floor = elev_floor;
    p.azim_sin = sin(deg2rad(360.0) / (double)p.L);
    p.azim_cos = cos(deg2rad(360.0) / (double)p.L);
    p.elev_sin_2ha = sin(2.0 * p.hori_acc);
    p.elev_cos_2ha = cos(2.0 * p.hori_acc);
    p.shift_sin = sin(-shift[0]);
    p.shift_cos = cos(-shift[0]);
    p.horizon = P.horizon;
    p.skyview = P.skyview;
    p.counters = bb.counters;
    p.err = bb.err;
    HZ_CUDA(trace_exact(p, opt.count_work != 0, s));
  } else {
    DomainDesc* desc = reinterpret_cast<DomainDesc*>(pin + 64 + 5 * (size_t)n + 8);
    // Learned warm start: height rasters over each domain's triangle-centre
    // bounds (from the BVH build, on the device), then features + MLP.
    const bool learned = b[0].rz != nullptr;
    long long total = 0, total_items = 0;
    // Border cells (of a vertex with a -2 entry) search several times as long
    // as inner ones; when the call's items fill the GPU's lanes several times
    // over they are queued first in each domain, so that none starts in the
    // search's last wave. In a single wave the Hilbert order, which spreads
    // them over the warps of the border's neighbourhood, is faster.
    long long items = 0, lanes = 0;
    for (int d = 0; d < n; d++) items += (long long)pr[d].cell_count * pr[d].groups;
    const int rl = resident_lanes(&lanes);
    if (rl) return rl;
    const bool border_first = items >= kBorderFirstWaves * lanes;
    // Queue order of the domains: least work (cells x azimuths) first, so
    // that the small domains of a batch complete early (shortest job first:
    // the lowest mean completion time for the same total work).
    std::vector<int> queue(n);
    for (int d = 0; d < n; d++) queue[d] = d;
    std::stable_sort(queue.begin(), queue.end(), [&](int x, int y) {
      return (long long)pr[x].cell_count * pr[x].nhori * pr[x].refine <
             (long long)pr[y].cell_count * pr[y].nhori * pr[y].refine;
    });
    Fork fk(E, s, n);
    HZ_CUDA(fk.begin());
    for (int j = 0; j < n; j++) {
      const int d = queue[j];
      const Problem& P = pr[d];
      const int L = P.nhori * P.refine;
      HZ_CUDA(trace_tables(b[d].azim_cs, b[d].elev_cs, b[d].svf_lattice, L, shift[d],
                           hori_acc, P.svf_type, fk.on(d)));
      if (learned) {
        HZ_CUDA(raster_build(b[d].vert32, b[d].vot, out->n_tri[d], b[d].bvh.bounds,
                             b[d].raster_budget, b[d].rdesc, b[d].rz_bits, b[d].rz, fk.on(d)));
        LearnParams q;
        std::memset(&q, 0, sizeof(q));
        q.cell_enu = b[d].cell_enu;
        q.centre = frames[d].centre;
        q.pole = frames[d].pole;
        q.ray_org_elev = P.ray_org_elev;
        q.ncell = P.ncell;
        q.cell_begin = P.cell_begin;
        q.cell_count = P.cell_count;
        q.nhori = P.nhori;
        q.L = L;
        // Predictions feed the first azimuth of each search item (of the
        // cell's chain, or of each of its azimuth groups) unless every
        // azimuth uses them; features for training cover every azimuth.
        if ((opt.features != nullptr && n == 1) || opt.mlp_every_azimuth) {
          q.n_pred = L;
          q.a_stride = 1;
        } else {
          q.n_pred = P.groups;
          q.a_stride = L / P.groups;
        }
        q.dist_search = (float)P.dist_search;
        q.azim_cs = b[d].azim_cs;
        q.raster = b[d].rdesc;
        q.features = n == 1 ? opt.features : nullptr;
        q.start_m = b[d].start_m;
        HZ_CUDA(learn_features(q, opt.mlp_params ? bb.mlp : nullptr, fk.on(d)));
      }
      HZ_CUDA(cell_order(b[d].cell_enu, border_first ? P.cov : nullptr, P.nvert, P.ncell,
                         P.cell_begin, P.cell_count,
                         (int)(total - P.cell_begin),
                         bb.order + total, b[d].order_scratch, b[d].cell_bounds, bb.work,
                         fk.on(d)));
      DomainDesc D;
      std::memset(&D, 0, sizeof(D));
      D.cell_enu = b[d].cell_enu;
      D.cell_frame = b[d].cell_frame;
      D.cell_origin = b[d].cell_origin;
      D.k_begin = total;
      D.cell_begin = P.cell_begin;
      D.nodes = b[d].nodes;
      D.nodes4 = b[d].nodes4;
      D.tris = b[d].tris;
      D.tri_lo = b[d].tri_lo;
      D.horizon = P.horizon;
      D.skyview = P.skyview;
      D.azim_cs = b[d].azim_cs;
      D.elev_cs = b[d].elev_cs;
      D.svf_lattice = b[d].svf_lattice;
      D.done = n > 1 ? bb.done + 2 * d : nullptr;
      D.start_m = opt.mlp_params ? b[d].start_m : opt.start_index;
      D.start_all = opt.mlp_every_azimuth ? 1 : 0;
      D.groups = P.groups;
      D.deep_walk = opt.elev_walk == HZ_WALK_BISECT ? 1 : 0;
      D.occ_cache = opt.occluder_cache != 0 ? 1 : 0;
      D.item_begin = total_items;
      D.svf_part = b[d].svf_part;
      D.raw_j = n == 1 ? opt.raw_index : nullptr;
      D.centre = frames[d].centre;
      D.pole = frames[d].pole;
      D.ray_org_elev = P.ray_org_elev;
      D.hori_acc = hori_acc;
      D.two_ha = 2.0 * hori_acc;
      D.elev_floor = elev_floor;
      D.cell_offset = total - P.cell_begin;
      D.root = out->n_tri[d] > 0 ? 0 : kEmptyRef;
      D.n_tri = out->n_tri[d];
      D.ncell = P.ncell;
      D.ncell_traced = P.cell_count;
      D.nhori = P.nhori;
      D.refine = P.refine;
      D.L = L;
      D.svf_type = P.svf_type;
      D.tfar = (float)P.dist_search;
      desc[j] = D;  // in queue order: k_begin and item_begin increase with j
      total += P.cell_count;
      total_items += (long long)P.cell_count * P.groups;
    }
    HZ_CUDA(fk.end());
    if (total_items > INT32_MAX - (1ll << 26))
      return fail(HZ_ERR_VALUE, "more than 2^31 - 2^26 search items (cells x azimuth groups) "
                                "in one call");
    HZ_CUDA(cudaMemcpyAsync(bb.doms, desc, sizeof(DomainDesc) * (size_t)n,
                            cudaMemcpyHostToDevice, s));
    const int adv =
        opt.advance_min >= 1 && opt.advance_min <= 32 ? opt.advance_min : kDefaultAdvanceMin;
    const int leaf = opt.leaf_min >= 1 && opt.leaf_min <= 32 ? opt.leaf_min : kDefaultLeafMin;
    const int variant = trace_variant(opt);
    k_stamp<<<1, 1, 0, s>>>(bb.t0);
    note_launches(1);
    HZ_CUDA(cudaGetLastError());
    const TraceKnobs knobs{adv, leaf, opt.queue_chunk, variant};
    HZ_CUDA(trace_flat(bb.doms, n, bb.order, (int)total, (int)total_items, bb.work,
                       bb.counters, bb.err, knobs, opt.count_work != 0,
                       b[0].tri_lo != nullptr, s));
  }
  HZ_CUDA(cap.record(E.ev[3]));
  phase.next("hz: readback");

  // Counters, error word, and per-domain completion times.
  unsigned long long* rb = pin;  // words 0..15 (descriptors live beyond word 64)
  HZ_CUDA(cudaMemcpyAsync(rb + 8, bb.counters, 3 * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaMemcpyAsync(rb + 12, bb.err, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaMemcpyAsync(rb + 14, bb.t0, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  unsigned long long* rb_done = pin + 64;  // the totals / error slots are no longer needed
  if (n > 1)
    HZ_CUDA(cudaMemcpyAsync(rb_done, bb.done, 2 * sizeof(unsigned long long) * (size_t)n,
                            cudaMemcpyDeviceToHost, s));
#ifdef HZ_DIAG
  HZ_CUDA(cudaMemcpyAsync(rb + 32, bb.counters, kCounterWords * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, s));
#endif
  HZ_CUDA(cap.end_and_launch(&E.graph));
  s = s_call;
  HZ_CUDA(cudaStreamSynchronize(s));
#ifdef HZ_DIAG
  fprintf(stderr, "hz_diag");
  for (int k = 0; k < kCounterWords; k++) fprintf(stderr, " %llu", rb[32 + k]);
  fprintf(stderr, "\n");
#endif
  const int* errw = reinterpret_cast<const int*>(rb + 12);  // bit word, check code, index
  const int err1 = errw[0];
  if (err1 & kErrStack) return fail(HZ_ERR_INTERNAL, "BVH traversal stack overflow");
  if (err1 & kErrBounds)
    return fail(HZ_ERR_INTERNAL, "bounds check failed in the search: check %d, index %d",
                errw[1], errw[2]);
  if (n > 1)
    for (int d = 0; d < n; d++)
      out->latency_ms[d] = rb_done[2 * d + 1] > rb[14]
                               ? (double)(rb_done[2 * d + 1] - rb[14]) * 1e-6
                               : 0.0;
  if (st) {
    st->kernel_launches = g_launches;
    st->num_rays = (int64_t)rb[8];
    st->node_visits = (int64_t)rb[9];
    st->tri_tests = (int64_t)rb[10];
    long long ntri = 0, nmv = 0;
    for (int d = 0; d < n; d++) {
      ntri += out->n_tri[d];
      nmv += out->n_mv[d];
    }
    st->n_tri = (int32_t)std::min<long long>(ntri, INT32_MAX);
    st->n_mesh_vert = (int32_t)std::min<long long>(nmv, INT32_MAX);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, E.ev[0], E.ev[1]);
    st->ms_mesh = ms;
    cudaEventElapsedTime(&ms, E.ev[1], E.ev[2]);
    st->ms_bvh = ms;
    cudaEventElapsedTime(&ms, E.ev[2], E.ev[3]);
    st->ms_trace = ms;
  }
  // Progress lines in the reference's order and wording (cpp:240-241,
  // 278-279, 315, 427-428, 589-594, 606-608, 639-641, 671-680, 765-776), with
  // the GPU phase times.
  float ms_mesh = 0.f, ms_bvh = 0.f, ms_ray = 0.f;
  cudaEventElapsedTime(&ms_mesh, E.ev[0], E.ev[1]);
  cudaEventElapsedTime(&ms_bvh, E.ev[1], E.ev[2]);
  cudaEventElapsedTime(&ms_ray, E.ev[2], E.ev[3]);
  g_log += kRule;
  log_line("Horizon and SVF computation on the GPU (horayzon_gb300 %d.%d.%d)\n",
           HZ_VERSION / 100, (HZ_VERSION / 10) % 10, HZ_VERSION % 10);
  g_log += kRule;
  long long evals = 0;
  for (int d = 0; d < n; d++) {
    if (n > 1) log_line("Domain %d of %d\n", d + 1, n);
    log_line("Build triangle mesh %s\n",
             pr[d].grid_type == 0
                 ? "solely from ICON grid cell circumcenters\n (non-unique triangulation)"
                 : "from ICON grid cell circumcenters and vertices\n (unique triangulation)");
    log_line("Number of triangles in mesh: %d\n", out->n_tri[d]);
    if (d == 0) log_line("Triangle mesh building: %.2f s\n", 1e-3 * ms_mesh);
    log_line("Origin of ENU coordinate system: %.4f deg lat, %.4f deg lon\n",
             out->origin_lat[d], out->origin_lon[d]);
    if (d == 0) log_line("Building bounding volume hierarchy (BVH): %.2f s\n", 1e-3 * ms_bvh);
    static const char* kSvf[3] = {"pure geometric SVF", "geometric scaled with sin(horizon)",
                                  "geometric scaled with sin(horizon)**2"};
    log_line("Sky View Factor computation algorithm: %s\n", kSvf[pr[d].svf_type]);
    evals += (long long)pr[d].cell_count * pr[d].nhori;
  }
  log_line("Ray tracing: %.2f s\n", 1e-3 * ms_ray);
  log_line("Number of rays shot: %lld\n", (long long)rb[8]);
  log_line("Average number of rays per cell and azimuth sector: %.2f\n",
           (double)rb[8] / (double)(evals > 0 ? evals : 1));
  g_log += kRule;
  if (opt.verbose) {
    fputs(g_log.c_str(), stdout);
    fflush(stdout);
  }
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

int cell_range(const hz_options& opt, int ncell, int* begin, int* count) {
  *begin = 0;
  *count = ncell;
  if (opt.cell_count > 0) {
    if (opt.cell_begin < 0 || (long long)opt.cell_begin + opt.cell_count > ncell)
      return fail(HZ_ERR_VALUE, "cell range [%d, %d) outside [0, %d)", opt.cell_begin,
                  opt.cell_begin + opt.cell_count, ncell);
    *begin = opt.cell_begin;
    *count = opt.cell_count;
  }
  return HZ_OK;
}

// Host <-> device staging of one domain for the host entry points.
int stage_inputs(Engine& E, const hz_domain& h, const Buffers& b, cudaStream_t s) {
  const size_t nc = (size_t)h.num_cell, nv = (size_t)h.num_vertex;
  Staging* st = E.staging;
  HZ_CUDA(copy_from_host(st, b.clon, h.clon, nc * 8, s));
  HZ_CUDA(copy_from_host(st, b.clat, h.clat, nc * 8, s));
  HZ_CUDA(copy_from_host(st, b.hsurf, h.hsurf, nc * 8, s));
  if (nv) {
    HZ_CUDA(copy_from_host(st, b.vlon, h.vlon, nv * 8, s));
    HZ_CUDA(copy_from_host(st, b.vlat, h.vlat, nv * 8, s));
    HZ_CUDA(copy_from_host(st, b.cov, h.cells_of_vertex, nv * 6 * 4, s));
  }
  return HZ_OK;
}

int unstage_outputs(Engine& E, const hz_domain& h, const Buffers& b, int begin, int count,
                    cudaStream_t s) {
  const size_t nc = (size_t)h.num_cell;
  if (begin != 0 || count != h.num_cell) {
    // Only the traced columns: the caller's other entries stay untouched.
    const size_t c0 = (size_t)begin, cn = (size_t)count;
    HZ_CUDA(cudaMemcpy2DAsync(h.horizon + c0, nc * 8, b.horizon + c0, nc * 8, cn * 8,
                              (size_t)h.num_hori, cudaMemcpyDeviceToHost, s));
    HZ_CUDA(cudaMemcpyAsync(h.skyview + c0, b.skyview + c0, cn * 8, cudaMemcpyDeviceToHost, s));
  } else {
    HZ_CUDA(copy_to_host(E.staging, h.horizon, b.horizon, (size_t)h.num_hori * nc * 8, s));
    HZ_CUDA(copy_to_host(E.staging, h.skyview, b.skyview, nc * 8, s));
  }
  return HZ_OK;
}

// Search items per traced cell for each domain (DomainDesc::groups) from
// hz_options.mlp_azimuth_groups: 1 without a learned start or for 0 / 1; an
// explicit G must divide every domain's num_hori; -1 picks, per domain, the
// smallest divisor G of num_hori that gives the call at least
// kItemsPerLane x the GPU's resident lanes of search items (the largest
// divisor up to num_hori / 2 when none does), so that small domains spread
// each cell's azimuths over G lanes while domains that fill the GPU keep the
// reference's chain.
constexpr int kItemsPerLane = 4;

int azimuth_groups(const hz_domain* doms, int n, const hz_options& opt, int* groups) {
  for (int d = 0; d < n; d++) groups[d] = 1;
  const int G = opt.mlp_azimuth_groups;
  if ((opt.mlp_params == nullptr && opt.start_index == nullptr) || opt.mlp_every_azimuth ||
      G == 0 || G == 1)
    return HZ_OK;
  if (G > 1) {
    for (int d = 0; d < n; d++) {
      if (doms[d].num_hori % G != 0)
        return fail(HZ_ERR_VALUE, "mlp_azimuth_groups %d does not divide num_hori %d", G,
                    doms[d].num_hori);
      groups[d] = G;
    }
    return HZ_OK;
  }
  if (G != -1) return fail(HZ_ERR_VALUE, "mlp_azimuth_groups must be -1, 0 or >= 1");
  long long lanes = 0;
  const int rc = resident_lanes(&lanes);
  if (rc) return rc;
  const long long target = (long long)kItemsPerLane * lanes;
  long long cells = 0;
  for (int d = 0; d < n; d++)
    cells += opt.cell_count > 0 && n == 1 ? opt.cell_count : doms[d].num_cell;
  for (int d = 0; d < n; d++) {
    // At most num_hori / 2 groups: every item keeps two azimuths of the
    // chain (an item per azimuth restarts every bracket at its proposal,
    // which exposes more of the evaluations whose result depends on the
    // start; see the parity figures of the split modes).
    const int nh = doms[d].num_hori;
    int pick = 1;
    for (int g = 1; g <= nh / 2; g++)
      if (nh % g == 0) {
        pick = g;
        if (cells * g >= target) break;
      }
    groups[d] = pick;
  }
  return HZ_OK;
}

// Shared implementation of the host / device, single / batch entry points.
int run_entry(hz_domain* doms, int n, bool on_device, cudaStream_t user_stream,
              const hz_options& opt, hz_stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  if (n < 1) return fail(HZ_ERR_VALUE, "no domains");
  // The search packs the domain index of a cell in 16 bits.
  if (n > 65535) return fail(HZ_ERR_VALUE, "at most 65535 domains per call");
  long long total_cells = 0;
  for (int d = 0; d < n; d++) {
    const hz_domain& h = doms[d];
    int rc = validate(h.num_cell, h.num_vertex, h.num_hori, h.grid_type, h.dist_search,
                      h.ray_org_elev, h.refine_factor, h.svf_type);
    if (rc) return rc;
    if (!h.clon || !h.clat || !h.hsurf || !h.horizon || !h.skyview ||
        (h.num_vertex > 0 && (!h.vlon || !h.vlat || !h.cells_of_vertex)))
      return fail(HZ_ERR_VALUE, "null array pointer");
    total_cells += h.num_cell;
  }
  if (n > 1 && opt.cell_count > 0)
    return fail(HZ_ERR_VALUE, "a cell range applies to single-domain calls only");
  Engine* E = nullptr;
  int rc = get_engine(opt.device, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  HZ_CUDA(cudaSetDevice(E->device));
  cudaStream_t s = on_device ? user_stream : E->stream;

  const bool precise = opt.precision == HZ_PRECISION_LOCAL;
  if (precise && opt.kernel == HZ_KERNEL_PER_CELL)
    return fail(HZ_ERR_VALUE, "HZ_PRECISION_LOCAL needs the persistent kernel");
  const bool learned = opt.mlp_params != nullptr || opt.features != nullptr;
  if (learned && opt.kernel == HZ_KERNEL_PER_CELL)
    return fail(HZ_ERR_VALUE, "the learned warm start needs the persistent kernel");
  if (opt.kernel < HZ_KERNEL_PERSISTENT || opt.kernel > HZ_KERNEL_PERSISTENT_BVH2)
    return fail(HZ_ERR_VALUE, "unknown kernel %d", opt.kernel);
  if (opt.elev_walk != HZ_WALK_REFERENCE && opt.elev_walk != HZ_WALK_BISECT)
    return fail(HZ_ERR_VALUE, "unknown elev_walk %d", opt.elev_walk);
  if (opt.elev_walk == HZ_WALK_BISECT && opt.kernel == HZ_KERNEL_PER_CELL)
    return fail(HZ_ERR_VALUE, "HZ_WALK_BISECT needs the persistent kernel");
  const bool wide = opt.kernel != HZ_KERNEL_PER_CELL && trace_variant(opt) == kTraceWide;
  if ((opt.raw_index || opt.features) && (n != 1 || !on_device))
    return fail(HZ_ERR_VALUE, "raw_index / features are outputs of the device entry point");
  if (opt.start_index && (n != 1 || !on_device || opt.mlp_params))
    return fail(HZ_ERR_VALUE, "start_index is an input of the device entry point (one domain, "
                              "no mlp_params)");
  std::vector<int> groups(n, 1);
  rc = azimuth_groups(doms, n, opt, groups.data());
  if (rc) return rc;
  auto svf_part_len = [&](int d) {
    return groups[d] > 1 && doms[d].refine_factor > 1
               ? (long long)groups[d] * doms[d].num_cell : 0ll;
  };
  Carver dry(nullptr);
  for (int d = 0; d < n; d++)
    carve_domain(dry, doms[d].num_cell, doms[d].num_vertex, doms[d].num_hori,
                 doms[d].grid_type, !on_device, precise, learned,
                 (long long)doms[d].num_hori * doms[d].refine_factor, wide, svf_part_len(d));
  carve_batch(dry, n, total_cells);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  std::vector<Buffers> b(n);
  for (int d = 0; d < n; d++)
    b[d] = carve_domain(c, doms[d].num_cell, doms[d].num_vertex, doms[d].num_hori,
                        doms[d].grid_type, !on_device, precise, learned,
                        (long long)doms[d].num_hori * doms[d].refine_factor, wide,
                        svf_part_len(d));
  const BatchBuffers bb = carve_batch(c, n, total_cells);

  std::vector<Problem> pr(n);
  // Host <-> device phases are timed on the host: pageable buffers are
  // copied partly by host threads.
  const auto t_h2d = std::chrono::steady_clock::now();
  for (int d = 0; d < n; d++) {
    const hz_domain& h = doms[d];
    if (!on_device) {
      rc = stage_inputs(*E, h, b[d], s);
      if (rc) return rc;
    }
    Problem& P = pr[d];
    P.clon = on_device ? h.clon : b[d].clon;
    P.clat = on_device ? h.clat : b[d].clat;
    P.hsurf = on_device ? h.hsurf : b[d].hsurf;
    P.vlon = on_device ? h.vlon : b[d].vlon;
    P.vlat = on_device ? h.vlat : b[d].vlat;
    P.cov = on_device ? h.cells_of_vertex : b[d].cov;
    P.horizon = on_device ? h.horizon : b[d].horizon;
    P.skyview = on_device ? h.skyview : b[d].skyview;
    P.ncell = h.num_cell;
    P.nvert = h.num_vertex;
    P.nhori = h.num_hori;
    P.grid_type = h.grid_type;
    P.dist_search = h.dist_search;
    P.ray_org_elev = h.ray_org_elev;
    P.refine = h.refine_factor;
    P.svf_type = h.svf_type;
    rc = cell_range(opt, h.num_cell, &P.cell_begin, &P.cell_count);
    if (rc) return rc;
    P.groups = groups[d];
  }
  double ms_h2d = 0.0;
  if (!on_device) {
    HZ_CUDA(cudaStreamSynchronize(s));
    ms_h2d = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_h2d)
                 .count();
  }
  if (stats) std::memset(stats, 0, sizeof(*stats));
  RunOut out;
  rc = run_batch(*E, pr.data(), b.data(), n, bb, s, opt, stats, Stop::kFull, &out);
  if (rc) return rc;
  for (int d = 0; d < n; d++) doms[d].latency_ms = out.latency_ms[d];
  const auto t_d2h = std::chrono::steady_clock::now();
  if (!on_device) {
    for (int d = 0; d < n; d++) {
      rc = unstage_outputs(*E, doms[d], b[d], pr[d].cell_begin, pr[d].cell_count, s);
      if (rc) return rc;
    }
  }
  HZ_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    if (!on_device) {
      stats->ms_h2d = ms_h2d;
      stats->ms_d2h =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_d2h)
              .count();
    }
    stats->ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return HZ_OK;
}

hz_domain make_domain(const double* clon, const double* clat, const double* hsurf,
                      const double* vlon, const double* vlat, const int32_t* cov,
                      double* horizon, double* skyview, int num_cell, int num_vertex,
                      int num_hori, int grid_type, double dist_search, double ray_org_elev,
                      int refine_factor, int svf_type) {
  hz_domain h;
  std::memset(&h, 0, sizeof(h));
  h.clon = clon;
  h.clat = clat;
  h.hsurf = hsurf;
  h.vlon = vlon;
  h.vlat = vlat;
  h.cells_of_vertex = cov;
  h.horizon = horizon;
  h.skyview = skyview;
  h.num_cell = num_cell;
  h.num_vertex = num_vertex;
  h.num_hori = num_hori;
  h.grid_type = grid_type;
  h.dist_search = dist_search;
  h.ray_org_elev = ray_org_elev;
  h.refine_factor = refine_factor;
  h.svf_type = svf_type;
  return h;
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
  opt->occluder_cache = 1;
}

const char* hz_last_error(void) { return g_last_error.c_str(); }

int hz_version(void) { return HZ_VERSION; }

int hz_release_workspace(int device) {
  static_forget_device(device);
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
  const hz_options opt = resolve(opt_in);
  hz_domain h = make_domain(clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon, skyview,
                            num_cell, num_vertex, num_hori, grid_type, dist_search,
                            ray_org_elev, refine_factor, svf_type);
  return run_entry(&h, 1, true, (cudaStream_t)stream, opt, stats);
}

int hz_horizon_svf(const double* clon, const double* clat, const double* hsurf,
                   const double* vlon, const double* vlat, const int32_t* cells_of_vertex,
                   double* horizon, double* skyview, int num_cell, int num_vertex,
                   int num_hori, int grid_type, double dist_search, double ray_org_elev,
                   int refine_factor, int svf_type, const hz_options* opt_in,
                   hz_stats* stats) {
  g_last_error.clear();
  const hz_options opt = resolve(opt_in);
  hz_domain h = make_domain(clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon, skyview,
                            num_cell, num_vertex, num_hori, grid_type, dist_search,
                            ray_org_elev, refine_factor, svf_type);
  return run_entry(&h, 1, false, nullptr, opt, stats);
}

int hz_mlp_num_params(void) { return kMlpParams; }

int hz_mlp_train_step(float* params, float* adam_m, float* adam_v, const float* X,
                      const float* T, int n, int step, float lr, float* loss, float* grads,
                      void* stream) {
  g_last_error.clear();
  if (!params || !X || !T || !loss || !grads || n < 1 || step < 1 ||
      (lr > 0.f && (!adam_m || !adam_v)))
    return fail(HZ_ERR_VALUE, "invalid MLP training arguments");
  Engine* E = nullptr;
  int rc = get_engine(-1, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  cudaStream_t s = (cudaStream_t)stream;
  rc = E->reserve(sizeof(float) * mlp_train_scratch_floats(n), s);
  if (rc) return rc;
  HZ_CUDA(mlp_train_step(params, adam_m, adam_v, X, T, n, step, lr, loss, grads,
                         (float*)E->arena, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  return HZ_OK;
}

int hz_mlp_forward(const float* params, const float* X, int n, float* Y, void* stream) {
  g_last_error.clear();
  if (!params || !X || !Y || n < 0) return fail(HZ_ERR_VALUE, "invalid MLP arguments");
  cudaStream_t s = (cudaStream_t)stream;
  HZ_CUDA(mlp_forward(params, X, n, Y, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  return HZ_OK;
}

int hz_horizon_svf_batch(hz_domain* domains, int n_domains, int on_device, void* stream,
                         const hz_options* opt_in, hz_stats* stats) {
  g_last_error.clear();
  if (!domains || n_domains < 1) return fail(HZ_ERR_VALUE, "no domains");
  const hz_options opt = resolve(opt_in);
  return run_entry(domains, n_domains, on_device != 0, (cudaStream_t)stream, opt, stats);
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

void horizon_svf_comp_buffer(double* clon, double* clat, double* hsurf, double* vlon,
                             double* vlat, int* cells_of_vertex, double* horizon,
                             double* skyview, int num_cell, int num_vertex, int num_hori,
                             int grid_type, double dist_search, double ray_org_elev,
                             int refine_factor, int svf_type, char* buffer, int* buffer_len) {
  hz_options opt;
  hz_default_options(&opt);
  g_log.clear();
  int rc = hz_horizon_svf(clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon, skyview,
                          num_cell, num_vertex, num_hori, grid_type, dist_search,
                          ray_org_elev, refine_factor, svf_type, &opt, nullptr);
  if (rc != HZ_OK) {
    g_log += "horizon_svf_comp: ";
    g_log += hz_last_error();
    g_log += "\n";
    if (horizon && skyview && num_cell > 0 && num_hori > 0) {
      for (long long k = 0; k < (long long)num_hori * num_cell; k++) horizon[k] = NAN;
      for (int k = 0; k < num_cell; k++) skyview[k] = NAN;
    }
  }
  // cpp:778-784: copy min(*buffer_len, length) bytes, no terminator, and
  // return the count in *buffer_len.
  if (buffer && buffer_len) {
    const int n = std::max(0, std::min(*buffer_len, (int)g_log.size()));
    if (n > 0) std::memcpy(buffer, g_log.data(), (size_t)n);
    *buffer_len = n;
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
  Carver dry(nullptr);
  carve_domain(dry, num_cell, num_vertex, 4, grid_type, true);
  carve_batch(dry, 1, num_cell);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  const Buffers b = carve_domain(c, num_cell, num_vertex, 4, grid_type, true);
  const BatchBuffers bb = carve_batch(c, 1, num_cell);
  hz_domain h = make_domain(clon, clat, hsurf, vlon, vlat, cov, nullptr, nullptr, num_cell,
                            num_vertex, 4, grid_type, 1e4, 1.0, 1, 0);
  rc = stage_inputs(*E, h, b, s);
  if (rc) return rc;
  Problem pr;
  std::memset(&pr, 0, sizeof(pr));
  pr.clon = b.clon;
  pr.clat = b.clat;
  pr.hsurf = b.hsurf;
  pr.vlon = b.vlon;
  pr.vlat = b.vlat;
  pr.cov = b.cov;
  pr.ncell = num_cell;
  pr.nvert = num_vertex;
  pr.nhori = 4;
  pr.grid_type = grid_type;
  pr.refine = 1;
  pr.cell_count = num_cell;
  hz_options opt;
  hz_default_options(&opt);
  RunOut out;
  rc = run_batch(*E, &pr, &b, 1, bb, s, opt, nullptr, want_enu ? Stop::kEnu : Stop::kMesh,
                 &out);
  if (rc) return rc;
  const int nmv = out.n_mv[0], ntri = out.n_tri[0];
  if (nmv > cap_vert || ntri > cap_tri)
    return fail(HZ_ERR_VALUE, "output capacity too small (%d vertices, %d triangles)", nmv,
                ntri);
  const size_t nc = (size_t)num_cell;
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

int hz_occluded32(const float* vert, int n_vert, const int32_t* vertex_of_triangle, int n_tri,
                  const float* org, const float* dir, int n_ray, float tfar, uint8_t* hit,
                  int tree, int leaf_size, int device) {
  g_last_error.clear();
  if (n_vert < 0 || n_tri < 0 || n_ray < 0 || (tree != 0 && tree != 1) ||
      (n_vert > 0 && !vert) || (n_tri > 0 && !vertex_of_triangle) ||
      (n_ray > 0 && (!org || !dir || !hit)))
    return fail(HZ_ERR_VALUE, "invalid arguments");
  if (n_tri >= (1 << 27)) return fail(HZ_ERR_VALUE, "more than 2^27 triangles");
  for (long long k = 0; k < 3LL * n_tri; k++)
    if (vertex_of_triangle[k] < 0 || vertex_of_triangle[k] >= n_vert)
      return fail(HZ_ERR_INDEX, "vertex_of_triangle index out of range");
  if (n_ray == 0) return HZ_OK;
  Engine* E = nullptr;
  int rc = get_engine(device, &E);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(E->mu);
  HZ_CUDA(cudaSetDevice(E->device));
  cudaStream_t s = E->stream;
  const bool wide = tree == 0;
  const long long nt = n_tri > 0 ? n_tri : 1;
  auto carve = [&](Carver& c, float*& v, int*& t, float*& o, float*& d, uint8_t*& h, int*& err,
                   Node*& nodes, Node4*& nodes4, Tri*& tris, BvhScratch& sc) {
    v = c.take<float>(3LL * (n_vert > 0 ? n_vert : 1));
    t = c.take<int>(3 * nt);
    o = c.take<float>(3LL * n_ray);
    d = c.take<float>(3LL * n_ray);
    h = c.take<uint8_t>(n_ray);
    err = c.take<int>(4);
    nodes = c.take<Node>(nt > 1 ? nt - 1 : 1);
    nodes4 = wide ? c.take<Node4>(nt > 1 ? nt - 1 : 1) : nullptr;
    tris = c.take<Tri>(nt);
    sc.keys = c.take<uint32_t>(nt);
    sc.vals = c.take<int32_t>(nt);
    sc.keys_alt = c.take<uint32_t>(nt);
    sc.vals_alt = c.take<int32_t>(nt);
    sc.cxy = c.take<float2>(nt);
    sc.parent = c.take<int>(nt);
    sc.nsize = c.take<int>(nt);
    sc.counter = c.take<int>(nt);
    sc.cost = c.take<float>(nt);
    sc.bounds = c.take<unsigned>(16);
    sc.sort_scratch = c.take<char>(radix_scratch_u32(nt));
  };
  float *v, *o, *d;
  int *t, *err;
  uint8_t* h;
  Node* nodes;
  Node4* nodes4;
  Tri* tris;
  BvhScratch sc;
  Carver dry(nullptr);
  carve(dry, v, t, o, d, h, err, nodes, nodes4, tris, sc);
  rc = E->reserve(dry.off, s);
  if (rc) return rc;
  Carver c(E->arena);
  carve(c, v, t, o, d, h, err, nodes, nodes4, tris, sc);
  if (n_vert > 0)
    HZ_CUDA(copy_from_host(E->staging, v, vert, sizeof(float) * 3 * (size_t)n_vert, s));
  if (n_tri > 0)
    HZ_CUDA(copy_from_host(E->staging, t, vertex_of_triangle, sizeof(int) * 3 * (size_t)n_tri,
                           s));
  HZ_CUDA(copy_from_host(E->staging, o, org, sizeof(float) * 3 * (size_t)n_ray, s));
  HZ_CUDA(copy_from_host(E->staging, d, dir, sizeof(float) * 3 * (size_t)n_ray, s));
  HZ_CUDA(cudaMemsetAsync(err, 0, 4 * sizeof(int), s));
  HZ_CUDA(bvh_build(v, t, n_tri, nodes, tris, sc, s, nullptr, nullptr, nodes4,
                    leaf_size > 0 ? leaf_size : kLeafMax));
  HZ_CUDA(trace_rays(nodes, nodes4, tris, n_tri > 0 ? 0 : kEmptyRef, o, d, n_ray, tfar, wide, h,
                     err, s));
  HZ_CUDA(copy_to_host(E->staging, hit, h, (size_t)n_ray, s));
  int err_h = 0;
  HZ_CUDA(cudaMemcpyAsync(&err_h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  HZ_CUDA(cudaStreamSynchronize(s));
  if (err_h & kErrStack) return fail(HZ_ERR_INTERNAL, "traversal stack overflow");
  return HZ_OK;
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
