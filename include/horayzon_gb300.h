/*
 * horayzon_gb300.h -- C ABI of the GB300 (sm_103a) terrain-horizon and
 * sky-view-factor library (libhorayzon_gb300.so).
 *
 * The library replaces the reference's horizon_svf_comp
 * (mo_lradtopo_horayzon.h:4-11, mo_lradtopo_horayzon.cpp:562-785) and the
 * Cython binding above it (horizon_svf.pyx:15-124). Inputs and outputs keep
 * the reference layouts:
 *
 *   clon, clat, hsurf   [num_cell]        FP64 cell circumcentres [rad], elevation [m]
 *   vlon, vlat          [num_vertex]      FP64 ICON vertices [rad]
 *   cells_of_vertex     [6][num_vertex]   int32, C order, -2 = no cell
 *   horizon             [num_hori][num_cell]  FP64 horizon angle [deg]
 *   skyview             [num_cell]        FP64 sky view factor [-]
 *
 * Every entry point except horizon_svf_comp returns a status (HZ_OK = 0) and
 * leaves a message for hz_last_error(). No entry point aborts the process.
 * Calls on one device are serialised by the library; the caller owns all
 * buffers. Internally each call builds the triangle mesh, the LBVH and runs
 * the horizon search on one GPU.
 */
#ifndef HORAYZON_GB300_H
#define HORAYZON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HZ_VERSION 100  /* 1.0.0 */

enum {
    HZ_OK = 0,
    HZ_ERR_VALUE = 1,     /* argument out of range (horizon_svf.pyx:79-103, ValueError) */
    HZ_ERR_TYPE = 2,      /* ray_org_elev < 0.1 (horizon_svf.pyx:98-99, TypeError) */
    HZ_ERR_INDEX = 3,     /* cells_of_vertex entry outside [0, num_cell) and != -2
                             (horizon_svf.pyx:88-90) */
    HZ_ERR_CUDA = 4,      /* CUDA runtime error (no device, out of memory, ...) */
    HZ_ERR_INTERNAL = 5   /* traversal-stack overflow or mesh capacity exceeded */
};

typedef struct hz_options {
    int32_t size;            /* sizeof(hz_options); filled by hz_default_options */
    int32_t device;          /* CUDA device ordinal; -1 = the calling thread's current device */
    int32_t count_work;      /* 1: also count BVH node visits and triangle tests */
    int32_t verbose;         /* 1: print the reference's progress lines to stdout */
    double elev_floor_deg;   /* lower bound of the downward elevation walk; the
                                reference's is -85 (mo_lradtopo_horayzon.cpp:578) */
    int32_t cell_begin;      /* trace only cells [cell_begin, cell_begin + cell_count); */
    int32_t cell_count;      /* cell_count <= 0: all cells. Other entries of horizon /
                                skyview are left untouched (multi-GPU cell shards). */
    int32_t kernel;          /* HZ_KERNEL_PERSISTENT (default) or HZ_KERNEL_PER_CELL */
    int32_t advance_min;     /* persistent kernel: lanes of a warp that must wait before
                                the search state advances (1..32; 0 = library default) */
    int32_t precision;       /* HZ_PRECISION_REFERENCE (default) or HZ_PRECISION_LOCAL */
    /* Learned warm start: host pointer to hz_mlp_num_params() FP32 parameters
       of the 32-64-64-1 MLP, or NULL for the reference's chained start. The
       bracket of the first azimuth of every cell (which the reference starts
       at 0 deg, cpp:511) -- or, with mlp_every_azimuth, of every azimuth --
       then starts at the MLP's proposal, and the same bracketing search
       refines it. Persistent kernel only. */
    const float* mlp_params;
    int32_t mlp_every_azimuth;
    /* Device outputs for training data (hz_horizon_svf_device, one domain):
       raw_index [L][num_cell] int16, the unclipped horizon of every azimuth in
       quarter degrees; features [L][num_cell][32] float, the MLP inputs. L =
       num_hori * refine_factor. NULL = not written. */
    int16_t* raw_index;
    float* features;
    int32_t leaf_min;        /* persistent kernel: lanes of a warp that must hold a
                                postponed leaf before a triangle pass (1..32; 0 =
                                library default) */
    int32_t leaf_size;       /* most triangles per BVH leaf (1..8; 0 = 2) */
    int32_t queue_chunk;     /* persistent kernel: consecutive cells (curve order) a
                                warp takes from the work queue at a time (0 = 32) */
    int32_t direct_launch;   /* 1: launch every kernel directly instead of replaying a
                                captured CUDA graph of the BVH build and search */
    /* Learned warm start: search items per cell. 0 or 1: one item runs the
       cell's azimuths as the reference's chain, the MLP's proposal starting
       the first one. G > 1 (a divisor of num_hori): G items of num_hori / G
       sectors each, every item starting at the proposal of its first
       azimuth, so that one cell's azimuths run on G lanes at once (small
       domains fill the GPU). -1: the library picks G per domain, the
       smallest divisor of num_hori that gives the call at least four search
       items per resident GPU thread (1 for domains that fill the GPU), at
       most num_hori / 2 (two azimuths per item). */
    int32_t mlp_azimuth_groups;
    /* Given warm start (hz_horizon_svf_device, one domain, in place of the
       MLP): device int16 [L][num_cell] lattice indices m of the starting
       elevation m * 0.5 deg (clamped to [-170, 180]), e.g. the horizons of
       an earlier run on the same grid in quarter degrees (raw_index) halved.
       Used like the MLP's proposals: at the first azimuth of each search
       item (mlp_azimuth_groups) or at every azimuth (mlp_every_azimuth).
       NULL = not used. */
    const int16_t* start_index;
    /* 1: restructure the binary BVH by treelets of 5 leaves (Karras & Aila,
       HPG 2013) before the 4-wide collapse; same results, tree quality
       only. 0 (default): the plain LBVH. */
    int32_t bvh_treelets;
    /* The downward elevation walk (mo_lradtopo_horayzon.cpp:536-547) once it
       is at or below +0.25 deg, where every further step gives a horizon
       clipped to 0 and only decides the elevation carried into the next
       azimuth: HZ_WALK_REFERENCE (default) one step per ray as the
       reference; HZ_WALK_BISECT doubling steps then bisection for the same
       stop, which it finds wherever the rays below it hit and those above
       it miss (visibility monotone in elevation) -- then the outputs are the
       reference's, from fewer rays (hz_stats.num_rays counts the rays cast).
       Persistent kernel only. */
    int32_t elev_walk;
    /* 1 (default): an upward step of the elevation walk first tests the
       triangle that hid the ray one step below; the query is any-hit, so a
       hit there is the full traversal's answer and the tree is not
       traversed for that ray. Same results, same ray count; 0 traverses
       every ray. Persistent kernels; the per-cell kernel ignores it. */
    int32_t occluder_cache;
} hz_options;

enum {
    HZ_WALK_REFERENCE = 0,
    HZ_WALK_BISECT = 1
};

enum {
    /* FP32 vertices and ray origins in one global ENU frame, as the reference
       traces them (mo_lradtopo_horayzon.cpp:403-410, 715-720): identical rays
       and hit decisions. */
    HZ_PRECISION_REFERENCE = 0,
    /* Vertices and ray origins kept as FP32 hi + lo pairs of their FP64 ENU
       values; each ray intersects FP32 vectors relative to its cell's FP64
       origin, which removes the centimetre-scale quantisation of the global
       FP32 frame. Persistent kernel only. */
    HZ_PRECISION_LOCAL = 1
};

enum {
    HZ_KERNEL_PERSISTENT = 0,  /* persistent search over Hilbert-ordered cells on a 4-wide
                                  BVH, warp-uniform loop, postponed leaves tested one
                                  triangle per pass */
    HZ_KERNEL_PER_CELL = 1,    /* one thread per cell, nested loops, binary BVH */
    HZ_KERNEL_PERSISTENT_BVH2 = 2  /* the persistent search on the binary BVH (same rays
                                      and results; its node visits are the binary-tree
                                      counts) */
};

typedef struct hz_stats {
    int64_t num_rays;        /* rays cast (reference prints it, cpp:769) */
    int64_t node_visits;     /* with count_work: BVH internal-node visits */
    int64_t tri_tests;       /* with count_work: ray/triangle tests */
    int32_t n_tri;           /* triangles in the mesh (cpp:314-315) */
    int32_t n_mesh_vert;     /* mesh vertices: cells + appended ICON vertices */
    /* Phase times: CUDA events on the stream that carries the work (nodes
     * of the call's graph, or the caller's stream when launched directly). */
    double ms_h2d;           /* host->device copies (host entry points) */
    double ms_mesh;          /* mesh assembly + geodetic frames */
    double ms_bvh;           /* LBVH build */
    double ms_trace;         /* learned start if any, frames, search, outputs */
    double ms_d2h;           /* device->host copies (host entry points) */
    double ms_total;         /* whole call, wall clock */
    int64_t kernel_launches; /* CUDA kernels this call launched */
} hz_stats;

/*
 * Distance of every cell circumcentre to the mesh border, replacing
 * functions.distance_to_border (functions.py:58-97): the chord distance [km]
 * on a sphere of radius 6371.0087714 km from each cell to the nearest ICON
 * vertex that has a missing neighbour cell (a -2 in cells_of_vertex); +inf
 * when no vertex has one. Arrays as in horizon_svf_comp; dist[num_cell].
 * on_device != 0: all pointers are device pointers and the work runs on
 * `stream`; otherwise host pointers.
 */
int hz_distance_to_border(const double* clon, const double* clat,
                          const double* vlon, const double* vlat,
                          const int32_t* cells_of_vertex, int num_cell,
                          int num_vertex, double* dist, int on_device,
                          void* stream);

/* Fills *opt with the defaults (device -1, elev_floor_deg -85, counters off). */
void hz_default_options(hz_options* opt);

/*
 * Drop-in for the reference function of the same name and signature
 * (mo_lradtopo_horayzon.h:4-11, mo_lradtopo_horayzon.cpp:562-569), with C
 * linkage so that Fortran (ISO_C_BINDING) and ctypes can bind it, as the
 * commented extern "C" at mo_lradtopo_horayzon.cpp:561 intends. Host buffers.
 * Like the reference it returns nothing; on an error it prints
 * hz_last_error() to stderr and fills horizon and skyview with NaN.
 */
void horizon_svf_comp(double* clon, double* clat, double* hsurf,
                      double* vlon, double* vlat,
                      int* cells_of_vertex,
                      double* horizon, double* skyview,
                      int num_cell, int num_vertex, int num_hori,
                      int grid_type, double dist_search,
                      double ray_org_elev, int refine_factor,
                      int svf_type);

/*
 * The reference's dormant Fortran variant (mo_lradtopo_horayzon.cpp:561-574,
 * 778-784): the same computation, with the progress lines that
 * horizon_svf_comp prints (with HZ_VERBOSE=1) captured into the caller's
 * buffer instead of stdout. On entry *buffer_len is the buffer's capacity; on
 * return it is the number of bytes written (the first *buffer_len bytes of
 * the text, no terminating NUL). Errors append "horizon_svf_comp: <message>"
 * to the text and fill horizon and skyview with NaN.
 */
void horizon_svf_comp_buffer(double* clon, double* clat, double* hsurf,
                             double* vlon, double* vlat,
                             int* cells_of_vertex,
                             double* horizon, double* skyview,
                             int num_cell, int num_vertex, int num_hori,
                             int grid_type, double dist_search,
                             double ray_org_elev, int refine_factor,
                             int svf_type, char* buffer, int* buffer_len);

/*
 * Same computation with a status, options and statistics. Host buffers; the
 * arguments are validated as horizon_svf.pyx:79-103 does. opt and stats may
 * be NULL.
 */
int hz_horizon_svf(const double* clon, const double* clat, const double* hsurf,
                   const double* vlon, const double* vlat,
                   const int32_t* cells_of_vertex,
                   double* horizon, double* skyview,
                   int num_cell, int num_vertex, int num_hori,
                   int grid_type, double dist_search,
                   double ray_org_elev, int refine_factor, int svf_type,
                   const hz_options* opt, hz_stats* stats);

/*
 * Same as hz_horizon_svf with every array already in device memory of the
 * selected device. Work is enqueued on `stream` (a cudaStream_t; NULL = the
 * legacy default stream) and the call returns when it has completed. No
 * reference counterpart: it lets callers that keep fields on the GPU skip the
 * host round trip of horizon_svf.pyx:106-122.
 */
int hz_horizon_svf_device(const double* clon, const double* clat, const double* hsurf,
                          const double* vlon, const double* vlat,
                          const int32_t* cells_of_vertex,
                          double* horizon, double* skyview,
                          int num_cell, int num_vertex, int num_hori,
                          int grid_type, double dist_search,
                          double ray_org_elev, int refine_factor, int svf_type,
                          void* stream, const hz_options* opt, hz_stats* stats);

/* One regional domain of a batch call (same layouts as hz_horizon_svf). */
typedef struct hz_domain {
    const double* clon;
    const double* clat;
    const double* hsurf;
    const double* vlon;
    const double* vlat;
    const int32_t* cells_of_vertex;
    double* horizon;
    double* skyview;
    int32_t num_cell, num_vertex, num_hori, grid_type;
    double dist_search, ray_org_elev;
    int32_t refine_factor, svf_type;
    double latency_ms;       /* out: completion time of the domain's last cell,
                                measured from the start of the search launch */
} hz_domain;

/*
 * Many independent domains in one call: mesh, frames and BVH per domain
 * (each BVH in its own slice of one device arena), then ONE persistent
 * search launch over the cells of all domains. Every domain carries its own
 * arguments (num_hori, grid_type, ...); 1 <= n_domains <= 65535. on_device
 * = 0: host arrays (copied in and out); on_device = 1: device arrays, work
 * enqueued on `stream`. The search takes the domains in ascending order of
 * work (cells x azimuths), so small domains complete first (latency_ms).
 * No reference counterpart: the reference computes one domain per call
 * (mo_lradtopo_horayzon.cpp:562-785).
 */
int hz_horizon_svf_batch(hz_domain* domains, int n_domains, int on_device, void* stream,
                         const hz_options* opt, hz_stats* stats);

/*
 * Any-hit occlusion of arbitrary rays against a triangle soup: the query the
 * search makes for every ray (Embree's rtcOccluded1 with the reference's ray
 * setup, mo_lradtopo_horayzon.cpp:446-460), built and traced with the same
 * BVH build, box tests, traversal and watertight triangle test. vert: FP32
 * [n_vert][3]; vertex_of_triangle: int32 [n_tri][3]; org, dir: FP32
 * [n_ray][3] (dir need not be unit length); hit[i] = 1 when ray i meets a
 * triangle at 0 < t <= tfar, t in units of |dir|. Host buffers. tree: 0 =
 * the 4-wide BVH of the persistent search, 1 = the binary BVH; leaf_size:
 * triangles per leaf (0 = 2). No reference counterpart as an entry point.
 */
int hz_occluded32(const float* vert, int n_vert, const int32_t* vertex_of_triangle, int n_tri,
                  const float* org, const float* dir, int n_ray, float tfar, uint8_t* hit,
                  int tree, int leaf_size, int device);

/*
 * Triangle-mesh assembly alone (mo_lradtopo_horayzon.cpp:228-317), on the
 * GPU, host buffers: mesh vertex (lon, lat, elevation) for the cells followed
 * by the appended ICON vertices, and three vertex indices per triangle.
 * Capacities: cap_vert >= num_cell + num_vertex, cap_tri >= 6 * num_vertex.
 */
int hz_build_mesh(const double* clon, const double* clat, const double* hsurf,
                  const double* vlon, const double* vlat,
                  const int32_t* cells_of_vertex, int num_cell, int num_vertex,
                  int grid_type, double* mesh_lon, double* mesh_lat, double* mesh_h,
                  int cap_vert, int32_t* vertex_of_triangle, int cap_tri,
                  int* n_mesh_vert, int* n_tri, int device);

/*
 * The FP32 vertices in the domain's ENU frame that rays are intersected with
 * (mo_lradtopo_horayzon.cpp:611-644, 403-410), plus the triangle list.
 * Capacities as for hz_build_mesh; enu32 holds 3 * cap_vert floats.
 */
int hz_mesh_enu32(const double* clon, const double* clat, const double* hsurf,
                  const double* vlon, const double* vlat,
                  const int32_t* cells_of_vertex, int num_cell, int num_vertex,
                  int grid_type, float* enu32, int cap_vert,
                  int32_t* vertex_of_triangle, int cap_tri,
                  int* n_mesh_vert, int* n_tri, int device);

/*
 * No counterpart in the reference. The same computation as
 * hz_horizon_svf_device (device pointers, `stream` a cudaStream_t or NULL)
 * for callers that cannot allocate GPU memory -- for example a model whose
 * device memory is all owned by another allocator, or a time-stepping code
 * on a shared GPU that cannot afford the device-wide synchronisation of
 * cudaMalloc/cudaFree. It allocates nothing: all intermediate data lives in
 * one fixed 64 MiB __device__ array inside the library (held by every GPU
 * that loads it until the process exits). That limits a domain to about
 * 90,000 cells with grid_type 1 and 120,000 with grid_type 0, at ICON's ratio
 * of one vertex per two cells (the scratch is about 700 bytes per cell, or
 * 540 with grid_type 0); larger domains are rejected with HZ_ERR_VALUE and a
 * message naming the limit. The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress) with that device current and keeps
 * it; after a cudaDeviceReset call hz_release_workspace(device), which
 * forgets it. The function cannot be called while `stream` is being
 * captured: it reads results back to the host and waits for the stream
 * mid-call. All calls share the array: calls whose GPU work overlapped would
 * race on it, so the function serialises its callers, and every return after
 * its first queued operation (success or error) waits for the work on
 * `stream` to finish. The down-walk bound is the reference's -85 deg; errors
 * are reported through hz_last_error().
 */
int hz_horizon_svf_device_static(const double* clon, const double* clat,
                                 const double* hsurf, const double* vlon,
                                 const double* vlat, const int32_t* cells_of_vertex,
                                 double* horizon, double* skyview,
                                 int num_cell, int num_vertex, int num_hori,
                                 int grid_type, double dist_search,
                                 double ray_org_elev, int refine_factor, int svf_type,
                                 void* stream);

/*
 * Learned warm start, no reference counterpart. Parameters are packed FP32:
 * W1[32][64], b1[64], W2[64][64], b2[64], W3[64], b3; the forward pass rounds
 * them to BF16 and accumulates in FP32 (ReLU hidden layers). Targets are the
 * horizon in units of 8 deg (quarter-degree index / 32). All arrays are
 * device pointers; work runs on `stream` and the call returns when it is done.
 */
int hz_mlp_num_params(void);
/* One training step on n samples X[n][32], T[n]: writes the mean-squared-error
 * loss to *loss and the gradient to grads[hz_mlp_num_params()]; with lr > 0
 * also an Adam step (beta 0.9 / 0.999, eps 1e-8, step >= 1) on params using
 * the moment buffers adam_m, adam_v. */
int hz_mlp_train_step(float* params, float* adam_m, float* adam_v, const float* X,
                      const float* T, int n, int step, float lr, float* loss, float* grads,
                      void* stream);
/* Y[n] = MLP(X[n][32]). */
int hz_mlp_forward(const float* params, const float* X, int n, float* Y, void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* hz_last_error(void);

/* HZ_VERSION of the loaded library. */
int hz_version(void);

/* Frees the cached device workspace of `device` (-1 = all devices) and
 * forgets the cached address of hz_horizon_svf_device_static's array there. */
int hz_release_workspace(int device);

#ifdef __cplusplus
}
#endif
#endif /* HORAYZON_GB300_H */
