/*
 * hz_oracle.h -- C interface of the CPU oracle (hz_oracle.c).
 *
 * TEST INFRASTRUCTURE: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py only, as the checker of the CUDA path.
 */
#ifndef HZ_ORACLE_H
#define HZ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int precision;          /* 0: FP32 rays in one global ENU frame (reference),
                               1: FP64 vertices, rays and triangle test */
    int nthreads;           /* worker threads, 0 = all online CPUs */
    const int32_t* cells;   /* optional subset of cells to trace (NULL = all) */
    int n_cells;            /* length of `cells` */
    double elev_floor_deg;  /* lower bound of the downward walk (reference: -85) */
    int brute_force;        /* 1: test every triangle instead of the BVH */
    /* Optional warm start (the GPU library's learned / given start): lattice
       indices start_m[L][ncell] (elevation m * 0.5 deg, clamped to
       [-170, 180]). Each cell's azimuths form `groups` runs of L / groups;
       a run's first azimuth starts at its index instead of the chained
       elevation (the reference's first azimuth starts at 0, cpp:511), or
       every azimuth does with start_all. NULL = the reference's chain. */
    const int16_t* start_m;
    int groups;
    int start_all;
    /* 1: the GPU library's HZ_WALK_BISECT: a downward walk at or below the
       clip (elevation <= hori_acc) finds its stop by doubling steps then
       bisection, the rays at intermediate steps rotated but not cast; 0 =
       the reference's step walk. */
    int bisect_walk;
} hzo_options;

typedef struct {
    int64_t num_rays;       /* rays cast (reference: cpp:524-544, printed :769) */
    int64_t node_visits;    /* BVH internal-node visits over all rays */
    int64_t tri_tests;      /* ray/triangle tests over all rays */
    int64_t overflow;       /* traversal-stack overflows (0 expected) */
    int n_tri;              /* triangles in the mesh */
    int n_mesh_vert;        /* mesh vertices (cells + appended ICON vertices) */
    double t_mesh;          /* seconds: mesh assembly + frames */
    double t_bvh;           /* seconds: BVH build */
    double t_rays;          /* seconds: horizon search + SVF */
} hzo_result;

void hzo_default_options(hzo_options* opt);

/* mo_lradtopo_horayzon.cpp:228-317. Capacities: mesh arrays >= ncell + nvert,
 * vot >= 18 * nvert (grid_type 1) or 12 * nvert (grid_type 0). */
int hzo_build_mesh(const double* clon, const double* clat, const double* hsurf,
                   const double* vlon, const double* vlat, const int32_t* cov,
                   int ncell, int nvert, int grid_type,
                   double* mlon, double* mlat, double* mh, int cap_vert,
                   int32_t* vot, int cap_tri, int* n_mesh_vert, int* n_tri);

/* Mesh vertices in the global ENU frame (mo_lradtopo_horayzon.cpp:611-644),
 * both as the FP64 values and as the FP32 copy the reference traces against
 * (cpp:403-410). Capacities as for hzo_build_mesh. */
int hzo_mesh_enu(const double* clon, const double* clat, const double* hsurf,
                 const double* vlon, const double* vlat, const int32_t* cov,
                 int ncell, int nvert, int grid_type,
                 double* enu64, float* enu32, int cap_vert,
                 int32_t* vot, int cap_tri, int* n_mesh_vert, int* n_tri);

/* Full horizon + SVF path (mo_lradtopo_horayzon.cpp:562-785). */
int hzo_horizon_svf(const double* clon, const double* clat, const double* hsurf,
                    const double* vlon, const double* vlat, const int32_t* cov,
                    double* horizon, double* skyview,
                    int ncell, int nvert, int nhori, int grid_type,
                    double dist_search, double ray_org_elev, int refine_factor,
                    int svf_type, const hzo_options* opt, hzo_result* res);

/* One occlusion query against a mesh given by FP32 vertices (tests). */
int hzo_occluded32(const float* vert, const int32_t* vot, int n_tri,
                   const float* org, const float* dir, float tfar, int n_ray,
                   int brute_force, uint8_t* hit);

#ifdef __cplusplus
}
#endif
#endif
