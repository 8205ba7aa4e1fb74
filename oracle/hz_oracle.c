/*
 * hz_oracle.c -- CPU oracle of the HORAYZON terrain-horizon / sky-view-factor
 * path.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs load this library, as the checker of the CUDA path (and,
 * on machines where the reference itself cannot be compiled, as its timed CPU
 * stand-in). The product (horayzon_extpar_gb300) never links or calls it.
 *
 * It restates the reference algorithm, mo_lradtopo_horayzon.cpp:
 *   deg2rad / rad2deg ................. cpp:59-70
 *   dot / cross / unit / Rodrigues .... cpp:78-130
 *   sort_index ........................ cpp:137-146 (insertion sort: std::sort
 *                                       on <= 16 elements is an insertion sort)
 *   lonlat2ecef / ecef2enu_point ...... cpp:158-201
 *   build_triangle_mesh ............... cpp:228-317
 *   SVF kernels ....................... cpp:333-358
 *   ENU origin and frames ............. cpp:611-644
 *   per-cell frame and ray origin ..... cpp:694-722
 *   terrain_horizon ................... cpp:490-555
 *   clip, sector mean, SVF ............ cpp:736-754
 *   tbb::parallel_reduce over cells ... cpp:686-761 (pthreads here)
 * with the ray query of hz_occlusion.h in place of Embree's rtcOccluded1.
 * Every floating-point expression keeps the reference's operation order; the
 * file is compiled with -ffp-contract=off.
 *
 * One intentional difference: build_triangle_mesh indexes cells_of_vertex by
 * the position of a cell among the *valid* entries of a vertex (cpp:265-271,
 * 304-306). That equals the slot whenever a vertex's -2 entries trail its valid
 * ones; any other layout makes the reference read index -2 (undefined). Here the
 * sorted positions are mapped back to their slots, which agrees with the
 * reference on every input where the reference is defined.
 */
#define _GNU_SOURCE
#include "hz_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <time.h>
#include <unistd.h>

#include "hz_occlusion.h"
#define HZO_REAL float
#define HZO_SFX 32
#include "hz_occlusion.h"
#undef HZO_REAL
#undef HZO_SFX
#define HZO_REAL double
#define HZO_SFX 64
#include "hz_occlusion.h"
#undef HZO_REAL
#undef HZO_SFX

typedef struct { double x, y, z; } v3d;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* cpp:59-70 */
static inline double deg2rad(double ang) { return ((ang / 180.0) * M_PI); }
static inline double rad2deg(double ang) { return ((ang / M_PI) * 180.0); }

/* cpp:78-130 */
static inline double dot3(v3d a, v3d b) { return (a.x * b.x + a.y * b.y + a.z * b.z); }
static inline v3d cross3(v3d a, v3d b) {
    v3d c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return c;
}
static inline void unit3(v3d* a) {
    double m = sqrt(a->x * a->x + a->y * a->y + a->z * a->z);
    a->x /= m;
    a->y /= m;
    a->z /= m;
}
static inline v3d rotate3(v3d v, v3d k, double s, double c) {
    v3d r;
    double term = dot3(k, v) * (1.0 - c);
    r.x = v.x * c + (k.y * v.z - k.z * v.y) * s + k.x * term;
    r.y = v.y * c + (k.z * v.x - k.x * v.z) * s + k.y * term;
    r.z = v.z * c + (k.x * v.y - k.y * v.x) * s + k.z * term;
    return r;
}

void hzo_default_options(hzo_options* opt) {
    memset(opt, 0, sizeof(*opt));
    opt->elev_floor_deg = -85.0;
}

/* cpp:228-317 */
int hzo_build_mesh(const double* clon, const double* clat, const double* hsurf,
                   const double* vlon, const double* vlat, const int32_t* cov,
                   int ncell, int nvert, int grid_type,
                   double* mlon, double* mlat, double* mh, int cap_vert,
                   int32_t* vot, int cap_tri, int* n_mesh_vert, int* n_tri) {
    if (cap_vert < ncell) return -1;
    for (int i = 0; i < ncell; i++) {
        mlon[i] = clon[i];
        mlat[i] = clat[i];
        mh[i] = hsurf[i];
    }
    int ntri = 0, nmv = ncell;
    for (int v = 0; v < nvert; v++) {
        double ang[6];
        int slot[6];
        int n = 0;
        double hsum = 0.0;
        for (int j = 0; j < 6; j++) {
            int c = cov[(size_t)nvert * j + v];
            if (c != -2) {
                double a = atan2(clon[c] - vlon[v], clat[c] - vlat[v]);
                if (a < 0.0) a += 2.0 * M_PI;
                ang[n] = a;
                slot[n] = j;
                n++;
                hsum += hsurf[c];
            }
        }
        /* sort_index (cpp:137-146): stable ascending order of angles */
        int ord[6];
        for (int k = 0; k < n; k++) ord[k] = k;
        for (int k = 1; k < n; k++) {
            int x = ord[k];
            int m = k - 1;
            while (m >= 0 && ang[x] < ang[ord[m]]) { ord[m + 1] = ord[m]; m--; }
            ord[m + 1] = x;
        }
        int cs[6];
        for (int k = 0; k < n; k++) cs[k] = cov[(size_t)nvert * slot[ord[k]] + v];
        if (grid_type == 0) {
            if (n >= 3) {
                for (int k = 0; k < n - 2; k++) {
                    if (ntri >= cap_tri) return -2;
                    vot[3 * (size_t)ntri + 0] = cs[0];
                    vot[3 * (size_t)ntri + 1] = cs[k + 1];
                    vot[3 * (size_t)ntri + 2] = cs[k + 2];
                    ntri++;
                }
            }
        } else if (n == 6) {
            if (nmv >= cap_vert) return -1;
            mlon[nmv] = vlon[v];
            mlat[nmv] = vlat[v];
            mh[nmv] = hsum / 6.0;
            static const int ind[7] = {0, 1, 2, 3, 4, 5, 0};
            for (int k = 0; k < 6; k++) {
                if (ntri >= cap_tri) return -2;
                vot[3 * (size_t)ntri + 0] = cs[ind[k]];
                vot[3 * (size_t)ntri + 1] = cs[ind[k + 1]];
                vot[3 * (size_t)ntri + 2] = nmv;
                ntri++;
            }
            nmv++;
        }
    }
    *n_mesh_vert = nmv;
    *n_tri = ntri;
    return 0;
}

typedef struct {
    double lon_orig, lat_orig;
    v3d centre, pole; /* Earth centre and North Pole in ENU */
} enu_frame;

/* cpp:158-169 followed by cpp:611-644 on the first ncell (cell) vertices */
static void mesh_to_enu(const double* mlon, const double* mlat, const double* mh,
                        int nmv, int ncell, double* enu, enu_frame* fr) {
    const double R = 6371229.0; /* cpp:584 */
    for (int i = 0; i < nmv; i++) {
        double sin_lon = sin(mlon[i]), cos_lon = cos(mlon[i]);
        double sin_lat = sin(mlat[i]), cos_lat = cos(mlat[i]);
        double e = mh[i];
        enu[3 * (size_t)i + 0] = (R + e) * cos_lat * cos_lon;
        enu[3 * (size_t)i + 1] = (R + e) * cos_lat * sin_lon;
        enu[3 * (size_t)i + 2] = (R + e) * sin_lat;
    }
    double xo = 0.0, yo = 0.0, zo = 0.0;
    for (int i = 0; i < ncell; i++) {
        xo += enu[3 * (size_t)i + 0];
        yo += enu[3 * (size_t)i + 1];
        zo += enu[3 * (size_t)i + 2];
    }
    double radius = sqrt(xo * xo + yo * yo + zo * zo);
    double lon_o = atan2(yo, xo);
    double lat_o = asin(zo / radius);
    fr->lon_orig = lon_o;
    fr->lat_orig = lat_o;
    /* cpp:178-201 */
    double sin_lon = sin(lon_o), cos_lon = cos(lon_o);
    double sin_lat = sin(lat_o), cos_lat = cos(lat_o);
    double xe = R * cos(lat_o) * cos(lon_o);
    double ye = R * cos(lat_o) * sin(lon_o);
    double ze = R * sin(lat_o);
    double pts[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, R}};
    for (int i = 0; i < nmv + 2; i++) {
        double* p = i < nmv ? enu + 3 * (size_t)i : pts[i - nmv];
        double x = p[0], y = p[1], z = p[2];
        double xn = -sin_lon * (x - xe) + cos_lon * (y - ye);
        double yn = -sin_lat * cos_lon * (x - xe) - sin_lat * sin_lon * (y - ye)
                    + cos_lat * (z - ze);
        double zn = +cos_lat * cos_lon * (x - xe) + cos_lat * sin_lon * (y - ye)
                    + sin_lat * (z - ze);
        p[0] = xn;
        p[1] = yn;
        p[2] = zn;
    }
    fr->centre = (v3d){pts[0][0], pts[0][1], pts[0][2]};
    fr->pole = (v3d){pts[1][0], pts[1][1], pts[1][2]};
}

int hzo_mesh_enu(const double* clon, const double* clat, const double* hsurf,
                 const double* vlon, const double* vlat, const int32_t* cov,
                 int ncell, int nvert, int grid_type,
                 double* enu64, float* enu32, int cap_vert,
                 int32_t* vot, int cap_tri, int* n_mesh_vert, int* n_tri) {
    double* mlon = malloc(sizeof(double) * (size_t)cap_vert);
    double* mlat = malloc(sizeof(double) * (size_t)cap_vert);
    double* mh = malloc(sizeof(double) * (size_t)cap_vert);
    if (!mlon || !mlat || !mh) { free(mlon); free(mlat); free(mh); return -3; }
    int rc = hzo_build_mesh(clon, clat, hsurf, vlon, vlat, cov, ncell, nvert,
                            grid_type, mlon, mlat, mh, cap_vert, vot, cap_tri,
                            n_mesh_vert, n_tri);
    if (rc == 0) {
        enu_frame fr;
        mesh_to_enu(mlon, mlat, mh, *n_mesh_vert, ncell, enu64, &fr);
        for (size_t i = 0; i < 3 * (size_t)*n_mesh_vert; i++)
            enu32[i] = (float)enu64[i];
    }
    free(mlon); free(mlat); free(mh);
    return rc;
}

/* ------------------------------------------------------------------------- */

typedef struct {
    /* inputs */
    const double* enu;       /* FP64 ENU of mesh vertices; cells first */
    enu_frame fr;
    const hzo_bvh_32* bvh32;
    const hzo_bvh_64* bvh64;
    int precision, brute;
    double* horizon;
    double* skyview;
    int ncell, nhori, refine, svf_type;
    double dist_search, ray_org_elev;
    double hori_acc, elev_floor;
    double azim_sin, azim_cos, elev_sin_2ha, elev_cos_2ha, azim_shift;
    const int32_t* cells;
    int n_work;
    const int16_t* start_m;
    int groups, start_all, bisect_walk;
    atomic_int next;
    /* per-run totals */
    atomic_llong rays, nodes, tris, overflow;
} trace_job;

static int cast_ray(const trace_job* J, const v3d* o64, const float* o32, v3d dir,
                    hzo_counts* cnt) {
    if (J->precision == 0) {
        float d[3] = {(float)dir.x, (float)dir.y, (float)dir.z};
        hzo_ray_32 r;
        hzo_ray_setup_32(&r, o32, d, 0.0f, (float)J->dist_search);
        return J->brute ? hzo_occluded_brute_32(J->bvh32, &r, cnt)
                        : hzo_occluded_32(J->bvh32, &r, cnt);
    }
    double o[3] = {o64->x, o64->y, o64->z};
    double d[3] = {dir.x, dir.y, dir.z};
    hzo_ray_64 r;
    hzo_ray_setup_64(&r, o, d, 0.0, J->dist_search);
    return J->brute ? hzo_occluded_brute_64(J->bvh64, &r, cnt)
                    : hzo_occluded_64(J->bvh64, &r, cnt);
}

/* cpp:694-754 for one cell, with terrain_horizon (cpp:490-555) inlined and
 * the clip / sector mean / SVF of cpp:736-754 accumulated per azimuth. */
static int64_t trace_cell(const trace_job* J, int i, hzo_counts* cnt) {
    const double* p = J->enu + 3 * (size_t)i;
    v3d normal = {p[0] - J->fr.centre.x, p[1] - J->fr.centre.y, p[2] - J->fr.centre.z};
    unit3(&normal);
    v3d v_n = {J->fr.pole.x - p[0], J->fr.pole.y - p[1], J->fr.pole.z - p[2]};
    double dp = dot3(v_n, normal);
    v3d north = {v_n.x - dp * normal.x, v_n.y - dp * normal.y, v_n.z - dp * normal.z};
    unit3(&north);
    float o32[3] = {(float)(p[0] + normal.x * J->ray_org_elev),
                    (float)(p[1] + normal.y * J->ray_org_elev),
                    (float)(p[2] + normal.z * J->ray_org_elev)};
    v3d o64 = {p[0] + normal.x * J->ray_org_elev, p[1] + normal.y * J->ray_org_elev,
               p[2] + normal.z * J->ray_org_elev};

    const int L = J->nhori * J->refine;
    const double ha = J->hori_acc;
    int64_t rays = 0;
    v3d dir = rotate3(north, normal, sin(-J->azim_shift), cos(-J->azim_shift));
    double elev = 0.0;
    double sector = 0.0, svf = 0.0;
    const int span = J->groups > 1 ? L / J->groups : L;
    const v3d east = cross3(north, normal);
    for (int a = 0; a < L; a++) {
        if (J->start_m && (J->start_all || a % span == 0)) {
            /* Warm start: lattice elevation m at azimuth a, the direction in
             * closed form cos(e) h_a + sin(e) U with the horizontal direction
             * h_a = cos(theta_a) N + sin(theta_a) E (the GPU library's form). */
            int m = J->start_m[(size_t)a * J->ncell + i];
            m = m < -170 ? -170 : (m > 180 ? 180 : m);
            elev = (double)m * (2.0 * ha);
            const double th = J->azim_shift + (double)a * ((2.0 * M_PI) / (double)L);
            const double ct = cos(th), st = sin(th), ce = cos(elev), se = sin(elev);
            const v3d hz = {ct * north.x + st * east.x, ct * north.y + st * east.y,
                            ct * north.z + st * east.z};
            dir.x = ce * hz.x + se * normal.x;
            dir.y = ce * hz.y + se * normal.y;
            dir.z = ce * hz.z + se * normal.z;
        }
        v3d axis = cross3(dir, normal);
        unit3(&axis);
        int hit = cast_ray(J, &o64, o32, dir, cnt);
        rays++;
        double h;
        if (hit) {
            /* The reference's walk never ends for an origin enclosed by the
             * mesh; both implementations stop after one turn (720 steps). */
            int up = 0;
            while (hit && up++ < 720) {
                elev += (2.0 * ha);
                dir = rotate3(dir, axis, J->elev_sin_2ha, J->elev_cos_2ha);
                hit = cast_ray(J, &o64, o32, dir, cnt);
                rays++;
            }
            h = elev - ha;
        } else {
            /* With bisect_walk the step walk stops at the clip (elev <= ha),
             * where every further candidate's horizon is clipped to 0. */
            while ((!hit) && (elev > J->elev_floor) && !(J->bisect_walk && elev <= ha)) {
                elev -= (2.0 * ha);
                dir = rotate3(dir, axis, -J->elev_sin_2ha, J->elev_cos_2ha);
                hit = cast_ray(J, &o64, o32, dir, cnt);
                rays++;
            }
            if (!hit && elev > J->elev_floor) {
                /* The stop of the step walk from e0 = elev: the first k with
                 * a hit, or K (the first step at or below the floor). Probe
                 * k = 1, 2, 4, ... then bisect; the direction of step k is
                 * the step walk's, k incremental rotations from e0. */
                int K = 0;
                double e = elev;
                do {
                    e -= (2.0 * ha);
                    K++;
                } while (e > J->elev_floor);
                const v3d d0 = dir;
                int lo = 0, hi = K + 1, next = 1;
                while (next > 0) {
                    v3d d = d0;
                    for (int q = 0; q < next; q++)
                        d = rotate3(d, axis, -J->elev_sin_2ha, J->elev_cos_2ha);
                    if (cast_ray(J, &o64, o32, d, cnt)) hi = next;
                    else lo = next;
                    rays++;
                    if (hi > K) next = lo >= K ? 0 : (2 * lo > K ? K : (2 * lo < 1 ? 1 : 2 * lo));
                    else next = hi - lo > 1 ? (lo + hi) / 2 : 0;
                }
                const int ks = hi > K ? K : hi;
                for (int q = 0; q < ks; q++) {
                    elev -= (2.0 * ha);
                    dir = rotate3(dir, axis, -J->elev_sin_2ha, J->elev_cos_2ha);
                }
            }
            h = elev + ha;
        }
        dir = rotate3(dir, normal, -J->azim_sin, J->azim_cos);
        if (h < 0.0) h = 0.0;
        sector += h;
        if ((a + 1) % J->refine == 0) {
            int j = a / J->refine;
            J->horizon[(size_t)j * J->ncell + i] = rad2deg(sector) / (double)J->refine;
            sector = 0.0;
        }
        double s = sin(h);
        if (J->svf_type == 0) svf += (1.0 - s);
        else if (J->svf_type == 1) svf += (1.0 - (s * s));
        else svf += (1.0 - (s * s * s));
    }
    J->skyview[i] = svf / (double)L;
    return rays;
}

static void* trace_worker(void* arg) {
    trace_job* J = (trace_job*)arg;
    hzo_counts cnt = {0, 0, 0};
    int64_t rays = 0;
    const int chunk = 64;
    for (;;) {
        int s = atomic_fetch_add(&J->next, chunk);
        if (s >= J->n_work) break;
        int e = s + chunk < J->n_work ? s + chunk : J->n_work;
        for (int k = s; k < e; k++) {
            int i = J->cells ? J->cells[k] : k;
            rays += trace_cell(J, i, &cnt);
        }
    }
    atomic_fetch_add(&J->rays, rays);
    atomic_fetch_add(&J->nodes, cnt.node_visits);
    atomic_fetch_add(&J->tris, cnt.tri_tests);
    atomic_fetch_add(&J->overflow, cnt.overflow);
    return NULL;
}

int hzo_horizon_svf(const double* clon, const double* clat, const double* hsurf,
                    const double* vlon, const double* vlat, const int32_t* cov,
                    double* horizon, double* skyview,
                    int ncell, int nvert, int nhori, int grid_type,
                    double dist_search, double ray_org_elev, int refine_factor,
                    int svf_type, const hzo_options* opt_in, hzo_result* res) {
    hzo_options opt;
    if (opt_in) opt = *opt_in; else hzo_default_options(&opt);
    memset(res, 0, sizeof(*res));
    if (ncell <= 0 || nvert < 0 || nhori < 1 || refine_factor < 1) return -1;
    double t0 = now_s();
    int cap_vert = ncell + nvert;
    int cap_tri = 6 * nvert;
    double* mlon = malloc(sizeof(double) * (size_t)cap_vert);
    double* mlat = malloc(sizeof(double) * (size_t)cap_vert);
    double* mh = malloc(sizeof(double) * (size_t)cap_vert);
    double* enu = malloc(sizeof(double) * 3 * (size_t)cap_vert);
    int32_t* vot = malloc(sizeof(int32_t) * 3 * (size_t)(cap_tri > 0 ? cap_tri : 1));
    if (!mlon || !mlat || !mh || !enu || !vot) {
        free(mlon); free(mlat); free(mh); free(enu); free(vot);
        return -3;
    }
    int nmv = 0, ntri = 0;
    int rc = hzo_build_mesh(clon, clat, hsurf, vlon, vlat, cov, ncell, nvert,
                            grid_type, mlon, mlat, mh, cap_vert, vot, cap_tri,
                            &nmv, &ntri);
    if (rc != 0) {
        free(mlon); free(mlat); free(mh); free(enu); free(vot);
        return rc;
    }
    trace_job J;
    memset(&J, 0, sizeof(J));
    mesh_to_enu(mlon, mlat, mh, nmv, ncell, enu, &J.fr);
    free(mlon); free(mlat); free(mh);
    double t1 = now_s();

    hzo_bvh_32 b32;
    hzo_bvh_64 b64;
    memset(&b32, 0, sizeof(b32));
    memset(&b64, 0, sizeof(b64));
    if (opt.precision == 0) {
        float* v32 = malloc(sizeof(float) * 3 * (size_t)nmv);
        for (size_t k = 0; k < 3 * (size_t)nmv; k++) v32[k] = (float)enu[k];
        rc = hzo_bvh_build_32(&b32, v32, vot, ntri);
        free(v32);
    } else {
        rc = hzo_bvh_build_64(&b64, enu, vot, ntri);
    }
    free(vot);
    if (rc != 0) { free(enu); return -3; }
    double t2 = now_s();

    /* cpp:577-581, 651-668 */
    J.enu = enu;
    J.bvh32 = &b32;
    J.bvh64 = &b64;
    J.precision = opt.precision;
    J.brute = opt.brute_force;
    J.horizon = horizon;
    J.skyview = skyview;
    J.ncell = ncell;
    J.nhori = nhori;
    J.refine = refine_factor;
    J.svf_type = svf_type;
    J.dist_search = dist_search;
    J.ray_org_elev = ray_org_elev;
    J.hori_acc = deg2rad(0.25);
    J.elev_floor = deg2rad(opt.elev_floor_deg);
    int L = nhori * refine_factor;
    J.azim_sin = sin(deg2rad(360.0) / (double)L);
    J.azim_cos = cos(deg2rad(360.0) / (double)L);
    J.elev_sin_2ha = sin(2.0 * J.hori_acc);
    J.elev_cos_2ha = cos(2.0 * J.hori_acc);
    if (refine_factor == 1) J.azim_shift = 0.0;
    else J.azim_shift = -(deg2rad(360.0) / (2.0 * nhori))
                        + (deg2rad(360.0) / (2.0 * (double)L));
    J.cells = opt.cells;
    J.n_work = opt.cells ? opt.n_cells : ncell;
    J.start_m = opt.start_m;
    J.groups = opt.groups;
    J.start_all = opt.start_all;
    J.bisect_walk = opt.bisect_walk;
    if (J.start_m && J.groups > 1 && (nhori % J.groups) != 0) {
        free(enu);
        return -1;
    }
    atomic_init(&J.next, 0);
    atomic_init(&J.rays, 0);
    atomic_init(&J.nodes, 0);
    atomic_init(&J.tris, 0);
    atomic_init(&J.overflow, 0);

    int nth = opt.nthreads > 0 ? opt.nthreads : (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (nth < 1) nth = 1;
    if (nth > 1024) nth = 1024;
    pthread_t th[1024];
    int started = 0;
    for (int k = 1; k < nth; k++)
        if (pthread_create(&th[started], NULL, trace_worker, &J) == 0) started++;
    trace_worker(&J);
    for (int k = 0; k < started; k++) pthread_join(th[k], NULL);
    double t3 = now_s();

    res->num_rays = atomic_load(&J.rays);
    res->node_visits = atomic_load(&J.nodes);
    res->tri_tests = atomic_load(&J.tris);
    res->overflow = atomic_load(&J.overflow);
    res->n_tri = ntri;
    res->n_mesh_vert = nmv;
    res->t_mesh = t1 - t0;
    res->t_bvh = t2 - t1;
    res->t_rays = t3 - t2;
    hzo_bvh_free_32(&b32);
    hzo_bvh_free_64(&b64);
    free(enu);
    return 0;
}

int hzo_occluded32(const float* vert, const int32_t* vot, int n_tri,
                   const float* org, const float* dir, float tfar, int n_ray,
                   int brute_force, uint8_t* hit) {
    hzo_bvh_32 b;
    if (hzo_bvh_build_32(&b, vert, vot, n_tri) != 0) return -3;
    hzo_counts cnt = {0, 0, 0};
    for (int k = 0; k < n_ray; k++) {
        hzo_ray_32 r;
        hzo_ray_setup_32(&r, org + 3 * (size_t)k, dir + 3 * (size_t)k, 0.0f, tfar);
        hit[k] = (uint8_t)(brute_force ? hzo_occluded_brute_32(&b, &r, &cnt)
                                       : hzo_occluded_32(&b, &r, &cnt));
    }
    hzo_bvh_free_32(&b);
    return 0;
}
