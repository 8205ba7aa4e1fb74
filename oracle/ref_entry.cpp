/*
 * ref_entry.cpp -- C-linkage entry points into the unmodified reference,
 * compiled together with it into oracle/_ref/libhorayzon_ref.so.
 *
 * TEST INFRASTRUCTURE: used to pin the oracle and to generate golden fixtures.
 * The reference declares horizon_svf_comp with C++ linkage
 * (mo_lradtopo_horayzon.h:4-11) and build_triangle_mesh as an ordinary
 * external function (mo_lradtopo_horayzon.cpp:228-317); these wrappers give
 * ctypes a stable name for each.
 */
#include <cstring>
#include <vector>

#include "mo_lradtopo_horayzon.h"

/* Same layout as the reference's geom_point (mo_lradtopo_horayzon.cpp:27-30). */
struct geom_point {
    double x, y, z;
};
int build_triangle_mesh(double* clon, double* clat, double* hsurf, double* vlon,
                        double* vlat, int* cells_of_vertex, int num_cell,
                        int num_vertex, int grid_type,
                        std::vector<geom_point>& vertices,
                        std::vector<int>& vertex_of_triangle);

extern "C" {

void hzref_horizon_svf_comp(double* clon, double* clat, double* hsurf,
                            double* vlon, double* vlat, int* cells_of_vertex,
                            double* horizon, double* skyview, int num_cell,
                            int num_vertex, int num_hori, int grid_type,
                            double dist_search, double ray_org_elev,
                            int refine_factor, int svf_type) {
    horizon_svf_comp(clon, clat, hsurf, vlon, vlat, cells_of_vertex, horizon,
                     skyview, num_cell, num_vertex, num_hori, grid_type,
                     dist_search, ray_org_elev, refine_factor, svf_type);
}

/* Runs build_triangle_mesh; copies out at most the given capacities and
 * returns the triangle count (mesh vertex count in *n_mesh_vert). */
int hzref_build_triangle_mesh(double* clon, double* clat, double* hsurf,
                              double* vlon, double* vlat, int* cells_of_vertex,
                              int num_cell, int num_vertex, int grid_type,
                              double* mesh_xyz, int cap_vert, int* vot,
                              int cap_tri, int* n_mesh_vert) {
    std::vector<geom_point> vertices(num_cell);
    std::vector<int> vertex_of_triangle;
    int ntri = build_triangle_mesh(clon, clat, hsurf, vlon, vlat, cells_of_vertex,
                                   num_cell, num_vertex, grid_type, vertices,
                                   vertex_of_triangle);
    *n_mesh_vert = (int)vertices.size();
    size_t nv = vertices.size() < (size_t)cap_vert ? vertices.size() : (size_t)cap_vert;
    for (size_t i = 0; i < nv; i++) {
        mesh_xyz[3 * i] = vertices[i].x;
        mesh_xyz[3 * i + 1] = vertices[i].y;
        mesh_xyz[3 * i + 2] = vertices[i].z;
    }
    size_t nt = (size_t)ntri < (size_t)cap_tri ? (size_t)ntri : (size_t)cap_tri;
    std::memcpy(vot, vertex_of_triangle.data(), sizeof(int) * 3 * nt);
    return ntri;
}

}  // extern "C"
