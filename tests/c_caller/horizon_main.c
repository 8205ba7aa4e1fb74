/*
 * A C program calling the library the way EXTPAR's code would: the
 * reference's prototype horizon_svf_comp (mo_lradtopo_horayzon.h:4-11) with
 * C linkage, its status-returning variant and the Fortran-buffer variant,
 * through include/horayzon_gb300.h only.
 *
 *   horizon_main <dir> <num_hori> <grid_type> <dist_search> <ray_org_elev>
 *                <refine_factor> <svf_type>
 *
 * <dir> holds the inputs as raw little-endian arrays (clon, clat, hsurf,
 * vlon, vlat: float64; cells_of_vertex: int32, C order (6, nvertex)) and
 * sizes.txt ("num_cell num_vertex"); the program writes horizon.bin and
 * skyview.bin (float64) from each entry point, with suffixes 1, 2, 3, and
 * the buffer entry's text to log.txt. Exit status 0 when all calls succeed.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "horayzon_gb300.h"

static void* load(const char* dir, const char* name, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "rb");
  void* p = malloc(bytes ? bytes : 1);
  if (!f || !p || fread(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "cannot read %s\n", path);
    exit(2);
  }
  fclose(f);
  return p;
}

static void save(const char* dir, const char* name, const void* p, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(2);
  }
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 8) {
    fprintf(stderr, "usage: %s dir num_hori grid_type dist_search ray_org_elev refine svf\n",
            argv[0]);
    return 2;
  }
  const char* dir = argv[1];
  const int num_hori = atoi(argv[2]), grid_type = atoi(argv[3]);
  const double dist_search = atof(argv[4]), ray_org_elev = atof(argv[5]);
  const int refine_factor = atoi(argv[6]), svf_type = atoi(argv[7]);
  char path[4096];
  snprintf(path, sizeof(path), "%s/sizes.txt", dir);
  FILE* f = fopen(path, "r");
  int num_cell = 0, num_vertex = 0;
  if (!f || fscanf(f, "%d %d", &num_cell, &num_vertex) != 2) return 2;
  fclose(f);
  const size_t nc = (size_t)num_cell, nv = (size_t)num_vertex;
  double* clon = load(dir, "clon.bin", 8 * nc);
  double* clat = load(dir, "clat.bin", 8 * nc);
  double* hsurf = load(dir, "hsurf.bin", 8 * nc);
  double* vlon = load(dir, "vlon.bin", 8 * nv);
  double* vlat = load(dir, "vlat.bin", 8 * nv);
  int* cov = load(dir, "cells_of_vertex.bin", 4 * 6 * nv);
  const size_t nh = (size_t)num_hori * nc;
  double* horizon = malloc(8 * nh);
  double* skyview = malloc(8 * nc);

  /* 1: the reference's prototype (void; errors are printed, outputs NaN). */
  horizon_svf_comp(clon, clat, hsurf, vlon, vlat, cov, horizon, skyview, num_cell, num_vertex,
                   num_hori, grid_type, dist_search, ray_org_elev, refine_factor, svf_type);
  if (skyview[0] != skyview[0]) return 1;
  save(dir, "horizon1.bin", horizon, 8 * nh);
  save(dir, "skyview1.bin", skyview, 8 * nc);

  /* 2: the status-returning variant with default options and statistics. */
  hz_options opt;
  hz_default_options(&opt);
  hz_stats st;
  memset(&st, 0, sizeof(st));
  int rc = hz_horizon_svf(clon, clat, hsurf, vlon, vlat, cov, horizon, skyview, num_cell,
                          num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
                          refine_factor, svf_type, &opt, &st);
  if (rc != HZ_OK) {
    fprintf(stderr, "hz_horizon_svf: %s\n", hz_last_error());
    return 1;
  }
  save(dir, "horizon2.bin", horizon, 8 * nh);
  save(dir, "skyview2.bin", skyview, 8 * nc);

  /* 3: the Fortran-buffer variant: progress text into the caller's buffer. */
  char text[8192];
  int text_len = (int)sizeof(text);
  horizon_svf_comp_buffer(clon, clat, hsurf, vlon, vlat, cov, horizon, skyview, num_cell,
                          num_vertex, num_hori, grid_type, dist_search, ray_org_elev,
                          refine_factor, svf_type, text, &text_len);
  save(dir, "horizon3.bin", horizon, 8 * nh);
  save(dir, "skyview3.bin", skyview, 8 * nc);
  save(dir, "log.txt", text, (size_t)text_len);
  printf("rays %lld\n", (long long)st.num_rays);
  return 0;
}
