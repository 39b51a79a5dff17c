/*
 * kernel_interface.cpp -- the 22 run_* entry points over the CPU oracle
 * kernels (TEST INFRASTRUCTURE; never linked into the product).
 *
 * Follows the reference backend's dispatch (TeaLeaf/c_kernels/sycl/
 * kernel_interface.cpp:34-371) call for call, so that linked under the
 * reference's own unchanged driver (oracle/Makefile target `ref`) or under
 * this project's driver (target `driver`) it behaves as the SYCL backend
 * would, with host arrays in place of SYCL buffers.
 *
 * Setting TL_PRINT_SUMMARY=1 makes run_field_summary print its four sums at
 * full precision (the driver prints only the temperature).
 */
#include <stdio.h>
#include <stdlib.h>

#include "kernel_interface.h"
#include "../../exploringsycl_gb300/host/tl_dump.h" /* header-only field dump */
#include "tl_oracle.h"

static double* alloc_zeroed(size_t n) {
  double* a = (double*)calloc(n ? n : 1, sizeof(double));
  if (!a) die(__LINE__, __FILE__, "Error allocating buffer\n");
  return a;
}

/* TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:31-80 */
void run_kernel_initialise(Chunk* chunk, Settings* settings) {
  print_and_log(settings, "Performing this solve with the CPU oracle %s solver\n",
                settings->solver_name);
  const size_t x = chunk->x, y = chunk->y;
  chunk->density0 = alloc_zeroed(x * y);
  chunk->density = alloc_zeroed(x * y);
  chunk->energy0 = alloc_zeroed(x * y);
  chunk->energy = alloc_zeroed(x * y);
  chunk->u = alloc_zeroed(x * y);
  chunk->u0 = alloc_zeroed(x * y);
  chunk->p = alloc_zeroed(x * y);
  chunk->r = alloc_zeroed(x * y);
  chunk->mi = alloc_zeroed(x * y);
  chunk->w = alloc_zeroed(x * y);
  chunk->kx = alloc_zeroed(x * y);
  chunk->ky = alloc_zeroed(x * y);
  chunk->sd = alloc_zeroed(x * y);
  chunk->volume = alloc_zeroed(x * y);
  chunk->x_area = alloc_zeroed((x + 1) * y);
  chunk->y_area = alloc_zeroed(x * (y + 1));
  chunk->cell_x = alloc_zeroed(x);
  chunk->cell_y = alloc_zeroed(y);
  chunk->cell_dx = alloc_zeroed(x);
  chunk->cell_dy = alloc_zeroed(y);
  chunk->vertex_dx = alloc_zeroed(x + 1);
  chunk->vertex_dy = alloc_zeroed(y + 1);
  chunk->vertex_x = alloc_zeroed(x + 1);
  chunk->vertex_y = alloc_zeroed(y + 1);
  chunk->ext->comms_buffer = alloc_zeroed((x > y ? x : y) * settings->halo_depth);
  chunk->cg_alphas = alloc_zeroed(settings->max_iters);
  chunk->cg_betas = alloc_zeroed(settings->max_iters);
  chunk->cheby_alphas = alloc_zeroed(settings->max_iters);
  chunk->cheby_betas = alloc_zeroed(settings->max_iters);
}

void run_kernel_finalise(Chunk* chunk, Settings* settings) {
  (void)settings;
  double* all[] = {chunk->density0, chunk->density, chunk->energy0, chunk->energy,
                   chunk->u, chunk->u0, chunk->p, chunk->r, chunk->mi, chunk->w,
                   chunk->kx, chunk->ky, chunk->sd, chunk->volume, chunk->x_area,
                   chunk->y_area, chunk->cell_x, chunk->cell_y, chunk->cell_dx,
                   chunk->cell_dy, chunk->vertex_dx, chunk->vertex_dy,
                   chunk->vertex_x, chunk->vertex_y, chunk->ext->comms_buffer,
                   chunk->cg_alphas, chunk->cg_betas, chunk->cheby_alphas,
                   chunk->cheby_betas};
  for (double* a : all) free(a);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:34-51 */
void run_set_chunk_data(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  double x_min = settings->grid_x_min + settings->dx * (double)chunk->left;
  double y_min = settings->grid_y_min + settings->dy * (double)chunk->bottom;
  orc_set_chunk_data_vertices(chunk->x, chunk->y, settings->halo_depth,
                              chunk->vertex_x, chunk->vertex_y, x_min, y_min,
                              settings->dx, settings->dy);
  orc_set_chunk_data(chunk->x, chunk->y, settings->halo_depth, chunk->vertex_x,
                     chunk->vertex_y, chunk->cell_x, chunk->cell_y, chunk->volume,
                     chunk->x_area, chunk->y_area, x_min, y_min, settings->dx,
                     settings->dy);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:53-70 */
void run_set_chunk_state(Chunk* chunk, Settings* settings, State* states) {
  START_PROFILING(settings->kernel_profile);
  orc_set_chunk_initial_state(chunk->x, chunk->y, states[0].energy,
                              states[0].density, chunk->energy0, chunk->density);
  for (int ii = 1; ii < settings->num_states; ++ii) {
    orc_state s;
    s.density = states[ii].density;
    s.energy = states[ii].energy;
    s.x_min = states[ii].x_min;
    s.y_min = states[ii].y_min;
    s.x_max = states[ii].x_max;
    s.y_max = states[ii].y_max;
    s.radius = states[ii].radius;
    s.geometry = (int)states[ii].geometry;
    orc_set_chunk_state(chunk->x, chunk->y, settings->halo_depth, &s,
                        chunk->energy0, chunk->density, chunk->u, chunk->cell_x,
                        chunk->cell_y, chunk->vertex_x, chunk->vertex_y);
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:100-127: faces L, R, T, B for
 * each flagged field, in the field order density, p, energy0, energy, u, sd. */
void run_local_halos(Chunk* chunk, Settings* settings, int depth) {
  const int faces[4] = {CHUNK_LEFT, CHUNK_RIGHT, CHUNK_TOP, CHUNK_BOTTOM};
  struct { int flag; double* f; } fields[6] = {
      {FIELD_DENSITY, chunk->density}, {FIELD_P, chunk->p},
      {FIELD_ENERGY0, chunk->energy0}, {FIELD_ENERGY1, chunk->energy},
      {FIELD_U, chunk->u},             {FIELD_SD, chunk->sd}};
  for (int ff = 0; ff < 6; ++ff) {
    if (!settings->fields_to_exchange[fields[ff].flag]) continue;
    for (int fc = 0; fc < 4; ++fc) {
      if (chunk->neighbours[faces[fc]] != EXTERNAL_FACE) continue;
      START_PROFILING(settings->kernel_profile);
      orc_update_face(chunk->x, chunk->y, settings->halo_depth, fields[ff].f,
                      faces[fc], depth);
      STOP_PROFILING(settings->kernel_profile, "update_face");
    }
  }
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:129-167 */
void run_pack_or_unpack(Chunk* chunk, Settings* settings, int depth, int face,
                        bool pack, FieldBufferType field, double* buffer) {
  START_PROFILING(settings->kernel_profile);
  orc_pack_or_unpack(chunk->x, chunk->y, settings->halo_depth, depth, face,
                     pack ? 1 : 0, field, buffer);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_store_energy(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_store_energy(chunk->x, chunk->y, chunk->energy, chunk->energy0);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_field_summary(Chunk* chunk, Settings* settings, double* vol,
                       double* mass, double* ie, double* temp) {
  START_PROFILING(settings->kernel_profile);
  orc_field_summary(chunk->x, chunk->y, settings->halo_depth, chunk->u,
                    chunk->density, chunk->energy0, chunk->volume, vol, mass, ie,
                    temp);
  const char* env = getenv("TL_PRINT_SUMMARY");
  if (env && env[0] == '1') {
    printf("TL_SUMMARY %.17e %.17e %.17e %.17e\n", *vol, *mass, *ie, *temp);
  }
  const char* dump = getenv("TL_DUMP_DIR");
  if (dump && *dump) {
    static int dump_count = 0;
    const struct { const char* name; double* f; } fields[] = {
        {"density", chunk->density}, {"energy", chunk->energy}, {"u", chunk->u}};
    for (const auto& fd : fields) {
      if (tl_dump_interior(dump, fd.name, dump_count, 0.0, chunk->x, chunk->y,
                           settings->halo_depth, fd.f) != 0) {
        die(__LINE__, __FILE__, "oracle backend: cannot write dumps to %s\n", dump);
      }
    }
    dump_count++;
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:192-243 */
void run_cg_init(Chunk* chunk, Settings* settings, double rx, double ry,
                 double* rro) {
  START_PROFILING(settings->kernel_profile);
  orc_cg_init_u(chunk->x, chunk->y, settings->coefficient, chunk->p, chunk->r,
                chunk->u, chunk->w, chunk->density, chunk->energy);
  orc_cg_init_k(chunk->x, chunk->y, settings->halo_depth, chunk->w, chunk->kx,
                chunk->ky, rx, ry);
  orc_cg_init_others(chunk->x, chunk->y, settings->halo_depth, chunk->kx,
                     chunk->ky, chunk->p, chunk->r, chunk->u, chunk->w, rro);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_w(Chunk* chunk, Settings* settings, double* pw) {
  START_PROFILING(settings->kernel_profile);
  orc_cg_calc_w(chunk->x, chunk->y, settings->halo_depth, chunk->w, chunk->p,
                chunk->kx, chunk->ky, pw);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_ur(Chunk* chunk, Settings* settings, double alpha,
                    double* rrn) {
  START_PROFILING(settings->kernel_profile);
  orc_cg_calc_ur(chunk->x, chunk->y, settings->halo_depth, chunk->u, chunk->r,
                 chunk->p, chunk->w, alpha, rrn);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_p(Chunk* chunk, Settings* settings, double beta) {
  START_PROFILING(settings->kernel_profile);
  orc_cg_calc_p(chunk->x, chunk->y, settings->halo_depth, beta, chunk->p,
                chunk->r);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:245-271 */
void run_cheby_init(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_cheby_init(chunk->x, chunk->y, settings->halo_depth, chunk->theta,
                 chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w, chunk->kx,
                 chunk->ky);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cheby_iterate(Chunk* chunk, Settings* settings, double alpha,
                       double beta) {
  START_PROFILING(settings->kernel_profile);
  orc_cheby_iterate(chunk->x, chunk->y, settings->halo_depth, alpha, beta,
                    chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w,
                    chunk->kx, chunk->ky);
  orc_cheby_calc_u(chunk->x, chunk->y, settings->halo_depth, chunk->p, chunk->u);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:273-300 */
void run_jacobi_init(Chunk* chunk, Settings* settings, double rx, double ry) {
  START_PROFILING(settings->kernel_profile);
  orc_jacobi_init(chunk->x, chunk->y, settings->halo_depth,
                  settings->coefficient, rx, ry, chunk->u, chunk->u0,
                  chunk->density, chunk->energy, chunk->kx, chunk->ky);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_jacobi_iterate(Chunk* chunk, Settings* settings, double* error) {
  START_PROFILING(settings->kernel_profile);
  orc_jacobi_copy_u(chunk->x, chunk->y, chunk->r, chunk->u);
  orc_jacobi_iterate(chunk->x, chunk->y, settings->halo_depth, chunk->u,
                     chunk->u0, chunk->r, chunk->kx, chunk->ky, error);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:302-328 */
void run_ppcg_init(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_ppcg_init(chunk->x, chunk->y, settings->halo_depth, chunk->theta,
                chunk->sd, chunk->r);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_ppcg_inner_iteration(Chunk* chunk, Settings* settings, double alpha,
                              double beta) {
  START_PROFILING(settings->kernel_profile);
  orc_ppcg_calc_ur(chunk->x, chunk->y, settings->halo_depth, chunk->sd,
                   chunk->r, chunk->u, chunk->kx, chunk->ky);
  orc_ppcg_calc_sd(chunk->x, chunk->y, settings->halo_depth, chunk->theta,
                   alpha, beta, chunk->sd, chunk->r);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:330-371 */
void run_copy_u(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_copy_u(chunk->x, chunk->y, settings->halo_depth, chunk->u, chunk->u0);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_calculate_residual(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_calculate_residual(chunk->x, chunk->y, settings->halo_depth, chunk->u,
                         chunk->u0, chunk->r, chunk->kx, chunk->ky);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_calculate_2norm(Chunk* chunk, Settings* settings,
                         FieldBufferType buffer, double* norm) {
  START_PROFILING(settings->kernel_profile);
  orc_calculate_2norm(chunk->x, chunk->y, settings->halo_depth, buffer, norm);
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_finalise(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  orc_finalise(chunk->x, chunk->y, settings->halo_depth, chunk->u,
               chunk->density, chunk->energy);
  STOP_PROFILING(settings->kernel_profile, __func__);
}
