/*
 * kernel_interface.cpp -- the GB300 kernel backend of TeaLeaf: the 22 run_*
 * entry points of kernel_interface.h implemented over the C ABI of
 * include/tealeaf_gb300.h.
 *
 * This file compiles unchanged against the reference's own driver headers
 * (TeaLeaf/kernel_interface.h, chunk.h, settings.h) and against this
 * project's driver (exploringsycl_gb300/host/); it is what a TeaLeaf
 * maintainer adds as c_kernels/gb300/. It follows the dispatch of the
 * reference's SYCL backend (TeaLeaf/c_kernels/sycl/kernel_interface.cpp:
 * 34-371) call for call, with two additions:
 *
 * Run-ahead CG. With settings->solver == CG_SOLVER (and TL_CG_MODE not set
 * to "stepwise"), run_cg_init performs the whole solve of the timestep on
 * the device (tl_cg_solve: one persistent kernel, no host round trip per
 * step) using the driver's own stop rule, sqrt(|rrn|) < eps, and max_iters.
 * It records pw and rrn of every step. The driver's loop that follows
 * (TeaLeaf/drivers/cg_driver.c:18-25) is then replayed: run_copy_u and the
 * u/p halo updates are no-ops (already done on the device),
 * run_cg_calc_w / run_cg_calc_ur return the recorded scalars, and
 * run_cg_calc_ur / run_cg_calc_p check that the driver's alpha and beta are
 * bit-identical to the device's (both are the same IEEE divisions of the
 * same recorded values); a mismatch stops the run with an error. The final
 * device state, the scalars and the iteration count are those of the
 * step-wise path, bit for bit. Should the driver ask for more steps than
 * the device recorded (the device stopped early: both apply the same stop
 * rule to the same values), the replay ends after the last recorded step
 * and the remaining steps run on the step-wise kernels from the device's
 * final state.
 *
 * Errors. Every failing call ends the run through die() with the backend's
 * message, as the reference's fatal errors do (TeaLeaf/shared.c:98-111).
 * There is no CPU fallback: without a usable GPU, run_kernel_initialise
 * fails.
 *
 * Solver replacement. With the deck key `gb300_solver <cg64|mixed|
 * mixed-jacobi|mixed-learned|mixed-learned-coarse>` (or TL_SOLVER in the environment;
 * `preconditioner_on` alone selects mixed-jacobi; mixed-learned reads the
 * network's weights from `gb300_weights <file>` or TL_WEIGHTS: raw
 * little-endian FP32, tl_net_num_params() values), run_cg_init solves the timestep with
 * tl_solve to a relative FP64 true residual (`gb300_rel_tol`, default
 * 1e-10; `gb300_inner_tol`, default the method's own; `gb300_projection K`,
 * default 0, starts each solve from the A-norm best combination of u0 and
 * the last K solutions instead of from u0) and then reports rro = pw = 1,
 * rrn = 0, so that the driver's CG loop ends after one pass and prints
 * "CG: 0 iterations"; the backend prints the true counts and the true
 * residual on a TL_SOLVE line. The reference driver ignores the gb300_* keys
 * (TeaLeaf/parse_config.c:77-192 skips unknown lines).
 *
 * FP64 arithmetic. `gb300_fp64 fused` (or TL_FP64=fused) selects the fused
 * multiply-add contract of the persistent FP64 CG (tl_set_fp64_contract);
 * the default, exact, is bit-identical to the reference's C kernels.
 *
 * Environment: TL_DEVICE (GPU index, default 0), TL_CG_MODE ("fused", the
 * default, or "stepwise"), TL_SOLVER (as gb300_solver), TL_WEIGHTS (as
 * gb300_weights), TL_FP64 (as gb300_fp64), TL_PRINT_SUMMARY=1
 * (print the four field-summary sums at full precision), TL_PRINT_SOLVE=1
 * (print per-solve device steps), TL_DUMP_DIR=<dir> (write density, energy
 * and u as VisIt BOV files at every field summary).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "kernel_interface.h"
#include "tealeaf_gb300.h"
#include "../host/tl_dump.h" /* header-only field dump */

#define TL_TRY(call, what)                                                     \
  do {                                                                         \
    int rc_ = (call);                                                          \
    if (rc_ != TL_OK)                                                          \
      die(__LINE__, __FILE__, "GB300 backend: %s failed (code %d): %s\n", what, \
          rc_, tl_last_error());                                               \
  } while (0)

static double* device_field(tl_context* ctx, size_t n) {
  double* d = NULL;
  TL_TRY(tl_field_alloc(ctx, n, &d), "field allocation");
  return d;
}

static bool env_is(const char* name, const char* value) {
  const char* v = getenv(name);
  return v && strcmp(v, value) == 0;
}

static int method_from_name(const char* name) {
  if (!name || !*name) return -1;
  if (strcmp(name, "cg64") == 0) return TL_METHOD_CG64;
  if (strcmp(name, "mixed") == 0) return TL_METHOD_MIXED_CG;
  if (strcmp(name, "mixed-jacobi") == 0) return TL_METHOD_MIXED_JACOBI;
  if (strcmp(name, "mixed-learned") == 0) return TL_METHOD_MIXED_LEARNED;
  if (strcmp(name, "mixed-learned-coarse") == 0) return TL_METHOD_MIXED_LEARNED_COARSE;
  if (strcmp(name, "cg") == 0 || strcmp(name, "reference") == 0) return -1;
  die(__LINE__, __FILE__, "GB300 backend: unknown solver '%s'\n", name);
  return -1;
}

static int fp64_from_name(const char* name) {
  if (strcmp(name, "exact") == 0) return 0;
  if (strcmp(name, "fused") == 0) return 1;
  die(__LINE__, __FILE__, "GB300 backend: unknown FP64 contract '%s'\n", name);
  return 0;
}

/* The learned preconditioner's weights: a raw little-endian FP32 file of
 * tl_net_num_params() values. */
static void load_network(ChunkExtension* ext, const char* path) {
  if (!path || !*path) {
    die(__LINE__, __FILE__,
        "GB300 backend: mixed-learned needs the weights file (gb300_weights or TL_WEIGHTS)\n");
  }
  const int n = tl_net_num_params();
  std::vector<float> w((size_t)n);
  FILE* f = fopen(path, "rb");
  if (!f) die(__LINE__, __FILE__, "GB300 backend: cannot open weights file %s\n", path);
  const size_t got = fread(w.data(), sizeof(float), (size_t)n, f);
  const bool extra = fgetc(f) != EOF;
  fclose(f);
  if (got != (size_t)n || extra) {
    die(__LINE__, __FILE__, "GB300 backend: %s does not hold %d FP32 weights\n", path, n);
  }
  TL_TRY(tl_net_create(ext->ctx, &ext->net), "network creation");
  TL_TRY(tl_net_set_weights(ext->net, w.data(), n), "network weights");
}

/* The backend's own deck keys (gb300_*), read from the same tea.in. */
static void read_backend_keys(Settings* settings, ChunkExtension* ext) {
  ext->replace_method = settings->preconditioner ? TL_METHOD_MIXED_JACOBI : -1;
  ext->replace_rel_tol = 1e-10;
  ext->replace_inner_tol = 0.0; /* the method's default */
  ext->replace_projection = 0;  /* start each solve from u0, as the reference */
  ext->fp64_fused = 0;
  char weights[512] = "";
  FILE* f = fopen(settings->tea_in_filename, "r");
  if (f) {
    char line[512], word[128];
    double v;
    int iv;
    while (fgets(line, sizeof(line), f)) {
      if (sscanf(line, " gb300_solver %127s", word) == 1) ext->replace_method = method_from_name(word);
      if (sscanf(line, " gb300_rel_tol %lf", &v) == 1) ext->replace_rel_tol = v;
      if (sscanf(line, " gb300_inner_tol %lf", &v) == 1) ext->replace_inner_tol = v;
      if (sscanf(line, " gb300_projection %d", &iv) == 1) ext->replace_projection = iv;
      if (sscanf(line, " gb300_fp64 %127s", word) == 1) ext->fp64_fused = fp64_from_name(word);
      char path[512];
      if (sscanf(line, " gb300_weights %511s", path) == 1) snprintf(weights, sizeof(weights), "%s", path);
    }
    fclose(f);
  }
  const char* env = getenv("TL_SOLVER");
  if (env) ext->replace_method = method_from_name(env);
  env = getenv("TL_FP64");
  if (env) ext->fp64_fused = fp64_from_name(env);
  env = getenv("TL_WEIGHTS");
  if (env) snprintf(weights, sizeof(weights), "%s", env);
  TL_TRY(tl_set_fp64_contract(ext->ctx, ext->fp64_fused ? TL_FP64_FUSED : TL_FP64_EXACT),
         "FP64 contract");
  if (ext->replace_method == TL_METHOD_MIXED_LEARNED ||
      ext->replace_method == TL_METHOD_MIXED_LEARNED_COARSE)
    load_network(ext, weights);
}

/* TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:31-80 */
void run_kernel_initialise(Chunk* chunk, Settings* settings) {
  print_and_log(settings, "Performing this solve with the GB300 %s solver\n",
                settings->solver_name);
  ChunkExtension* ext = chunk->ext;
  memset(ext, 0, sizeof(*ext));
  const char* dev = getenv("TL_DEVICE");
  TL_TRY(tl_context_create(dev ? atoi(dev) : 0, NULL, &ext->ctx), "context creation");
  tl_context* ctx = ext->ctx;
  const size_t x = chunk->x, y = chunk->y;
  chunk->density0 = device_field(ctx, x * y);
  chunk->density = device_field(ctx, x * y);
  chunk->energy0 = device_field(ctx, x * y);
  chunk->energy = device_field(ctx, x * y);
  chunk->u = device_field(ctx, x * y);
  chunk->u0 = device_field(ctx, x * y);
  chunk->p = device_field(ctx, x * y);
  chunk->r = device_field(ctx, x * y);
  chunk->mi = device_field(ctx, x * y);
  chunk->w = device_field(ctx, x * y);
  chunk->kx = device_field(ctx, x * y);
  chunk->ky = device_field(ctx, x * y);
  chunk->sd = device_field(ctx, x * y);
  chunk->volume = device_field(ctx, x * y);
  chunk->x_area = device_field(ctx, (x + 1) * y);
  chunk->y_area = device_field(ctx, x * (y + 1));
  chunk->cell_x = device_field(ctx, x);
  chunk->cell_y = device_field(ctx, y);
  chunk->cell_dx = device_field(ctx, x);
  chunk->cell_dy = device_field(ctx, y);
  chunk->vertex_dx = device_field(ctx, x + 1);
  chunk->vertex_dy = device_field(ctx, y + 1);
  chunk->vertex_x = device_field(ctx, x + 1);
  chunk->vertex_y = device_field(ctx, y + 1);
  ext->comms_buffer = NULL;
  const size_t iters = settings->max_iters > 0 ? (size_t)settings->max_iters : 1;
  chunk->cg_alphas = (double*)calloc(iters, sizeof(double));
  chunk->cg_betas = (double*)calloc(iters, sizeof(double));
  chunk->cheby_alphas = (double*)calloc(iters, sizeof(double));
  chunk->cheby_betas = (double*)calloc(iters, sizeof(double));
  ext->ra_pw = (double*)calloc(iters, sizeof(double));
  ext->ra_rrn = (double*)calloc(iters, sizeof(double));
  ext->ra_cap = (int)iters;
  ext->fused_cg = !env_is("TL_CG_MODE", "stepwise");
  read_backend_keys(settings, ext);
  /* The whole-timestep paths solve this chunk alone. With more than one
   * chunk (several per rank, or several ranks: TeaLeaf/initialise.c:34-38)
   * the chunks' solves must be coupled through the driver's sums of pw and
   * rrn over chunks and ranks, which only the step-wise kernels take part
   * in: run-ahead gives way to them, and a solver replacement, which has no
   * step-wise form, is refused. */
  if (settings->num_chunks_per_rank > 1 || settings->num_ranks > 1) {
    if (ext->replace_method >= 0) {
      die(__LINE__, __FILE__,
          "GB300 backend: gb300_solver / preconditioner_on solve one chunk; this run has "
          "%d chunks per rank on %d ranks\n",
          settings->num_chunks_per_rank, settings->num_ranks);
    }
    ext->fused_cg = 0;
  }
}

/* TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:82-125 */
void run_kernel_finalise(Chunk* chunk, Settings* settings) {
  (void)settings;
  ChunkExtension* ext = chunk->ext;
  double* fields[] = {chunk->density0, chunk->density, chunk->energy0, chunk->energy,
                      chunk->u, chunk->u0, chunk->p, chunk->r, chunk->mi, chunk->w,
                      chunk->kx, chunk->ky, chunk->sd, chunk->volume, chunk->x_area,
                      chunk->y_area, chunk->cell_x, chunk->cell_y, chunk->cell_dx,
                      chunk->cell_dy, chunk->vertex_dx, chunk->vertex_dy,
                      chunk->vertex_x, chunk->vertex_y};
  for (double* f : fields) TL_TRY(tl_field_free(ext->ctx, f), "field release");
  free(chunk->cg_alphas);
  free(chunk->cg_betas);
  free(chunk->cheby_alphas);
  free(chunk->cheby_betas);
  free(ext->ra_pw);
  free(ext->ra_rrn);
  if (ext->net) TL_TRY(tl_net_destroy(ext->net), "network release");
  ext->net = NULL;
  TL_TRY(tl_context_destroy(ext->ctx), "context release");
  ext->ctx = NULL;
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:34-51 */
void run_set_chunk_data(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  tl_context* ctx = chunk->ext->ctx;
  const double x_min = settings->grid_x_min + settings->dx * (double)chunk->left;
  const double y_min = settings->grid_y_min + settings->dy * (double)chunk->bottom;
  TL_TRY(tl_set_chunk_data_vertices(ctx, chunk->x, chunk->y, settings->halo_depth,
                                    chunk->vertex_x, chunk->vertex_y, x_min, y_min,
                                    settings->dx, settings->dy),
         "set_chunk_data_vertices");
  TL_TRY(tl_set_chunk_data(ctx, chunk->x, chunk->y, settings->halo_depth,
                           chunk->vertex_x, chunk->vertex_y, chunk->cell_x,
                           chunk->cell_y, chunk->volume, chunk->x_area, chunk->y_area,
                           x_min, y_min, settings->dx, settings->dy),
         "set_chunk_data");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:53-70 */
void run_set_chunk_state(Chunk* chunk, Settings* settings, State* states) {
  START_PROFILING(settings->kernel_profile);
  tl_context* ctx = chunk->ext->ctx;
  TL_TRY(tl_set_chunk_initial_state(ctx, chunk->x, chunk->y, states[0].energy,
                                    states[0].density, chunk->energy0, chunk->density),
         "set_chunk_initial_state");
  for (int ii = 1; ii < settings->num_states; ++ii) {
    tl_state s;
    s.density = states[ii].density;
    s.energy = states[ii].energy;
    s.x_min = states[ii].x_min;
    s.y_min = states[ii].y_min;
    s.x_max = states[ii].x_max;
    s.y_max = states[ii].y_max;
    s.radius = states[ii].radius;
    s.geometry = (int)states[ii].geometry;
    TL_TRY(tl_set_chunk_state(ctx, chunk->x, chunk->y, settings->halo_depth, &s,
                              chunk->energy0, chunk->density, chunk->u, chunk->cell_x,
                              chunk->cell_y, chunk->vertex_x, chunk->vertex_y),
           "set_chunk_state");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:100-127: every flagged field,
 * faces L, R, T, B (external faces only), batched into one launch per face
 * pair. While a run-ahead solve is being replayed, u and p already hold
 * their final halos and are skipped. */
void run_local_halos(Chunk* chunk, Settings* settings, int depth) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  int mask = 0;
  const int faces[4] = {CHUNK_LEFT, CHUNK_RIGHT, CHUNK_BOTTOM, CHUNK_TOP};
  for (int f = 0; f < 4; ++f)
    if (chunk->neighbours[faces[f]] == EXTERNAL_FACE) mask |= 1 << faces[f];
  double* fields[NUM_FIELDS];
  int n = 0;
  if (settings->fields_to_exchange[FIELD_DENSITY]) fields[n++] = chunk->density;
  if (settings->fields_to_exchange[FIELD_P] && !ext->ra_active) fields[n++] = chunk->p;
  if (settings->fields_to_exchange[FIELD_ENERGY0]) fields[n++] = chunk->energy0;
  if (settings->fields_to_exchange[FIELD_ENERGY1]) fields[n++] = chunk->energy;
  if (settings->fields_to_exchange[FIELD_U] && !ext->ra_active) fields[n++] = chunk->u;
  if (settings->fields_to_exchange[FIELD_SD]) fields[n++] = chunk->sd;
  if (n > 0 && mask != 0) {
    TL_TRY(tl_local_halos(ext->ctx, chunk->x, chunk->y, settings->halo_depth, depth, mask,
                          fields, n),
           "local_halos");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:129-167 */
void run_pack_or_unpack(Chunk* chunk, Settings* settings, int depth, int face,
                        bool pack, FieldBufferType field, double* buffer) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_pack_or_unpack(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                           depth, face, pack ? 1 : 0, field, buffer),
         "pack_or_unpack");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:170-177 */
void run_store_energy(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_store_energy(chunk->ext->ctx, chunk->x, chunk->y, chunk->energy,
                         chunk->energy0),
         "store_energy");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:179-189 */
void run_field_summary(Chunk* chunk, Settings* settings, double* vol,
                       double* mass, double* ie, double* temp) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_field_summary(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                          chunk->u, chunk->density, chunk->energy0, chunk->volume,
                          vol, mass, ie, temp),
         "field_summary");
  if (env_is("TL_PRINT_SUMMARY", "1")) {
    printf("TL_SUMMARY %.17e %.17e %.17e %.17e\n", *vol, *mass, *ie, *temp);
  }
  const char* dump = getenv("TL_DUMP_DIR");
  if (dump && *dump) {
    /* density, energy and u of every field summary, numbered in order */
    static int dump_count = 0;
    std::vector<double> host((size_t)chunk->x * chunk->y);
    const struct { const char* name; double* f; } fields[] = {
        {"density", chunk->density}, {"energy", chunk->energy}, {"u", chunk->u}};
    for (const auto& fd : fields) {
      TL_TRY(tl_copy_to_host(chunk->ext->ctx, host.data(), fd.f, host.size()), "dump copy");
      if (tl_dump_interior(dump, fd.name, dump_count, 0.0, chunk->x, chunk->y,
                           settings->halo_depth, host.data()) != 0) {
        die(__LINE__, __FILE__, "GB300 backend: cannot write dumps to %s\n", dump);
      }
    }
    dump_count++;
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:192-210 */
void run_cg_init(Chunk* chunk, Settings* settings, double rx, double ry,
                 double* rro) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  if (ext->replace_method >= 0 && settings->solver == CG_SOLVER) {
    tl_solve_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.method = ext->replace_method;
    prm.learned = ext->net;
    prm.rel_tol = ext->replace_rel_tol;
    prm.inner_tol = ext->replace_inner_tol;
    prm.projection = ext->replace_projection;
    prm.max_inner = settings->max_iters;
    prm.max_outer = 12;
    prm.stall_factor = 0.5;
    prm.max_fallback = settings->max_iters;
    tl_solve_report rep;
    TL_TRY(tl_solve(ext->ctx, chunk->x, chunk->y, settings->halo_depth, settings->coefficient,
                    rx, ry, &prm, chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w, chunk->kx,
                    chunk->ky, chunk->density, chunk->energy, &rep),
           "solve");
    /* algorithmic bytes per cell and inner step of the method's kernel */
    const double bytes_per_cell = prm.method == TL_METHOD_CG64 ? 104.0
                                  : prm.method == TL_METHOD_MIXED_CG ? 48.0
                                  : prm.method == TL_METHOD_MIXED_JACOBI ? 56.0 : 52.0;
    const double cells = (double)(chunk->x - 2 * settings->halo_depth) *
                         (double)(chunk->y - 2 * settings->halo_depth);
    const double gbs = rep.inner_kernel_ms > 0.0f
                           ? bytes_per_cell * cells * (double)rep.inner_steps /
                                 ((double)rep.inner_kernel_ms * 1e-3) / 1e9
                           : 0.0;
    printf("TL_SOLVE method=%d outer=%d inner=%d fallback_events=%d fallback_steps=%d "
           "rel_residual=%.6e device_ms=%.3f inner_gbs=%.1f\n",
           prm.method, rep.outer_steps, rep.inner_steps, rep.fallback_events,
           rep.fallback_steps, rep.final_rel_residual, rep.device_ms, gbs);
    /* tl_solve falls back to FP64 CG whenever refinement does not reach the
     * target; only an exhausted FP64 CG (max_iters steps) ends above it. */
    if (!(rep.final_rel_residual <= prm.rel_tol)) {
      die(__LINE__, __FILE__,
          "GB300 backend: the solve ended at a relative residual of %.3e, above the "
          "target %.3e, after %d fall-back steps (max_iters %d)\n",
          rep.final_rel_residual, prm.rel_tol, rep.fallback_steps, settings->max_iters);
    }
    /* One synthetic step with pw = 1, rrn = 0: the driver's loop ends at once. */
    *rro += 1.0;
    ext->ra_rro0 = 1.0;
    ext->ra_pw[0] = 1.0;
    ext->ra_rrn[0] = 0.0;
    ext->ra_steps = 1;
    ext->ra_k = 0;
    ext->ra_active = 1;
  } else if (ext->fused_cg && settings->solver == CG_SOLVER) {
    if (settings->max_iters > ext->ra_cap) {
      die(__LINE__, __FILE__, "GB300 backend: max_iters grew after initialisation\n");
    }
    double rro0 = 0.0;
    int steps = 0;
    TL_TRY(tl_cg_solve(ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                       settings->coefficient, rx, ry, settings->eps, settings->max_iters,
                       chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w, chunk->kx,
                       chunk->ky, chunk->density, chunk->energy, &rro0, ext->ra_pw,
                       ext->ra_rrn, &steps),
           "cg_solve");
    *rro += rro0;
    ext->ra_rro0 = rro0;
    ext->ra_steps = steps;
    ext->ra_k = 0;
    ext->ra_active = 1;
    if (env_is("TL_PRINT_SOLVE", "1")) printf("TL_SOLVE device_steps=%d\n", steps);
  } else {
    TL_TRY(tl_cg_init(ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                      settings->coefficient, rx, ry, chunk->p, chunk->r, chunk->u,
                      chunk->w, chunk->kx, chunk->ky, chunk->density, chunk->energy, rro),
           "cg_init");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_w(Chunk* chunk, Settings* settings, double* pw) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  if (ext->ra_active) {
    if (ext->ra_k >= ext->ra_steps) {
      die(__LINE__, __FILE__, "GB300 backend: driver asked for CG step %d of %d\n",
          ext->ra_k + 1, ext->ra_steps);
    }
    *pw += ext->ra_pw[ext->ra_k];
  } else {
    TL_TRY(tl_cg_calc_w(ext->ctx, chunk->x, chunk->y, settings->halo_depth, chunk->w,
                        chunk->p, chunk->kx, chunk->ky, pw),
           "cg_calc_w");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_ur(Chunk* chunk, Settings* settings, double alpha, double* rrn) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  if (ext->ra_active) {
    const int k = ext->ra_k;
    const double rro = (k == 0) ? ext->ra_rro0 : ext->ra_rrn[k - 1];
    const double dev_alpha = rro / ext->ra_pw[k];
    if (memcmp(&dev_alpha, &alpha, sizeof(double)) != 0) {
      die(__LINE__, __FILE__,
          "GB300 backend: driver alpha %.17e differs from the device's %.17e at step %d\n",
          alpha, dev_alpha, k);
    }
    *rrn = ext->ra_rrn[k];
  } else {
    TL_TRY(tl_cg_calc_ur(ext->ctx, chunk->x, chunk->y, settings->halo_depth, chunk->u,
                         chunk->r, chunk->p, chunk->w, alpha, rrn),
           "cg_calc_ur");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cg_calc_p(Chunk* chunk, Settings* settings, double beta) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  if (ext->ra_active) {
    const int k = ext->ra_k;
    const double rro = (k == 0) ? ext->ra_rro0 : ext->ra_rrn[k - 1];
    const double dev_beta = ext->ra_rrn[k] / rro;
    if (memcmp(&dev_beta, &beta, sizeof(double)) != 0) {
      die(__LINE__, __FILE__,
          "GB300 backend: driver beta %.17e differs from the device's %.17e at step %d\n",
          beta, dev_beta, k);
    }
    ext->ra_k = k + 1;
    if (ext->ra_k == ext->ra_steps) ext->ra_active = 0;
  } else {
    TL_TRY(tl_cg_calc_p(ext->ctx, chunk->x, chunk->y, settings->halo_depth, beta,
                        chunk->p, chunk->r),
           "cg_calc_p");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:245-271 */
void run_cheby_init(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_cheby_init(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                       chunk->theta, chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w,
                       chunk->kx, chunk->ky),
         "cheby_init");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_cheby_iterate(Chunk* chunk, Settings* settings, double alpha, double beta) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_cheby_iterate(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                          alpha, beta, chunk->p, chunk->r, chunk->u, chunk->u0, chunk->w,
                          chunk->kx, chunk->ky),
         "cheby_iterate");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:273-300 */
void run_jacobi_init(Chunk* chunk, Settings* settings, double rx, double ry) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_jacobi_init(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                        settings->coefficient, rx, ry, chunk->u, chunk->u0,
                        chunk->density, chunk->energy, chunk->kx, chunk->ky),
         "jacobi_init");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_jacobi_iterate(Chunk* chunk, Settings* settings, double* error) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_jacobi_iterate(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                           chunk->u, chunk->u0, chunk->r, chunk->kx, chunk->ky, error),
         "jacobi_iterate");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:302-328 */
void run_ppcg_init(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_ppcg_init(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                      chunk->theta, chunk->sd, chunk->r),
         "ppcg_init");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_ppcg_inner_iteration(Chunk* chunk, Settings* settings, double alpha,
                              double beta) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_ppcg_inner_iteration(chunk->ext->ctx, chunk->x, chunk->y,
                                 settings->halo_depth, chunk->theta, alpha, beta,
                                 chunk->sd, chunk->r, chunk->u, chunk->kx, chunk->ky),
         "ppcg_inner_iteration");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/c_kernels/sycl/kernel_interface.cpp:330-371 */
void run_copy_u(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  ChunkExtension* ext = chunk->ext;
  if (ext->ra_active) {
    /* The device solve already set u0 = u before its first step. */
    if (ext->ra_steps == 0) ext->ra_active = 0;
  } else {
    TL_TRY(tl_copy_u(ext->ctx, chunk->x, chunk->y, settings->halo_depth, chunk->u,
                     chunk->u0),
           "copy_u");
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_calculate_residual(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_calculate_residual(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                               chunk->u, chunk->u0, chunk->r, chunk->kx, chunk->ky),
         "calculate_residual");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_calculate_2norm(Chunk* chunk, Settings* settings, FieldBufferType buffer,
                         double* norm) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_calculate_2norm(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth,
                            buffer, norm),
         "calculate_2norm");
  STOP_PROFILING(settings->kernel_profile, __func__);
}

void run_finalise(Chunk* chunk, Settings* settings) {
  START_PROFILING(settings->kernel_profile);
  TL_TRY(tl_finalise(chunk->ext->ctx, chunk->x, chunk->y, settings->halo_depth, chunk->u,
                     chunk->density, chunk->energy),
         "finalise");
  STOP_PROFILING(settings->kernel_profile, __func__);
}
