/*
 * fake_abi.cpp -- a scripted stand-in for libtealeaf_gb300.so, linked only
 * into a test build of the TeaLeaf host driver with the run_* backend
 * (exploringsycl_gb300/backend/kernel_interface.cpp). It lets the CPU tests
 * check the backend's host logic without a GPU: the run-ahead replay of the
 * driver's CG loop, the mapping of deck keys to solver calls, and how a
 * failing call ends the run. It computes nothing of the path: fields are
 * zeroed host arrays, and the CG scalars come from the script.
 *
 * Script (environment):
 *   FAKE_LOG=<file>      every call appends one line: its name and key arguments
 *   FAKE_RRO0=<v>        r.r after cg_init (default 1)
 *   FAKE_PW=<a,b,...>    p.w of CG steps 0, 1, ... (the last value repeats; default 2)
 *   FAKE_RRN=<a,b,...>   r.r after CG steps 0, 1, ... (as above; default 1e-40)
 *   FAKE_STOP_AFTER=<n>  tl_cg_solve reports at most n steps, as a device that
 *                        stopped early would
 *   FAKE_FAIL=<name>     the call of that name returns TL_ERR_CUDA
 *
 * tl_cg_solve applies the driver's stop rule (sqrt(|rrn|) < eps, at most
 * max_iters steps) to the scripted values, like the persistent kernel; the
 * step-wise calls return the same values one step at a time.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "tealeaf_gb300.h"

struct tl_context {
  int device;
};
struct tl_net {
  int n;
};

namespace {

std::string g_error;
int g_step = 0;
int g_summaries = 0;

void log_line(const char* fmt, ...) __attribute__((format(printf, 1, 2)));
void log_line(const char* fmt, ...) {
  const char* path = getenv("FAKE_LOG");
  if (!path || !*path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  va_list a;
  va_start(a, fmt);
  vfprintf(f, fmt, a);
  va_end(a);
  fputc('\n', f);
  fclose(f);
}

/* TL_ERR_CUDA with a message when the script fails this call, else TL_OK. */
int scripted(const char* name) {
  const char* fail = getenv("FAKE_FAIL");
  if (fail && strcmp(fail, name) == 0) {
    g_error = std::string("scripted failure of ") + name;
    return TL_ERR_CUDA;
  }
  return TL_OK;
}

double env_double(const char* name, double dflt) {
  const char* v = getenv(name);
  return (v && *v) ? atof(v) : dflt;
}

double scripted_value(const char* name, int k, double dflt) {
  const char* v = getenv(name);
  if (!v || !*v) return dflt;
  std::vector<double> vals;
  const char* p = v;
  while (*p) {
    char* end = nullptr;
    const double d = strtod(p, &end);
    if (end == p) break;
    vals.push_back(d);
    p = end;
    if (*p == ',') ++p;
  }
  if (vals.empty()) return dflt;
  return vals[k < (int)vals.size() ? k : (int)vals.size() - 1];
}

double pw_of(int k) { return scripted_value("FAKE_PW", k, 2.0); }
double rrn_of(int k) { return scripted_value("FAKE_RRN", k, 1e-40); }

}  // namespace

#define FAKE_CALL(name, ...)          \
  do {                                \
    log_line(__VA_ARGS__);            \
    int rc_ = scripted(name);         \
    if (rc_ != TL_OK) return rc_;     \
  } while (0)

extern "C" {

const char* tl_last_error(void) { return g_error.c_str(); }

int tl_context_create(int device, void* stream, tl_context** out) {
  (void)stream;
  FAKE_CALL("tl_context_create", "tl_context_create device=%d", device);
  *out = new tl_context{device};
  return TL_OK;
}

int tl_context_destroy(tl_context* ctx) {
  FAKE_CALL("tl_context_destroy", "tl_context_destroy");
  delete ctx;
  return TL_OK;
}

int tl_set_fp64_contract(tl_context*, int contract) {
  FAKE_CALL("tl_set_fp64_contract", "tl_set_fp64_contract %d", contract);
  return TL_OK;
}

int tl_field_alloc(tl_context*, size_t count, double** dev_out) {
  FAKE_CALL("tl_field_alloc", "tl_field_alloc %zu", count);
  *dev_out = (double*)calloc(count ? count : 1, sizeof(double));
  return *dev_out ? TL_OK : TL_ERR_CUDA;
}

int tl_field_free(tl_context*, double* dev) {
  free(dev);
  return scripted("tl_field_free");
}

int tl_copy_to_host(tl_context*, double* host, const double* dev, size_t count) {
  FAKE_CALL("tl_copy_to_host", "tl_copy_to_host %zu", count);
  memcpy(host, dev, count * sizeof(double));
  return TL_OK;
}

int tl_set_chunk_data_vertices(tl_context*, int x, int y, int hd, double*, double*, double,
                               double, double, double) {
  FAKE_CALL("tl_set_chunk_data_vertices", "tl_set_chunk_data_vertices %d %d %d", x, y, hd);
  return TL_OK;
}

int tl_set_chunk_data(tl_context*, int x, int y, int hd, const double*, const double*,
                      double*, double*, double*, double*, double*, double, double, double,
                      double) {
  FAKE_CALL("tl_set_chunk_data", "tl_set_chunk_data %d %d %d", x, y, hd);
  return TL_OK;
}

int tl_set_chunk_initial_state(tl_context*, int x, int y, double energy, double density,
                               double*, double*) {
  FAKE_CALL("tl_set_chunk_initial_state", "tl_set_chunk_initial_state %d %d %.17g %.17g", x,
            y, energy, density);
  return TL_OK;
}

int tl_set_chunk_state(tl_context*, int, int, int, const tl_state* s, double*, double*,
                       double*, const double*, const double*, const double*,
                       const double*) {
  FAKE_CALL("tl_set_chunk_state", "tl_set_chunk_state geometry=%d density=%.17g", s->geometry,
            s->density);
  return TL_OK;
}

int tl_local_halos(tl_context*, int, int, int, int depth, int face_mask, double* const*,
                   int nfields) {
  FAKE_CALL("tl_local_halos", "tl_local_halos depth=%d mask=%d nfields=%d", depth, face_mask,
            nfields);
  return TL_OK;
}

int tl_pack_or_unpack(tl_context*, int, int, int, int depth, int face, int pack, double*,
                      double*) {
  FAKE_CALL("tl_pack_or_unpack", "tl_pack_or_unpack depth=%d face=%d pack=%d", depth, face,
            pack);
  return TL_OK;
}

int tl_store_energy(tl_context*, int, int, double*, const double*) {
  FAKE_CALL("tl_store_energy", "tl_store_energy");
  return TL_OK;
}

int tl_field_summary(tl_context*, int, int, int, const double*, const double*, const double*,
                     const double*, double* vol, double* mass, double* ie, double* temp) {
  FAKE_CALL("tl_field_summary", "tl_field_summary");
  *vol = 100.0;
  *mass = 10.0;
  *ie = 1.0;
  *temp = 1.0 + g_summaries++;
  return TL_OK;
}

int tl_cg_solve(tl_context*, int, int, int, int coefficient, double, double, double eps,
                int max_iters, double*, double*, double*, double*, double*, double*, double*,
                const double*, const double*, double* rro0, double* pw_hist, double* rrn_hist,
                int* steps) {
  FAKE_CALL("tl_cg_solve", "tl_cg_solve coefficient=%d eps=%.3g max_iters=%d", coefficient,
            eps, max_iters);
  const int stop_after = (int)env_double("FAKE_STOP_AFTER", -1.0);
  *rro0 = env_double("FAKE_RRO0", 1.0);
  int n = 0;
  for (int k = 0; k < max_iters; ++k) {
    pw_hist[k] = pw_of(k);
    rrn_hist[k] = rrn_of(k);
    n = k + 1;
    if (sqrt(fabs(rrn_hist[k])) < eps) break;
    if (stop_after >= 0 && n >= stop_after) break;
  }
  *steps = n;
  return TL_OK;
}

int tl_cg_init(tl_context*, int, int, int, int coefficient, double, double, double*, double*,
               double*, double*, double*, double*, const double*, const double*,
               double* rro) {
  FAKE_CALL("tl_cg_init", "tl_cg_init coefficient=%d", coefficient);
  g_step = 0;
  *rro += env_double("FAKE_RRO0", 1.0);
  return TL_OK;
}

int tl_cg_calc_w(tl_context*, int, int, int, double*, const double*, const double*,
                 const double*, double* pw) {
  FAKE_CALL("tl_cg_calc_w", "tl_cg_calc_w");
  *pw += pw_of(g_step);
  return TL_OK;
}

int tl_cg_calc_ur(tl_context*, int, int, int, double*, double*, const double*, const double*,
                  double alpha, double* rrn) {
  FAKE_CALL("tl_cg_calc_ur", "tl_cg_calc_ur alpha=%.17g", alpha);
  *rrn = rrn_of(g_step);
  return TL_OK;
}

int tl_cg_calc_p(tl_context*, int, int, int, double beta, double*, const double*) {
  FAKE_CALL("tl_cg_calc_p", "tl_cg_calc_p beta=%.17g", beta);
  ++g_step;
  return TL_OK;
}

int tl_copy_u(tl_context*, int, int, int, const double*, double*) {
  FAKE_CALL("tl_copy_u", "tl_copy_u");
  return TL_OK;
}

int tl_calculate_residual(tl_context*, int, int, int, const double*, const double*, double*,
                          const double*, const double*) {
  FAKE_CALL("tl_calculate_residual", "tl_calculate_residual");
  return TL_OK;
}

int tl_calculate_2norm(tl_context*, int, int, int, const double*, double* norm) {
  FAKE_CALL("tl_calculate_2norm", "tl_calculate_2norm");
  *norm = 0.0;
  return TL_OK;
}

int tl_finalise(tl_context*, int, int, int, const double*, const double*, double*) {
  FAKE_CALL("tl_finalise", "tl_finalise");
  return TL_OK;
}

int tl_jacobi_init(tl_context*, int, int, int, int, double, double, double*, double*,
                   const double*, const double*, double*, double*) {
  FAKE_CALL("tl_jacobi_init", "tl_jacobi_init");
  return TL_OK;
}

int tl_jacobi_iterate(tl_context*, int, int, int, double*, const double*, double*,
                      const double*, const double*, double* error) {
  FAKE_CALL("tl_jacobi_iterate", "tl_jacobi_iterate");
  *error = 0.0;
  return TL_OK;
}

int tl_cheby_init(tl_context*, int, int, int, double, double*, double*, const double*,
                  const double*, double*, const double*, const double*) {
  FAKE_CALL("tl_cheby_init", "tl_cheby_init");
  return TL_OK;
}

int tl_cheby_iterate(tl_context*, int, int, int, double, double, double*, double*, double*,
                     const double*, double*, const double*, const double*) {
  FAKE_CALL("tl_cheby_iterate", "tl_cheby_iterate");
  return TL_OK;
}

int tl_ppcg_init(tl_context*, int, int, int, double, double*, const double*) {
  FAKE_CALL("tl_ppcg_init", "tl_ppcg_init");
  return TL_OK;
}

int tl_ppcg_inner_iteration(tl_context*, int, int, int, double, double, double, double*,
                            double*, double*, const double*, const double*) {
  FAKE_CALL("tl_ppcg_inner_iteration", "tl_ppcg_inner_iteration");
  return TL_OK;
}

int tl_solve(tl_context*, int, int, int, int, double, double, const tl_solve_params* prm,
             double*, double*, double*, double*, double*, double*, double*, const double*,
             const double*, tl_solve_report* rep) {
  FAKE_CALL("tl_solve",
            "tl_solve method=%d rel_tol=%.17g inner_tol=%.17g max_inner=%d learned=%d "
            "projection=%d",
            prm->method, prm->rel_tol, prm->inner_tol, prm->max_inner, prm->learned != nullptr,
            prm->projection);
  memset(rep, 0, sizeof(*rep));
  rep->outer_steps = 3;
  rep->inner_steps = 123;
  rep->initial_rel_residual = 1.0;
  /* FAKE_UNCONVERGED=1: a solve that ended above its target */
  rep->final_rel_residual = getenv("FAKE_UNCONVERGED") ? 4.0 * prm->rel_tol
                                                      : 0.5 * prm->rel_tol;
  rep->device_ms = 1.0f;
  rep->inner_kernel_ms = 0.5f;
  return TL_OK;
}

int tl_net_num_params(void) { return 7056; }

int tl_net_create(tl_context*, tl_net** out) {
  FAKE_CALL("tl_net_create", "tl_net_create");
  *out = new tl_net{0};
  return TL_OK;
}

int tl_net_set_weights(tl_net* net, const float* w, int n) {
  FAKE_CALL("tl_net_set_weights", "tl_net_set_weights n=%d first=%.9g last=%.9g", n,
            (double)w[0], (double)w[n - 1]);
  net->n = n;
  return TL_OK;
}

int tl_net_destroy(tl_net* net) {
  FAKE_CALL("tl_net_destroy", "tl_net_destroy");
  delete net;
  return TL_OK;
}

}  // extern "C"
