/*
 * tl_oracle.c -- CPU oracle for the TeaLeaf CG hot path (test infrastructure).
 *
 * A plain-C restatement of the semantics of the reference's SYCL kernels in
 * TeaLeaf/c_kernels/sycl/. Each function names the reference lines it follows.
 * Used only by tests/, the smoke check and bench.py's CPU baseline; the
 * product never links it.
 *
 * Reduction order. The reference reduces every dot product in two stages:
 *  (1) each work-group of 64 consecutive linear indices (halo cells included,
 *      contributing 0) sums its values with a pairwise tree whose stride
 *      doubles from 1 to 32 (TeaLeaf/c_kernels/sycl/cg.cpp:113-126);
 *  (2) the vector of group sums is reduced again by the same 64-wide tree,
 *      level after level, until one value is left
 *      (TeaLeaf/c_kernels/sycl/sycl_shared.hpp:35-79), padding with zeros.
 * orc_tree64() and reduce_levels() restate that order. The reference's
 * second stage writes each level in place, so a group may read a slot that
 * another group has already overwritten (a data race that real devices rarely
 * expose); the oracle keeps the intended, race-free meaning by reducing each
 * level into a separate buffer.
 *
 * Must be compiled with -ffp-contract=off (see oracle/Makefile).
 */
#include "tl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define WG 64

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Pairwise tree over 64 values, stride 1, 2, 4, ..., 32
 * (TeaLeaf/c_kernels/sycl/cg.cpp:115-121). */
static double orc_tree64(double* a) {
  for (int stride = 1; stride < WG; stride *= 2) {
    for (int i = 0; i < WG; i += 2 * stride) {
      a[i] = a[i] + a[i + stride];
    }
  }
  return a[0];
}

/* Second stage: reduce n partial sums level by level with the 64-wide tree
 * (TeaLeaf/c_kernels/sycl/sycl_shared.hpp:35-79). Consumes `part`. */
static double reduce_levels(double* part, long n) {
  double* next = (double*)malloc(sizeof(double) * (size_t)((n + WG - 1) / WG + 1));
  while (n != 1) {
    long ng = (n + WG - 1) / WG;
#pragma omp parallel for if (ng > 256) schedule(static)
    for (long g = 0; g < ng; ++g) {
      double a[WG];
      for (int l = 0; l < WG; ++l) {
        long idx = g * WG + l;
        a[l] = (idx < n) ? part[idx] : 0.0;
      }
      next[g] = orc_tree64(a);
    }
    memcpy(part, next, sizeof(double) * (size_t)ng);
    n = ng;
  }
  free(next);
  return part[0];
}

double orc_reduce_sycl_order(const double* vals, long n) {
  if (n <= 0) return 0.0;
  long ng = (n + WG - 1) / WG;
  double* part = (double*)malloc(sizeof(double) * (size_t)ng);
#pragma omp parallel for schedule(static)
  for (long g = 0; g < ng; ++g) {
    double a[WG];
    for (int l = 0; l < WG; ++l) {
      long idx = g * WG + l;
      a[l] = (idx < n) ? vals[idx] : 0.0;
    }
    part[g] = orc_tree64(a);
  }
  double s = reduce_levels(part, ng);
  free(part);
  return s;
}

/* Interior test used by every masked kernel. */
#define INTERIOR(kk, jj) \
  ((kk) >= halo_depth && (kk) < x - halo_depth && (jj) >= halo_depth && \
   (jj) < y - halo_depth)

/* The 5-point operator (TeaLeaf/shared.h:59-63), with the same grouping of
 * additions and multiplications. */
static inline double smvp(const double* a, const double* kx, const double* ky,
                          long i, int x) {
  return (1.0 + (kx[i + 1] + kx[i]) + (ky[i + x] + ky[i])) * a[i] -
         (kx[i + 1] * a[i + 1] + kx[i] * a[i - 1]) -
         (ky[i + x] * a[i + x] + ky[i] * a[i - x]);
}

/* Runs a masked kernel body over all linear cells, one 64-cell group per
 * task, and returns the reference-ordered sum of the per-cell contributions
 * (0 outside the interior). BODY must assign `c`. */
#define REDUCING_KERNEL(result, BODY)                                   \
  do {                                                                  \
    long len_ = (long)x * (long)y;                                      \
    long ng_ = (len_ + WG - 1) / WG;                                    \
    double* part_ = (double*)malloc(sizeof(double) * (size_t)ng_);      \
    _Pragma("omp parallel for schedule(static)")                        \
    for (long g_ = 0; g_ < ng_; ++g_) {                                 \
      double a_[WG];                                                    \
      for (int l_ = 0; l_ < WG; ++l_) {                                 \
        long i = g_ * WG + l_;                                          \
        double c = 0.0;                                                 \
        if (i < len_) {                                                 \
          const int kk = (int)(i % x);                                  \
          const int jj = (int)(i / x);                                  \
          if (INTERIOR(kk, jj)) { BODY }                                \
        }                                                               \
        a_[l_] = c;                                                     \
      }                                                                 \
      part_[g_] = orc_tree64(a_);                                       \
    }                                                                   \
    result = reduce_levels(part_, ng_);                                 \
    free(part_);                                                        \
  } while (0)

/* ------------------------------------------------------------------ init */

/* TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:8-28 */
void orc_set_chunk_data_vertices(int x, int y, int halo_depth,
    double* vertex_x, double* vertex_y, double x_min, double y_min,
    double dx, double dy) {
  int n = (x > y ? x : y) + 1;
  for (int i = 0; i < n; ++i) {
    if (i < x + 1) vertex_x[i] = x_min + dx * (i - (double)halo_depth);
    if (i < y + 1) vertex_y[i] = y_min + dy * (i - (double)halo_depth);
  }
}

/* TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:31-64 */
void orc_set_chunk_data(int x, int y, int halo_depth,
    const double* vertex_x, const double* vertex_y, double* cell_x,
    double* cell_y, double* volume, double* x_area, double* y_area,
    double x_min, double y_min, double dx, double dy) {
  (void)halo_depth; (void)x_min; (void)y_min;
  long len = (long)x * y;
  for (int i = 0; i < x; ++i) cell_x[i] = 0.5 * (vertex_x[i] + vertex_x[i + 1]);
  for (int i = 0; i < y; ++i) cell_y[i] = 0.5 * (vertex_y[i] + vertex_y[i + 1]);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    volume[i] = dx * dy;
    x_area[i] = dy;
    y_area[i] = dx;
  }
}

/* TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:8-27 */
void orc_set_chunk_initial_state(int x, int y, double default_energy,
    double default_density, double* energy0, double* density) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    energy0[i] = default_energy;
    density[i] = default_density;
  }
}

/* TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:30-92 */
void orc_set_chunk_state(int x, int y, int halo_depth, const orc_state* s,
    double* energy0, double* density, double* u, const double* cell_x,
    const double* cell_y, const double* vertex_x, const double* vertex_y) {
  (void)halo_depth;
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    int apply = 0;
    if (s->geometry == ORC_RECTANGULAR) {
      apply = vertex_x[kk + 1] >= s->x_min && vertex_x[kk] < s->x_max &&
              vertex_y[jj + 1] >= s->y_min && vertex_y[jj] < s->y_max;
    } else if (s->geometry == ORC_CIRCULAR) {
      double radius = sqrt((cell_x[kk] - s->x_min) * (cell_x[kk] - s->x_min) +
                           (cell_y[jj] - s->y_min) * (cell_y[jj] - s->y_min));
      apply = radius <= s->radius;
    } else if (s->geometry == ORC_POINT) {
      apply = vertex_x[kk] == s->x_min && vertex_y[jj] == s->y_min;
    }
    if (apply) {
      energy0[i] = s->energy;
      density[i] = s->density;
    }
    if (kk > 0 && kk < x - 1 && jj > 0 && jj < y - 1) {
      u[i] = energy0[i] * density[i];
    }
  }
}

/* TeaLeaf/c_kernels/sycl/store_energy.cpp:6-24 */
void orc_store_energy(int x, int y, double* energy, const double* energy0) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) energy[i] = energy0[i];
}

/* ----------------------------------------------------------------- halos */

/* TeaLeaf/c_kernels/sycl/local_halos.cpp:7-102. Left/right reflect `depth`
 * columns on every row; top/bottom reflect `depth` full rows (corners
 * included), so the caller must apply faces in the order L, R, T, B. */
void orc_update_face(int x, int y, int halo_depth, double* f, int face,
    int depth) {
  if (face == ORC_CHUNK_LEFT) {
    for (int jj = 0; jj < y; ++jj)
      for (int flip = 0; flip < depth; ++flip)
        f[(long)jj * x + halo_depth - depth + flip] =
            f[(long)jj * x + halo_depth + depth - flip - 1];
  } else if (face == ORC_CHUNK_RIGHT) {
    for (int jj = 0; jj < y; ++jj)
      for (int flip = 0; flip < depth; ++flip)
        f[(long)jj * x + x - halo_depth + flip] =
            f[(long)jj * x + x - halo_depth - 1 - flip];
  } else if (face == ORC_CHUNK_TOP) {
    for (int line = 0; line < depth; ++line)
      for (int kk = 0; kk < x; ++kk)
        f[(long)(y - halo_depth + line) * x + kk] =
            f[(long)(y - halo_depth - 1 - line) * x + kk];
  } else if (face == ORC_CHUNK_BOTTOM) {
    for (int line = 0; line < depth; ++line)
      for (int kk = 0; kk < x; ++kk)
        f[(long)(halo_depth - 1 - line) * x + kk] =
            f[(long)(halo_depth + line) * x + kk];
  }
}

/* TeaLeaf/c_kernels/sycl/pack_halos.cpp:7-184 */
void orc_pack_or_unpack(int x, int y, int halo_depth, int depth, int face,
    int pack, double* field, double* buffer) {
  if (face == ORC_CHUNK_LEFT || face == ORC_CHUNK_RIGHT) {
    int col = 0;
    if (face == ORC_CHUNK_LEFT) col = pack ? halo_depth : halo_depth - depth;
    else col = pack ? x - halo_depth - depth : x - halo_depth;
    for (int jj = 0; jj < y; ++jj)
      for (int d = 0; d < depth; ++d) {
        long fi = (long)jj * x + col + d;
        long bi = (long)jj * depth + d;
        if (pack) buffer[bi] = field[fi]; else field[fi] = buffer[bi];
      }
  } else {
    int row = 0;
    if (face == ORC_CHUNK_BOTTOM) row = pack ? halo_depth : halo_depth - depth;
    else row = pack ? y - halo_depth - depth : y - halo_depth;
    for (long i = 0; i < (long)x * depth; ++i) {
      long fi = (long)row * x + i;
      if (pack) buffer[i] = field[fi]; else field[fi] = buffer[i];
    }
  }
}

/* --------------------------------------------------------- field summary */

/* TeaLeaf/c_kernels/sycl/field_summary.cpp:6-151: four sums, each in the
 * reference order; the outputs are overwritten, not accumulated
 * (field_summary.cpp:147-150). */
void orc_field_summary(int x, int y, int halo_depth, const double* u,
    const double* density, const double* energy0, const double* volume,
    double* vol, double* mass, double* ie, double* temp) {
  long len = (long)x * y;
  double* cv = (double*)malloc(sizeof(double) * (size_t)len);
  double* cm = (double*)malloc(sizeof(double) * (size_t)len);
  double* ci = (double*)malloc(sizeof(double) * (size_t)len);
  double* ct = (double*)malloc(sizeof(double) * (size_t)len);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    cv[i] = cm[i] = ci[i] = ct[i] = 0.0;
    if (INTERIOR(kk, jj)) {
      const double cell_vol = volume[i];
      const double cell_mass = cell_vol * density[i];
      cv[i] = cell_vol;
      cm[i] = cell_mass;
      ci[i] = cell_mass * energy0[i];
      ct[i] = cell_mass * u[i];
    }
  }
  *vol = orc_reduce_sycl_order(cv, len);
  *mass = orc_reduce_sycl_order(cm, len);
  *ie = orc_reduce_sycl_order(ci, len);
  *temp = orc_reduce_sycl_order(ct, len);
  free(cv); free(cm); free(ci); free(ct);
}

/* -------------------------------------------------------------------- CG */

/* TeaLeaf/c_kernels/sycl/cg.cpp:7-37 */
void orc_cg_init_u(int x, int y, int coefficient, double* p, double* r,
    double* u, double* w, const double* density, const double* energy) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    p[i] = 0.0;
    r[i] = 0.0;
    u[i] = energy[i] * density[i];
    if (jj > 0 && jj < y - 1 && kk > 0 && kk < x - 1) {
      w[i] = (coefficient == ORC_CONDUCTIVITY) ? density[i] : 1.0 / density[i];
    }
  }
}

/* TeaLeaf/c_kernels/sycl/cg.cpp:40-69 */
void orc_cg_init_k(int x, int y, int halo_depth, const double* w, double* kx,
    double* ky, double rx, double ry) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (jj >= halo_depth && jj < y - 1 && kk >= halo_depth && kk < x - 1) {
      kx[i] = rx * (w[i - 1] + w[i]) / (2.0 * w[i - 1] * w[i]);
      ky[i] = ry * (w[i - x] + w[i]) / (2.0 * w[i - x] * w[i]);
    }
  }
}

/* TeaLeaf/c_kernels/sycl/cg.cpp:72-134; rro is accumulated (cg.cpp:133). */
void orc_cg_init_others(int x, int y, int halo_depth, const double* kx,
    const double* ky, double* p, double* r, const double* u, double* w,
    double* rro) {
  double s;
  REDUCING_KERNEL(s, {
    w[i] = smvp(u, kx, ky, i, x);
    r[i] = u[i] - w[i];
    p[i] = r[i];
    c = r[i] * p[i];
  });
  *rro += s;
}

/* TeaLeaf/c_kernels/sycl/cg.cpp:137-195; pw is accumulated (cg.cpp:194). */
void orc_cg_calc_w(int x, int y, int halo_depth, double* w, const double* p,
    const double* kx, const double* ky, double* pw) {
  double s;
  REDUCING_KERNEL(s, {
    w[i] = smvp(p, kx, ky, i, x);
    c = w[i] * p[i];
  });
  *pw += s;
}

/* TeaLeaf/c_kernels/sycl/cg.cpp:198-254; rrn is overwritten (cg.cpp:253). */
void orc_cg_calc_ur(int x, int y, int halo_depth, double* u, double* r,
    const double* p, const double* w, double alpha, double* rrn) {
  double s;
  REDUCING_KERNEL(s, {
    u[i] += alpha * p[i];
    r[i] -= alpha * w[i];
    c = r[i] * r[i];
  });
  *rrn = s;
}

/* TeaLeaf/c_kernels/sycl/cg.cpp:257-281 */
void orc_cg_calc_p(int x, int y, int halo_depth, double beta, double* p,
    const double* r) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) p[i] = beta * p[i] + r[i];
  }
}

/* ------------------------------------------------ fused FP64 contract
 * The arithmetic of the GPU's TL_FP64_FUSED persistent CG
 * (include/tealeaf_gb300.h, tl_set_fp64_contract): C's fma() is correctly
 * rounded, as the GPU's fused multiply-add. The reduction order is the
 * reference's; only the first tree level pairs (a0*b0, a1*b1) become
 * fma(a0, b0, a1*b1). */

static double orc_tree64_fused(const double* ca, const double* cb) {
  double a[WG];
  for (int i = 0; i < WG; i += 2) a[i] = fma(ca[i], cb[i], ca[i + 1] * cb[i + 1]);
  for (int stride = 2; stride < WG; stride *= 2) {
    for (int i = 0; i < WG; i += 2 * stride) a[i] = a[i] + a[i + stride];
  }
  return a[0];
}

/* As REDUCING_KERNEL; BODY assigns the factors ca, cb of the cell's term
 * (0, 0 outside the interior). */
#define REDUCING_KERNEL_FUSED(result, BODY)                             \
  do {                                                                  \
    long len_ = (long)x * (long)y;                                      \
    long ng_ = (len_ + WG - 1) / WG;                                    \
    double* part_ = (double*)malloc(sizeof(double) * (size_t)ng_);      \
    _Pragma("omp parallel for schedule(static)")                        \
    for (long g_ = 0; g_ < ng_; ++g_) {                                 \
      double a_[WG], b_[WG];                                            \
      for (int l_ = 0; l_ < WG; ++l_) {                                 \
        long i = g_ * WG + l_;                                          \
        double ca = 0.0, cb = 0.0;                                      \
        if (i < len_) {                                                 \
          const int kk = (int)(i % x);                                  \
          const int jj = (int)(i / x);                                  \
          if (INTERIOR(kk, jj)) { BODY }                                \
        }                                                               \
        a_[l_] = ca;                                                    \
        b_[l_] = cb;                                                    \
      }                                                                 \
      part_[g_] = orc_tree64_fused(a_, b_);                             \
    }                                                                   \
    result = reduce_levels(part_, ng_);                                 \
    free(part_);                                                        \
  } while (0)

/* w = A p as diag*p minus the right, left, up and down neighbour terms by
 * fused multiply-adds, diag grouped as in smvp(); pw accumulated. */
void orc_cg_calc_w_fused(int x, int y, int halo_depth, double* w, const double* p,
    const double* kx, const double* ky, double* pw) {
  double s;
  REDUCING_KERNEL_FUSED(s, {
    const double diag = 1.0 + (kx[i + 1] + kx[i]) + (ky[i + x] + ky[i]);
    double t = diag * p[i];
    t = fma(-kx[i + 1], p[i + 1], t);
    t = fma(-kx[i], p[i - 1], t);
    t = fma(-ky[i + x], p[i + x], t);
    t = fma(-ky[i], p[i - x], t);
    w[i] = t;
    ca = t;
    cb = p[i];
  });
  *pw += s;
}

void orc_cg_calc_ur_fused(int x, int y, int halo_depth, double* u, double* r,
    const double* p, const double* w, double alpha, double* rrn) {
  double s;
  REDUCING_KERNEL_FUSED(s, {
    u[i] = fma(alpha, p[i], u[i]);
    r[i] = fma(-alpha, w[i], r[i]);
    ca = r[i];
    cb = r[i];
  });
  *rrn = s;
}

void orc_cg_calc_p_fused(int x, int y, int halo_depth, double beta, double* p,
    const double* r) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) p[i] = fma(beta, p[i], r[i]);
  }
}

/* -------------------------------------------------------- solver methods */

/* TeaLeaf/c_kernels/sycl/solver_methods.cpp:7-31 */
void orc_copy_u(int x, int y, int halo_depth, const double* u, double* u0) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) u0[i] = u[i];
  }
}

/* TeaLeaf/c_kernels/sycl/solver_methods.cpp:34-65 */
void orc_calculate_residual(int x, int y, int halo_depth, const double* u,
    const double* u0, double* r, const double* kx, const double* ky) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) {
      const double s = smvp(u, kx, ky, i, x);
      r[i] = u0[i] - s;
    }
  }
}

/* TeaLeaf/c_kernels/sycl/solver_methods.cpp:68-117; norm is overwritten
 * (solver_methods.cpp:116). */
void orc_calculate_2norm(int x, int y, int halo_depth, const double* buffer,
    double* norm) {
  double s;
  REDUCING_KERNEL(s, { c = buffer[i] * buffer[i]; });
  *norm = s;
}

/* TeaLeaf/c_kernels/sycl/solver_methods.cpp:120-145 */
void orc_finalise(int x, int y, int halo_depth, const double* u,
    const double* density, double* energy) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) energy[i] = u[i] / density[i];
  }
}

/* ---------------------------------------------------------------- Jacobi */

/* TeaLeaf/c_kernels/sycl/jacobi.cpp:7-56 */
void orc_jacobi_init(int x, int y, int halo_depth, int coefficient, double rx,
    double ry, double* u, double* u0, const double* density,
    const double* energy, double* kx, double* ky) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (kk > 0 && kk < x - 1 && jj > 0 && jj < y - 1) {
      u0[i] = energy[i] * density[i];
      u[i] = u0[i];
    }
    if (jj >= halo_depth && jj < y - 1 && kk >= halo_depth && kk < x - 1) {
      const int cond = coefficient == ORC_CONDUCTIVITY;
      double dc = cond ? density[i] : 1.0 / density[i];
      double dl = cond ? density[i - 1] : 1.0 / density[i - 1];
      double dd = cond ? density[i - x] : 1.0 / density[i - x];
      kx[i] = rx * (dl + dc) / (2.0 * dl * dc);
      ky[i] = ry * (dd + dc) / (2.0 * dd * dc);
    }
  }
}

/* TeaLeaf/c_kernels/sycl/jacobi.cpp:122-137 */
void orc_jacobi_copy_u(int x, int y, double* r, const double* u) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) r[i] = u[i];
}

/* TeaLeaf/c_kernels/sycl/jacobi.cpp:59-119; error is overwritten (:118). */
void orc_jacobi_iterate(int x, int y, int halo_depth, double* u,
    const double* u0, const double* r, const double* kx, const double* ky,
    double* error) {
  double s;
  REDUCING_KERNEL(s, {
    u[i] = (u0[i] + (kx[i + 1] * r[i + 1] + kx[i] * r[i - 1]) +
            (ky[i + x] * r[i + x] + ky[i] * r[i - x])) /
           (1.0 + (kx[i] + kx[i + 1]) + (ky[i] + ky[i + x]));
    c = fabs(u[i] - r[i]);
  });
  *error = s;
}

/* ------------------------------------------------------------- Chebyshev */

/* TeaLeaf/c_kernels/sycl/cheby.cpp:7-38 */
void orc_cheby_init(int x, int y, int halo_depth, double theta, double* p,
    double* r, const double* u, const double* u0, double* w,
    const double* kx, const double* ky) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) {
      w[i] = smvp(u, kx, ky, i, x);
      r[i] = u0[i] - w[i];
      p[i] = r[i] / theta;
    }
  }
}

/* TeaLeaf/c_kernels/sycl/cheby.cpp:67-110 */
void orc_cheby_iterate(int x, int y, int halo_depth, double alpha,
    double beta, double* p, double* r, const double* u, const double* u0,
    double* w, const double* kx, const double* ky) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) {
      w[i] = smvp(u, kx, ky, i, x);
      r[i] = u0[i] - w[i];
      p[i] = alpha * p[i] + beta * r[i];
    }
  }
}

/* TeaLeaf/c_kernels/sycl/cheby.cpp:41-64 */
void orc_cheby_calc_u(int x, int y, int halo_depth, const double* p,
    double* u) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) u[i] += p[i];
  }
}

/* ------------------------------------------------------------------ PPCG */

/* TeaLeaf/c_kernels/sycl/ppcg.cpp:7-30 */
void orc_ppcg_init(int x, int y, int halo_depth, double theta, double* sd,
    const double* r) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) sd[i] = r[i] / theta;
  }
}

/* TeaLeaf/c_kernels/sycl/ppcg.cpp:33-63 */
void orc_ppcg_calc_ur(int x, int y, int halo_depth, const double* sd,
    double* r, double* u, const double* kx, const double* ky) {
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) {
      const double s = smvp(sd, kx, ky, i, x);
      r[i] -= s;
      u[i] += sd[i];
    }
  }
}

/* TeaLeaf/c_kernels/sycl/ppcg.cpp:66-94 */
void orc_ppcg_calc_sd(int x, int y, int halo_depth, double theta,
    double alpha, double beta, double* sd, const double* r) {
  (void)theta;
  long len = (long)x * y;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < len; ++i) {
    const int kk = (int)(i % x);
    const int jj = (int)(i / x);
    if (INTERIOR(kk, jj)) sd[i] = alpha * sd[i] + beta * r[i];
  }
}
