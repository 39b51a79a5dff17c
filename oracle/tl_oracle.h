/*
 * tl_oracle.h -- CPU oracle for the TeaLeaf CG hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library restates, on the host, the
 * semantics of the reference's SYCL kernel backend
 * (TeaLeaf/c_kernels/sycl/*.cpp) so that the GB300 CUDA path can be checked
 * against it. Nothing in the product (exploringsycl_gb300/) links or calls
 * it; only tests/, the smoke check and the CPU-baseline leg of bench.py do.
 *
 * Every reducing kernel reproduces the reference's summation order exactly:
 * a 64-wide pairwise tree over consecutive linear cell indices
 * (TeaLeaf/c_kernels/sycl/cg.cpp:113-126) followed by the same 64-wide tree
 * applied level by level to the partial sums
 * (TeaLeaf/c_kernels/sycl/sycl_shared.hpp:35-79), with zero padding. The
 * library must be compiled with -ffp-contract=off so that no multiply-add is
 * fused; with that, every result is a deterministic function of the inputs.
 *
 * Field layout (all kernels): row-major doubles, index kk + jj*x, with
 * x = x_cells + 2*halo_depth and y = y_cells + 2*halo_depth; the interior
 * is kk in [halo_depth, x-halo_depth), jj in [halo_depth, y-halo_depth).
 *
 * Parity status: pinned. The oracle kernels linked under the reference's own
 * unchanged host driver reproduce TeaLeaf/tea.problems to the driver's
 * 0.001 % check (see oracle/Makefile target `ref` and tests/test_oracle_*).
 */
#ifndef TL_ORACLE_H
#define TL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry codes follow the order of the reference's Geometry enum
 * (TeaLeaf/settings.h:130-135). */
#define ORC_RECTANGULAR 0
#define ORC_CIRCULAR 1
#define ORC_POINT 2

/* Faces, as numbered by the reference (TeaLeaf/shared.h:34-37). */
#define ORC_CHUNK_LEFT 0
#define ORC_CHUNK_RIGHT 1
#define ORC_CHUNK_BOTTOM 2
#define ORC_CHUNK_TOP 3

#define ORC_CONDUCTIVITY 1
#define ORC_RECIP_CONDUCTIVITY 2

typedef struct orc_state {
  double density;
  double energy;
  double x_min;
  double y_min;
  double x_max;
  double y_max;
  double radius;
  int geometry;
} orc_state;

/* Number of worker threads used by the oracle (OpenMP); 1 without OpenMP. */
int orc_num_threads(void);
void orc_set_num_threads(int n);

/* Sum of vals[0..n) in the reference's reduction order (64-wide pairwise
 * tree, recursively over partials). Exposed for the reduction unit tests. */
double orc_reduce_sycl_order(const double* vals, long n);

/* --- initialisation (TeaLeaf/c_kernels/sycl/set_chunk_data.cpp,
 *     set_chunk_state.cpp, store_energy.cpp) --- */
void orc_set_chunk_data_vertices(int x, int y, int halo_depth,
    double* vertex_x, double* vertex_y, double x_min, double y_min,
    double dx, double dy);
void orc_set_chunk_data(int x, int y, int halo_depth,
    const double* vertex_x, const double* vertex_y, double* cell_x,
    double* cell_y, double* volume, double* x_area, double* y_area,
    double x_min, double y_min, double dx, double dy);
void orc_set_chunk_initial_state(int x, int y, double default_energy,
    double default_density, double* energy0, double* density);
void orc_set_chunk_state(int x, int y, int halo_depth, const orc_state* state,
    double* energy0, double* density, double* u, const double* cell_x,
    const double* cell_y, const double* vertex_x, const double* vertex_y);
void orc_store_energy(int x, int y, double* energy, const double* energy0);

/* --- halos (TeaLeaf/c_kernels/sycl/local_halos.cpp) --- */
void orc_update_face(int x, int y, int halo_depth, double* field, int face,
    int depth);
/* pack (pack != 0) copies the face strip into buffer; unpack copies it back
 * (TeaLeaf/c_kernels/sycl/pack_halos.cpp). */
void orc_pack_or_unpack(int x, int y, int halo_depth, int depth, int face,
    int pack, double* field, double* buffer);

/* --- field summary (TeaLeaf/c_kernels/sycl/field_summary.cpp) --- */
void orc_field_summary(int x, int y, int halo_depth, const double* u,
    const double* density, const double* energy0, const double* volume,
    double* vol, double* mass, double* ie, double* temp);

/* --- CG (TeaLeaf/c_kernels/sycl/cg.cpp) --- */
void orc_cg_init_u(int x, int y, int coefficient, double* p, double* r,
    double* u, double* w, const double* density, const double* energy);
void orc_cg_init_k(int x, int y, int halo_depth, const double* w, double* kx,
    double* ky, double rx, double ry);
void orc_cg_init_others(int x, int y, int halo_depth, const double* kx,
    const double* ky, double* p, double* r, const double* u, double* w,
    double* rro);
void orc_cg_calc_w(int x, int y, int halo_depth, double* w, const double* p,
    const double* kx, const double* ky, double* pw);
void orc_cg_calc_ur(int x, int y, int halo_depth, double* u, double* r,
    const double* p, const double* w, double alpha, double* rrn);
void orc_cg_calc_p(int x, int y, int halo_depth, double beta, double* p,
    const double* r);
/* The fused FP64 contract of the GPU's persistent CG (TL_FP64_FUSED). */
void orc_cg_calc_w_fused(int x, int y, int halo_depth, double* w, const double* p,
    const double* kx, const double* ky, double* pw);
void orc_cg_calc_ur_fused(int x, int y, int halo_depth, double* u, double* r,
    const double* p, const double* w, double alpha, double* rrn);
void orc_cg_calc_p_fused(int x, int y, int halo_depth, double beta, double* p,
    const double* r);

/* --- shared solver methods (TeaLeaf/c_kernels/sycl/solver_methods.cpp) --- */
void orc_copy_u(int x, int y, int halo_depth, const double* u, double* u0);
void orc_calculate_residual(int x, int y, int halo_depth, const double* u,
    const double* u0, double* r, const double* kx, const double* ky);
void orc_calculate_2norm(int x, int y, int halo_depth, const double* buffer,
    double* norm);
void orc_finalise(int x, int y, int halo_depth, const double* u,
    const double* density, double* energy);

/* --- Jacobi (TeaLeaf/c_kernels/sycl/jacobi.cpp) --- */
void orc_jacobi_init(int x, int y, int halo_depth, int coefficient, double rx,
    double ry, double* u, double* u0, const double* density,
    const double* energy, double* kx, double* ky);
void orc_jacobi_copy_u(int x, int y, double* r, const double* u);
void orc_jacobi_iterate(int x, int y, int halo_depth, double* u,
    const double* u0, const double* r, const double* kx, const double* ky,
    double* error);

/* --- Chebyshev (TeaLeaf/c_kernels/sycl/cheby.cpp) --- */
void orc_cheby_init(int x, int y, int halo_depth, double theta, double* p,
    double* r, const double* u, const double* u0, double* w,
    const double* kx, const double* ky);
void orc_cheby_iterate(int x, int y, int halo_depth, double alpha,
    double beta, double* p, double* r, const double* u, const double* u0,
    double* w, const double* kx, const double* ky);
void orc_cheby_calc_u(int x, int y, int halo_depth, const double* p,
    double* u);

/* --- PPCG (TeaLeaf/c_kernels/sycl/ppcg.cpp) --- */
void orc_ppcg_init(int x, int y, int halo_depth, double theta, double* sd,
    const double* r);
void orc_ppcg_calc_ur(int x, int y, int halo_depth, const double* sd,
    double* r, double* u, const double* kx, const double* ky);
void orc_ppcg_calc_sd(int x, int y, int halo_depth, double theta,
    double alpha, double beta, double* sd, const double* r);

#ifdef __cplusplus
}
#endif

#endif /* TL_ORACLE_H */
