/*
 * tealeaf_gb300.h -- C ABI of the GB300 TeaLeaf kernel backend.
 *
 * Plain C: device pointers, sizes and host scalars, no C++ or framework types.
 * The kernel entry points mirror, one for one, the kernel functions that the
 * reference's SYCL backend calls from its run_* layer
 * (TeaLeaf/c_kernels/sycl/c_kernels.hpp:1-217, dispatched from
 * TeaLeaf/c_kernels/sycl/kernel_interface.cpp:34-371); each declaration
 * names the reference function it replaces. A TeaLeaf maintainer binds them
 * from a C++ run_* layer (exploringsycl_gb300/backend/kernel_interface.cpp).
 *
 * Conventions
 *  - Fields are device arrays of doubles in the reference layout: row-major,
 *    index kk + jj*x, x = x_cells + 2*halo_depth, y = y_cells + 2*halo_depth,
 *    interior kk in [halo_depth, x-halo_depth), jj in [halo_depth, y-halo_depth).
 *    Allocate them with tl_field_alloc (256-byte aligned, zero-filled).
 *    A grid holds at most TL_MAX_CELLS cells, halos included (23,170^2; the
 *    deterministic reductions keep every partial sum of one level in one
 *    block's shared memory); calls on larger grids return TL_ERR_ARG.
 *  - Every call is issued on the context's stream. Calls that return a
 *    scalar through a host pointer synchronise that stream before returning;
 *    the others return as soon as the work is queued.
 *  - Scalars follow the reference: rro and pw are accumulated (+=), while
 *    rrn, norm, error and the field summary are overwritten
 *    (TeaLeaf/c_kernels/sycl/cg.cpp:133,194,253; solver_methods.cpp:116;
 *    jacobi.cpp:116; field_summary.cpp:147-150).
 *  - Reductions are deterministic and follow the reference's summation
 *    order exactly (64-wide pairwise trees over consecutive linear cells,
 *    then over partial sums: TeaLeaf/c_kernels/sycl/cg.cpp:113-126,
 *    sycl_shared.hpp:35-79), and the double-precision kernels round every
 *    product and sum separately, so results are bit-identical to a
 *    sequential evaluation of the reference's expressions.
 *  - Return value: TL_OK or an error code; tl_last_error() describes the
 *    most recent failure on the calling thread.
 */
#ifndef TEALEAF_GB300_H
#define TEALEAF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TL_OK 0
#define TL_ERR_CUDA 1      /* a CUDA call failed (message has details) */
#define TL_ERR_ARG 2       /* invalid argument (null pointer, bad size) */
#define TL_ERR_TIMEOUT 3   /* a bounded in-kernel wait gave up */
#define TL_ERR_STATE 4     /* call out of sequence */
#define TL_ERR_NUMERIC 5   /* non-finite value or breakdown in a solver */

/* Largest grid, x*y cells including halos (131,072 reduction tiles of 4096). */
#define TL_MAX_CELLS 536870912

/* Geometry codes of a state (TeaLeaf/settings.h:130-135). */
#define TL_RECTANGULAR 0
#define TL_CIRCULAR 1
#define TL_POINT 2

/* Faces (TeaLeaf/shared.h:34-37). */
#define TL_CHUNK_LEFT 0
#define TL_CHUNK_RIGHT 1
#define TL_CHUNK_BOTTOM 2
#define TL_CHUNK_TOP 3

/* Coefficient kinds (TeaLeaf/shared.h:47-48). */
#define TL_CONDUCTIVITY 1
#define TL_RECIP_CONDUCTIVITY 2

typedef struct tl_context tl_context;

/* One initial state of the deck (TeaLeaf/settings.h:137-145). */
typedef struct tl_state {
  double density;
  double energy;
  double x_min;
  double y_min;
  double x_max;
  double y_max;
  double radius;
  int geometry;
} tl_state;

/* ------------------------------------------------------------ context
 * Replaces the SYCL queue the reference creates in kernel_initialise
 * (TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:47) and the temporary
 * reduction buffers each reducing kernel allocates
 * (TeaLeaf/c_kernels/sycl/cg.cpp:80,145,206): a context owns a CUDA stream
 * (or borrows the caller's), reduction scratch, pinned result slots and an
 * error flag. `stream` may be NULL (the context creates its own). */
int tl_context_create(int device, void* stream, tl_context** out);
int tl_context_destroy(tl_context* ctx);
int tl_context_stream(tl_context* ctx, void** stream);
int tl_synchronize(tl_context* ctx);
const char* tl_last_error(void);
/* Number of this library's kernel launches issued on the context so far. */
long long tl_launch_count(tl_context* ctx);

/* Arithmetic contract of the persistent FP64 CG solve (tl_cg_solve, the
 * run-ahead path of run_cg_init, and TL_METHOD_CG64). TL_FP64_EXACT (the
 * default): no fused multiply-adds, each operation rounded as the
 * reference's C kernels compiled without contraction, bit-identical to the
 * CPU oracle. TL_FP64_FUSED: the stencil as diag*p followed by four fused
 * multiply-adds (right, left, up, down neighbours), u += alpha p,
 * r -= alpha w and p = beta p + r as single fused operations, and the first
 * level of each dot-product tree as fma(a0, b0, a1*b1): 11 instead of 19
 * FP64 instructions per cell and step, bit-identical to the oracle's fused
 * mode. No counterpart in the reference (whose GPU builds leave contraction
 * to the compiler). The step-wise kernels always use the exact contract. */
#define TL_FP64_EXACT 0
#define TL_FP64_FUSED 1
int tl_set_fp64_contract(tl_context* ctx, int contract);

/* -------------------------------------------------------------- fields
 * Replace the SYCL buffers of kernel_initialise / kernel_finalise
 * (TeaLeaf/c_kernels/sycl/kernel_initialise.cpp:31-125). */
int tl_field_alloc(tl_context* ctx, size_t count, double** dev_out);
int tl_field_free(tl_context* ctx, double* dev);
int tl_copy_to_device(tl_context* ctx, double* dev, const double* host,
                      size_t count);
int tl_copy_to_host(tl_context* ctx, double* host, const double* dev,
                    size_t count);

/* ---------------------------------------------------- initialisation */
/* set_chunk_data_vertices, TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:8-28 */
int tl_set_chunk_data_vertices(tl_context* ctx, int x, int y, int halo_depth,
                               double* vertex_x, double* vertex_y,
                               double x_min, double y_min, double dx,
                               double dy);
/* set_chunk_data, TeaLeaf/c_kernels/sycl/set_chunk_data.cpp:31-64 */
int tl_set_chunk_data(tl_context* ctx, int x, int y, int halo_depth,
                      const double* vertex_x, const double* vertex_y,
                      double* cell_x, double* cell_y, double* volume,
                      double* x_area, double* y_area, double x_min,
                      double y_min, double dx, double dy);
/* set_chunk_initial_state, TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:8-27 */
int tl_set_chunk_initial_state(tl_context* ctx, int x, int y,
                               double default_energy, double default_density,
                               double* energy0, double* density);
/* set_chunk_state, TeaLeaf/c_kernels/sycl/set_chunk_state.cpp:30-92 */
int tl_set_chunk_state(tl_context* ctx, int x, int y, int halo_depth,
                       const tl_state* state, double* energy0,
                       double* density, double* u, const double* cell_x,
                       const double* cell_y, const double* vertex_x,
                       const double* vertex_y);
/* store_energy, TeaLeaf/c_kernels/sycl/store_energy.cpp:6-24 */
int tl_store_energy(tl_context* ctx, int x, int y, double* energy,
                    const double* energy0);

/* ------------------------------------------------------------- halos */
/* update_left / update_right / update_top / update_bottom,
 * TeaLeaf/c_kernels/sycl/local_halos.cpp:7-102: reflect `depth` layers of
 * one face. */
int tl_update_face(tl_context* ctx, int x, int y, int halo_depth,
                   double* field, int face, int depth);
/* The whole of run_local_halos (TeaLeaf/c_kernels/sycl/kernel_interface.cpp:
 * 100-127) for `nfields` fields in one pass per face pair: faces whose bit
 * (1 << face) is set in face_mask are updated in the order L, R, T, B. */
int tl_local_halos(tl_context* ctx, int x, int y, int halo_depth, int depth,
                   int face_mask, double* const* fields, int nfields);
/* pack_* / unpack_*, TeaLeaf/c_kernels/sycl/pack_halos.cpp:7-184 together
 * with the host mirror copies of kernel_interface.cpp:129-167; `buffer` is
 * host memory of y*depth (left/right) or x*depth (top/bottom) doubles. */
int tl_pack_or_unpack(tl_context* ctx, int x, int y, int halo_depth,
                      int depth, int face, int pack, double* field,
                      double* buffer);

/* ----------------------------------------------------- field summary */
/* field_summary_func, TeaLeaf/c_kernels/sycl/field_summary.cpp:6-151 */
int tl_field_summary(tl_context* ctx, int x, int y, int halo_depth,
                     const double* u, const double* density,
                     const double* energy0, const double* volume,
                     double* vol, double* mass, double* ie, double* temp);

/* ---------------------------------------------------------------- CG */
/* cg_init_u + cg_init_k + cg_init_others,
 * TeaLeaf/c_kernels/sycl/cg.cpp:7-134 (as run_cg_init,
 * kernel_interface.cpp:192-210); rro += r.p */
int tl_cg_init(tl_context* ctx, int x, int y, int halo_depth, int coefficient,
               double rx, double ry, double* p, double* r, double* u,
               double* w, double* kx, double* ky, const double* density,
               const double* energy, double* rro);
/* cg_calc_w, TeaLeaf/c_kernels/sycl/cg.cpp:137-195; pw += w.p */
int tl_cg_calc_w(tl_context* ctx, int x, int y, int halo_depth, double* w,
                 const double* p, const double* kx, const double* ky,
                 double* pw);
/* Allocation-free variant of tl_cg_calc_w. It has no counterpart in the
 * reference. It is for callers that must not allocate device memory once
 * they are running: a TeaLeaf solve embedded in a larger application that
 * owns the device memory budget, or a caller holding a fixed memory pool,
 * where a cudaMalloc (which can fail and can synchronise the whole device)
 * is not allowed mid-run. It takes no context and calls no cudaMalloc,
 * cudaFree or other allocating routine. Its reduction scratch is a fixed
 * file-scope device array of 32770 doubles (about 256 KB) that every GPU
 * loading this library holds until the process exits; grids larger than
 * 134,217,728 cells (32768 tiles of 4096 cells) are rejected with
 * TL_ERR_ARG. The first call on a device, with that device current, looks
 * up the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture. The address is kept for the life of the
 * process: after cudaDeviceReset, or anything else that destroys the
 * device's primary context, do not call this entry point again in that
 * process. Every call shares the array and leaves
 * its last contents there (the ticket word is cleared at each call): calls
 * that overlap on the GPU race, so issue them on one stream or serialise
 * them. `stream` is the caller's cudaStream_t (NULL: the default stream).
 * Results equal tl_cg_calc_w's bit for bit; pw += w.p, and the call
 * synchronises `stream` before returning. */
int tl_cg_calc_w_noalloc(void* stream, int x, int y, int halo_depth, double* w,
                         const double* p, const double* kx, const double* ky,
                         double* pw);
/* cg_calc_ur, TeaLeaf/c_kernels/sycl/cg.cpp:198-254; rrn = r.r */
int tl_cg_calc_ur(tl_context* ctx, int x, int y, int halo_depth, double* u,
                  double* r, const double* p, const double* w, double alpha,
                  double* rrn);
/* cg_calc_p, TeaLeaf/c_kernels/sycl/cg.cpp:257-281 */
int tl_cg_calc_p(tl_context* ctx, int x, int y, int halo_depth, double beta,
                 double* p, const double* r);

/* Whole CG solve of one timestep on the device, for the run-ahead mode of
 * the run_* layer. Equivalent to the reference driver sequence
 * (TeaLeaf/drivers/cg_driver.c:7-66 with the kernels of cg.cpp):
 * cg_init (rro), halo update of u and p (depth 1), u0 = u, then up to
 * max_iters main steps {pw = w.p; alpha = rro/pw; rrn = r.r after the u/r
 * update; beta = rrn/rro; p = beta p + r; halo of u, p} stopping after the
 * first step with sqrt(|rrn|) < eps. Runs as one persistent cooperative
 * kernel with deterministic grid-wide reductions; results and per-step
 * scalars are bit-identical to the step-wise entry points.
 * On return: *rro0 += initial r.p; pw_hist[k], rrn_hist[k] (host arrays of
 * max_iters doubles) hold the scalars of step k; *steps = number of main
 * steps executed (the driver prints steps-1 when it converged). */
int tl_cg_solve(tl_context* ctx, int x, int y, int halo_depth,
                int coefficient, double rx, double ry, double eps,
                int max_iters, double* p, double* r, double* u, double* u0,
                double* w, double* kx, double* ky, const double* density,
                const double* energy, double* rro0, double* pw_hist,
                double* rrn_hist, int* steps);

/* ------------------------------------------- solver-replacement modes
 * Whole-timestep solves with a relative FP64 true-residual stop rule, for
 * the solver-replacement modes of the run_* layer (no counterpart in the
 * reference, which only has the absolute recurrence-residual rule of
 * TeaLeaf/drivers/cg_driver.c:24). Each starts as the reference's
 * cg_init_driver (u = energy*density, kx, ky, halos, u0 = u) and solves
 * A u = u0 until ||u0 - A u||_2 <= rel_tol ||u0||_2 over the interior,
 * measured in FP64 (with the reference's residual kernel for TL_METHOD_CG64
 * from u0; the other paths evaluate the same operator with fused
 * multiply-adds on its precomputed diagonal). TL_METHOD_CG64 from u0 stops as the
 * reference's CG loop does, on its recurrence residual (sqrt(r.r) <= rel_tol
 * ||u0||), so its true residual (final_rel_residual) can end a hair above;
 * from a projected guess, and in every fall-back, FP64 CG restarts from the
 * true residual until that meets the target. */
#define TL_METHOD_CG64 0          /* exact FP64 CG (the drop-in kernel) */
#define TL_METHOD_MIXED_CG 1      /* FP32 inner CG inside FP64 iterative refinement */
#define TL_METHOD_MIXED_JACOBI 2  /* as above, Jacobi-preconditioned inner CG */
#define TL_METHOD_MIXED_LEARNED 3 /* as above, inner PCG with the learned
                                     preconditioner (params->learned) collapsed to
                                     its 17x17 stencil: one persistent kernel,
                                     tensor-core stencil; interior width % 4 == 0 */
#define TL_METHOD_MIXED_LEARNED_COARSE 5 /* as TL_METHOD_MIXED_LEARNED, with a coarse
                                     level added to the preconditioner: M^-1 = the
                                     learned stencil + P (P^T A P)^-1 P^T over
                                     aggregates of 32, 64 or 128 cells square
                                     (interior H and W divisible by it, at most 4096
                                     coarse unknowns; see tl_coarse_inverse) */
#define TL_METHOD_MIXED_LEARNED_LAYERS 4 /* the same solve applying the network layer
                                     by layer (BF16 convolutions, ~25 launches per
                                     step; H % 4 == 0, W % 64 == 0): the reference
                                     point the collapsed stencil is checked against */

typedef struct tl_solve_params {
  int method;           /* TL_METHOD_* */
  double rel_tol;       /* relative FP64 true-residual target */
  double inner_tol;     /* residual reduction asked of each inner FP32 solve;
                           0 selects the method's default (3e-6 for the
                           learned methods, 1e-5 otherwise) */
  int max_inner;        /* inner CG steps per outer step (CG64: total steps) */
  int max_outer;        /* refinement steps; if they end above the target,
                           FP64 CG finishes the solve as after a stall */
  double stall_factor;  /* an outer step must shrink the residual below
                           stall_factor x the previous one, else FP64 CG
                           finishes the solve from the current iterate */
  int max_fallback;     /* FP64 CG steps allowed to the fall-back */
  struct tl_net* learned; /* TL_METHOD_MIXED_LEARNED: the network, else NULL */
  int projection;       /* 0: start from u = u0, as the reference does. 1 ..
                           TL_PROJ_MAX: keep the solutions of up to this many
                           earlier solves with the same operator (kx, ky and
                           the grid, checked by a content hash) in the
                           context, and start from the A-norm best
                           combination of u0 and them when its residual is
                           smaller (successive right-hand sides; see
                           tl_projection_reset) */
} tl_solve_params;

#define TL_PROJ_MAX 8

typedef struct tl_solve_report {
  int outer_steps;
  int inner_steps;
  int fallback_events;
  int fallback_steps;
  double initial_rel_residual;
  double final_rel_residual;  /* ||u0 - A u|| / ||u0|| in FP64 at return */
  float device_ms;            /* whole solve, CUDA events on the context stream */
  float inner_kernel_ms;      /* the persistent inner / CG64 kernels alone */
  int projection_basis;       /* directions of the starting guess (0: u0) */
} tl_solve_report;

int tl_solve(tl_context* ctx, int x, int y, int halo_depth, int coefficient,
             double rx, double ry, const tl_solve_params* params, double* p,
             double* r, double* u, double* u0, double* w, double* kx,
             double* ky, const double* density, const double* energy,
             tl_solve_report* report);
/* Drops the solutions that tl_solve keeps for its starting guesses
 * (tl_solve_params.projection): the next solve starts from u0. */
int tl_projection_reset(tl_context* ctx);

/* ----------------------------------------- learned preconditioner
 * M^-1 = D^-1 + S C^T C S: S = diag(D^-1/2) from the local operator diagonal, C four
 * bias-free 3x3 convolutions (1 -> 16 -> 16 -> 16 -> 16 channels), BF16
 * weights and activations, FP32 accumulation (tensor cores for 16 -> 16).
 * No counterpart in the reference. Arrays are device FP32 [batch][H][W] with
 * H % 4 == 0 and W % 64 == 0. The weight vector (tl_net_num_params() floats)
 * is layer 1 [tap][co] (144) then layers 2..4 [tap][ci][co] (2304 each),
 * tap = 3*(dy+1) + (dx+1) for input offset (dy, dx). */
typedef struct tl_net tl_net;
int tl_net_num_params(void);
/* A network lives on the context it is created on and uses its stream:
 * destroy it before that context. */
int tl_net_create(tl_context* ctx, tl_net** out);
int tl_net_destroy(tl_net* net);
int tl_net_set_weights(tl_net* net, const float* host_weights, int n);
int tl_net_get_weights(tl_net* net, float* host_weights, int n);
/* z = M^-1 r for B images (s = D^-1/2 per cell). */
int tl_net_apply(tl_net* net, int H, int W, int B, const float* r, const float* s,
                 float* z);
/* Training loss sum_b sum (A z - r)^2 / sum_b sum r^2 over cells at least
 * `margin` from the image edge, z = M^-1 r, A the 5-point operator with
 * coupling kx[p] (to the left neighbour) and ky[p] (to the one below);
 * leaves dL/dweights on the device (and in grad_host if not NULL). */
int tl_net_loss_grad(tl_net* net, int H, int W, int B, int margin, const float* r,
                     const float* s, const float* kx, const float* ky, double* loss,
                     float* grad_host);
/* One Adam step (beta1 0.9, beta2 0.999) with the last gradients. */
int tl_net_adam_step(tl_net* net, float lr);
/* The network collapsed to one stencil: C^T C is the 17x17 correlation
 * stencil K(d) = sum_u G(u).G(u + d), G the 16-channel 9x9 kernel of the
 * composed layers, so M^-1 r = D^-1 r + S (K * (S r)) with
 * (K * y)(j) = sum_d K(d) y(j + d) and y zero outside the field. Rebuilt on
 * the device whenever the weights change. host_k receives K (289 floats, row
 * dy = -8..8, column dx = -8..8); kscale (may be NULL) the power of two that
 * scales K before its FP16 rounding for the tensor cores. */
int tl_net_stencil(tl_net* net, float* host_k, float* kscale);
/* z = M^-1 r on one packed FP32 [H][W] field (W % 4 == 0) with the collapsed
 * stencil on the tensor cores (FP16 inputs scaled by 1 / RMS(r), FP32
 * accumulation). */
int tl_net_apply_stencil(tl_net* net, int H, int W, const float* r, const float* s,
                         float* z);
/* The learned PCG on its own, on packed FP32 [H][W] fields (W % 4 == 0):
 * solves A e = b, (A v)_i = v_i + sum over the cell's faces inside the field
 * of k (v_i - v_nb) (kx[j][i] couples cells i-1 and i of row j, ky[j][i] rows
 * j-1 and j; couplings across the field's edges are ignored: zero flux),
 * preconditioned by the network's collapsed stencil, M^-1 = D^-1 + S K S
 * with S = D^-1/2 from the same couplings, by the persistent tensor-core
 * kernel of the learned solver, until r.r <= tol^2 b.b or max_iters steps.
 * b, e and the couplings are device arrays of H*W floats; work holds 7 more.
 * iters and rr (may be NULL) receive the step count and the final r.r. */
int tl_net_pcg(tl_net* net, int H, int W, const float* kx, const float* ky, const float* b,
               float* e, float* work, double tol, int max_iters, int* iters, double* rr);
/* out[b] = crop of data[meta[3b]] at rows meta[3b+1].., columns meta[3b+2]..
 * (data: device [P][HS][WS]; meta: host int triples). */
int tl_net_gather_crops(tl_context* ctx, const float* data, int HS, int WS,
                        const int* meta, int B, int H, int W, float* out);
/* The coarse level of TL_METHOD_MIXED_LEARNED_COARSE for the couplings of a
 * packed FP32 [H][W] field (kx, ky as for tl_net_pcg): P piecewise constant
 * on blk x blk aggregates, blk the smallest of 32, 64, 128 that divides H
 * and W and leaves nc = (H/blk)(W/blk) <= 4096 coarse unknowns (else
 * TL_ERR_ARG), and Ac = P^T A P assembled from the couplings in FP64. Its
 * inverse is built on the device (banded Cholesky, then one band solve per
 * column) and kept in the context, as FP32 rows of nc floats, until H, W or
 * the couplings change. *blk and *nc receive the aggregate size and the
 * coarse size; ainv_host (may be NULL; capacity in floats) a copy of the
 * inverse, row I = Jc * (W/blk) + Ic. No counterpart in the reference. */
int tl_coarse_inverse(tl_context* ctx, int H, int W, const float* kx, const float* ky,
                      int* blk, int* nc, float* ainv_host, size_t capacity);
/* The copy of the same inverse that the two-level kernel reads: every entry
 * times 2^(*exp2) rounded to FP16 (round to nearest even), *exp2 chosen so
 * that the largest entry lies in [2^14, 2^15). half_host (may be NULL;
 * capacity in entries) receives the nc x nc FP16 bit patterns. No
 * counterpart in the reference. */
int tl_coarse_inverse_f16(tl_context* ctx, int H, int W, const float* kx, const float* ky,
                          uint16_t* half_host, size_t capacity, int* exp2);
/* Interior of a field (x*y with halos) to a packed FP32 [H][W] array times
 * scale; and the packed FP32 coefficients with s = D^-1/2. */
int tl_pack_interior(tl_context* ctx, int x, int y, int halo_depth,
                     const double* field, double scale, float* packed);
int tl_pack_coefficients(tl_context* ctx, int x, int y, int halo_depth,
                         const double* kx, const double* ky, float* kx_packed,
                         float* ky_packed, float* s_packed);

/* Device timing of the most recent solve on this context: the persistent
 * kernel alone, measured with CUDA events recorded on the context's stream
 * around its launch, and the number of solver steps it executed. */
typedef struct tl_solve_stats {
  float kernel_ms;
  int steps;
  int kernel_launches;
} tl_solve_stats;
int tl_last_solve_stats(tl_context* ctx, tl_solve_stats* out);

/* ------------------------------------------------- solver methods */
/* copy_u, TeaLeaf/c_kernels/sycl/solver_methods.cpp:7-31 */
int tl_copy_u(tl_context* ctx, int x, int y, int halo_depth, const double* u,
              double* u0);
/* calculate_residual, TeaLeaf/c_kernels/sycl/solver_methods.cpp:34-65 */
int tl_calculate_residual(tl_context* ctx, int x, int y, int halo_depth,
                          const double* u, const double* u0, double* r,
                          const double* kx, const double* ky);
/* calculate_2norm, TeaLeaf/c_kernels/sycl/solver_methods.cpp:68-117 */
int tl_calculate_2norm(tl_context* ctx, int x, int y, int halo_depth,
                       const double* buffer, double* norm);
/* finalise, TeaLeaf/c_kernels/sycl/solver_methods.cpp:120-145 */
int tl_finalise(tl_context* ctx, int x, int y, int halo_depth,
                const double* u, const double* density, double* energy);

/* ------------------------------------------------------------ Jacobi */
/* jacobi_init, TeaLeaf/c_kernels/sycl/jacobi.cpp:7-56 */
int tl_jacobi_init(tl_context* ctx, int x, int y, int halo_depth,
                   int coefficient, double rx, double ry, double* u,
                   double* u0, const double* density, const double* energy,
                   double* kx, double* ky);
/* jacobi_copy_u + jacobi_iterate, TeaLeaf/c_kernels/sycl/jacobi.cpp:59-137
 * (as run_jacobi_iterate, kernel_interface.cpp:287-300); error = sum|du| */
int tl_jacobi_iterate(tl_context* ctx, int x, int y, int halo_depth,
                      double* u, const double* u0, double* r,
                      const double* kx, const double* ky, double* error);

/* --------------------------------------------------------- Chebyshev */
/* cheby_init, TeaLeaf/c_kernels/sycl/cheby.cpp:7-38 */
int tl_cheby_init(tl_context* ctx, int x, int y, int halo_depth, double theta,
                  double* p, double* r, const double* u, const double* u0,
                  double* w, const double* kx, const double* ky);
/* cheby_iterate + cheby_calc_u, TeaLeaf/c_kernels/sycl/cheby.cpp:41-110 */
int tl_cheby_iterate(tl_context* ctx, int x, int y, int halo_depth,
                     double alpha, double beta, double* p, double* r,
                     double* u, const double* u0, double* w,
                     const double* kx, const double* ky);

/* -------------------------------------------------------------- PPCG */
/* ppcg_init, TeaLeaf/c_kernels/sycl/ppcg.cpp:7-30 */
int tl_ppcg_init(tl_context* ctx, int x, int y, int halo_depth, double theta,
                 double* sd, const double* r);
/* ppcg_calc_ur + ppcg_calc_sd, TeaLeaf/c_kernels/sycl/ppcg.cpp:33-94 */
int tl_ppcg_inner_iteration(tl_context* ctx, int x, int y, int halo_depth,
                            double theta, double alpha, double beta,
                            double* sd, double* r, double* u,
                            const double* kx, const double* ky);

/* ---------------------------------------------------- failure detection
 * Self-test of the bounded grid-barrier wait used by every persistent
 * kernel: a single block waits for a second arrival that never comes, gives
 * up after budget_ms (at most 1000) and records TL_ERR_TIMEOUT, which is
 * returned in *status; the context stays usable. No counterpart in the
 * reference (its host waits are unbounded, TeaLeaf/c_kernels/sycl/
 * sycl_shared.hpp:77, a blocking host accessor). */
int tl_selftest_barrier_timeout(tl_context* ctx, int budget_ms, int* status);

#ifdef __cplusplus
}
#endif

#endif /* TEALEAF_GB300_H */
