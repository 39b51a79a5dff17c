/*
 * chunk_extension.h -- what the GB300 backend adds to TeaLeaf's Chunk.
 *
 * Found by the driver through the include path (the reference driver
 * includes it from chunk.h:7). FieldBufferType is a device pointer: the
 * host never dereferences fields. The extension holds the backend context
 * and the state of the run-ahead CG mode (see kernel_interface.cpp).
 */
#pragma once

typedef double* FieldBufferType;

struct tl_context;
struct tl_net;

typedef struct ChunkExtension {
  struct tl_context* ctx;
  double* comms_buffer;   /* unused: halo staging lives in the context */
  int fused_cg;           /* 1: run_cg_init runs the whole solve on the device */
  int ra_active;          /* run-ahead replay in progress */
  int ra_steps;           /* CG steps executed by the device solve */
  int ra_k;               /* next step the driver will ask for */
  double ra_rro0;         /* initial r.p of the device solve */
  double* ra_pw;          /* host: pw of each device step */
  double* ra_rrn;         /* host: rrn of each device step */
  int ra_cap;
  int replace_method;     /* -1, or a TL_METHOD_* that replaces the CG solve */
  double replace_rel_tol; /* its relative FP64 true-residual target */
  double replace_inner_tol;
  int replace_projection; /* tl_solve_params.projection (gb300_projection) */
  struct tl_net* net;     /* the learned preconditioner (mixed-learned) */
  int fp64_fused;         /* 1: fused multiply-add contract of the FP64 CG */
} ChunkExtension;
