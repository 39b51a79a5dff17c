/*
 * kernel_interface.h -- the 22 backend entry points the driver calls.
 *
 * This is the drop-in boundary: the same names, arguments and C++ linkage
 * as the reference's TeaLeaf/kernel_interface.h:13-71, so a backend written
 * for one driver links under the other. Scalars returned through pointers
 * must be valid when the call returns.
 */
#pragma once
#include "chunk.h"
#include "settings.h"

void run_set_chunk_data(Chunk* chunk, Settings* settings);
void run_set_chunk_state(Chunk* chunk, Settings* settings, State* states);
void run_kernel_initialise(Chunk* chunk, Settings* settings);
void run_kernel_finalise(Chunk* chunk, Settings* settings);

void run_local_halos(Chunk* chunk, Settings* settings, int depth);
void run_pack_or_unpack(Chunk* chunk, Settings* settings, int depth, int face,
                        bool pack, FieldBufferType field, double* buffer);
void run_store_energy(Chunk* chunk, Settings* settings);
void run_field_summary(Chunk* chunk, Settings* settings, double* vol,
                       double* mass, double* ie, double* temp);

void run_cg_init(Chunk* chunk, Settings* settings, double rx, double ry,
                 double* rro);
void run_cg_calc_w(Chunk* chunk, Settings* settings, double* pw);
void run_cg_calc_ur(Chunk* chunk, Settings* settings, double alpha,
                    double* rrn);
void run_cg_calc_p(Chunk* chunk, Settings* settings, double beta);

void run_cheby_init(Chunk* chunk, Settings* settings);
void run_cheby_iterate(Chunk* chunk, Settings* settings, double alpha,
                       double beta);

void run_jacobi_init(Chunk* chunk, Settings* settings, double rx, double ry);
void run_jacobi_iterate(Chunk* chunk, Settings* settings, double* error);

void run_ppcg_init(Chunk* chunk, Settings* settings);
void run_ppcg_inner_iteration(Chunk* chunk, Settings* settings, double alpha,
                              double beta);

void run_copy_u(Chunk* chunk, Settings* settings);
void run_calculate_residual(Chunk* chunk, Settings* settings);
void run_calculate_2norm(Chunk* chunk, Settings* settings,
                         FieldBufferType buffer, double* norm);
void run_finalise(Chunk* chunk, Settings* settings);
