/*
 * chunk.h -- one rectangular piece of the mesh and its field buffers.
 *
 * The member list is the backend interface of the reference's Chunk
 * (TeaLeaf/chunk.h:10-79): FieldBufferType and struct ChunkExtension come
 * from the backend's own chunk_extension.h, found on the include path.
 */
#pragma once
#include <math.h>

#include "chunk_extension.h"
#include "settings.h"

typedef struct Chunk {
  double dt_init;

  int* neighbours;

  double* left_send;
  double* left_recv;
  double* right_send;
  double* right_recv;
  double* top_send;
  double* top_recv;
  double* bottom_send;
  double* bottom_recv;

  int left;
  int right;
  int bottom;
  int top;

  int x;
  int y;

  FieldBufferType density0;
  FieldBufferType density;
  FieldBufferType energy0;
  FieldBufferType energy;

  FieldBufferType u;
  FieldBufferType u0;
  FieldBufferType p;
  FieldBufferType r;
  FieldBufferType mi;
  FieldBufferType w;
  FieldBufferType kx;
  FieldBufferType ky;
  FieldBufferType sd;

  FieldBufferType cell_x;
  FieldBufferType cell_y;
  FieldBufferType cell_dx;
  FieldBufferType cell_dy;

  FieldBufferType vertex_dx;
  FieldBufferType vertex_dy;
  FieldBufferType vertex_x;
  FieldBufferType vertex_y;

  FieldBufferType volume;
  FieldBufferType x_area;
  FieldBufferType y_area;

  double theta;
  double eigmin;
  double eigmax;

  double* cg_alphas;
  double* cg_betas;
  double* cheby_alphas;
  double* cheby_betas;

  struct ChunkExtension* ext;
} Chunk;

void initialise_chunk(Chunk* chunk, Settings* settings, int x, int y);
void finalise_chunk(Chunk* chunk);
