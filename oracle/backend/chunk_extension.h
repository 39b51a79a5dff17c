/*
 * chunk_extension.h -- field storage of the CPU oracle backend (test
 * infrastructure): every field is a host array of doubles.
 */
#pragma once
typedef double* FieldBufferType;

typedef struct ChunkExtension {
  double* comms_buffer;
} ChunkExtension;
