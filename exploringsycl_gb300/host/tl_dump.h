/*
 * tl_dump.h -- field dumps in VisIt's brick-of-values format.
 *
 * Same file pair as the reference's write_to_visit (TeaLeaf/shared.c:114-150,
 * never called there): <name><step>.bov describes a raw little-endian array
 * of doubles in <name><step>.dat. Backends call tl_dump_interior after a
 * field summary when TL_DUMP_DIR names a directory, for visual and
 * regression checks (byte-compare two backends' dumps).
 */
#pragma once
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

/* Writes the interior (x - 2hd) x (y - 2hd) of a host field of x*y doubles. */
static inline int tl_dump_interior(const char* dir, const char* name, int step, double time,
                                   int x, int y, int hd, const double* field) {
  const int nx = x - 2 * hd, ny = y - 2 * hd;
  std::vector<double> inner((size_t)nx * ny);
  for (int jj = 0; jj < ny; ++jj)
    for (int kk = 0; kk < nx; ++kk)
      inner[(size_t)jj * nx + kk] = field[(size_t)(jj + hd) * x + kk + hd];
  const std::string base = std::string(dir) + "/" + name + std::to_string(step);
  const std::string dat_name = std::string(name) + std::to_string(step) + ".dat";
  FILE* bov = fopen((base + ".bov").c_str(), "w");
  if (!bov) return 1;
  fprintf(bov, "TIME: %.4f\n", time);
  fprintf(bov, "DATA_FILE: %s\n", dat_name.c_str());
  fprintf(bov, "DATA_SIZE: %d %d 1\n", nx, ny);
  fprintf(bov, "DATA_FORMAT: DOUBLE\n");
  fprintf(bov, "VARIABLE: %s\n", name);
  fprintf(bov, "DATA_ENDIAN: LITTLE\n");
  fprintf(bov, "CENTERING: zone\n");
  fprintf(bov, "BRICK_ORIGIN: 0. 0. 0.\n");
  fprintf(bov, "BRICK_SIZE: %d %d 1\n", nx, ny);
  fclose(bov);
  FILE* dat = fopen((base + ".dat").c_str(), "wb");
  if (!dat) return 1;
  const size_t n = fwrite(inner.data(), sizeof(double), inner.size(), dat);
  fclose(dat);
  return n == inner.size() ? 0 : 1;
}
