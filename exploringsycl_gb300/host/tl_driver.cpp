/*
 * tl_driver.cpp -- TeaLeaf host driver: deck parsing, mesh set-up, the
 * timestep loop and the solver loops that call the backend's run_* entry
 * points.
 *
 * This is a restatement, in this project's own code, of the behaviour of the
 * reference's unchanged C driver (TeaLeaf/main.c, diffuse.c, initialise.c,
 * parse_config.c, settings.c, shared.c, chunk.c, profiler.c, drivers/),
 * built without MPI (one rank). The reference driver cannot travel with this
 * repository, so this file plays its part wherever the reference sources are
 * absent; oracle/Makefile's `ref` target links the reference's own driver
 * against the CPU oracle to show that both drivers print identical results.
 *
 * Deliberate differences from the reference driver:
 *  - the tridiagonal eigenvalue problem of the Chebyshev/PPCG solvers is
 *    solved by Sturm-sequence bisection (own code) instead of the reference's
 *    QL iteration (drivers/eigenvalue_driver.c:71-122), so Chebyshev and
 *    PPCG agree with the reference to rounding, not bit for bit;
 *  - `-x` / `-y` are accepted and ignored (the reference parses the wrong
 *    argv entry after initialisation, main.c:76-85, so they never change the
 *    solve);
 *  - `-in`, `-out`, `-problems` name the deck, log and checking files
 *    (the reference always uses tea.in, tea.out, tea.problems in the
 *    working directory, which remain the defaults);
 *  - a missing tea.problems prints a warning and fails the check instead of
 *    dereferencing a null FILE* (field_summary_driver.c:58-70);
 *  - with more than one chunk (num_chunks_per_rank > 1) the halos between
 *    the chunks are exchanged: each chunk packs its faces through
 *    run_pack_or_unpack and the neighbouring chunk unpacks them, in the order
 *    of remote_halo_driver.c:11-129 (left/right, then bottom/top), where the
 *    reference built without MPI exchanges nothing (remote_halo_driver.c:14)
 *    and its chunks would solve uncoupled problems.
 */
#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cmath>
#include <string>
#include <vector>

#include "kernel_interface.h"

#define MAX_CHAR_LEN 256

/* ------------------------------------------------------------- profiler */
/* Same accounting as TeaLeaf/profiler.c:10-66: entries keyed by name,
 * accumulating calls and seconds from CLOCK_MONOTONIC. */

void profiler_start_timer(struct Profile* profile) {
  clock_gettime(CLOCK_MONOTONIC, &profile->profiler_start);
}

void profiler_end_timer(struct Profile* profile, const char* entry_name) {
  clock_gettime(CLOCK_MONOTONIC, &profile->profiler_end);
  int ii = 0;
  for (; ii < profile->profiler_entry_count; ++ii) {
    if (strmatch(profile->profiler_entries[ii].name, entry_name)) break;
  }
  if (ii >= PROFILER_MAX_ENTRIES) {
    printf("Attempted to profile too many entries, maximum is %d\n",
           PROFILER_MAX_ENTRIES);
    exit(1);
  }
  if (ii == profile->profiler_entry_count) {
    profile->profiler_entry_count++;
    snprintf(profile->profiler_entries[ii].name, PROFILER_MAX_NAME, "%s",
             entry_name);
    profile->profiler_entries[ii].time = 0.0;
    profile->profiler_entries[ii].calls = 0;
  }
  double elapsed =
      (double)(profile->profiler_end.tv_sec - profile->profiler_start.tv_sec) +
      (double)(profile->profiler_end.tv_nsec - profile->profiler_start.tv_nsec) *
          1.0E-9;
  profile->profiler_entries[ii].time += elapsed;
  profile->profiler_entries[ii].calls++;
}

void profiler_print_full_profile(struct Profile* profile) {
  printf("\n-------------------------------------------------------------\n");
  printf("\nProfiling Results:\n\n");
  printf("%-30s%8s%20s\n", "Kernel Name", "Calls", "Runtime (s)");
  double total = 0.0;
  for (int ii = 0; ii < profile->profiler_entry_count; ++ii) {
    total += profile->profiler_entries[ii].time;
    printf("%-30s%8d%20.03F\n", profile->profiler_entries[ii].name,
           profile->profiler_entries[ii].calls,
           profile->profiler_entries[ii].time);
  }
  printf("\nTotal elapsed time: %.03Fs, entries * are excluded.\n", total);
  printf("\n-------------------------------------------------------------\n\n");
}

void profiler_print_simple_profile(struct Profile* profile) {
  for (int ii = 0; ii < profile->profiler_entry_count; ++ii) {
    printf("%s: %.3lfs (%d calls)\n", profile->profiler_entries[ii].name,
           profile->profiler_entries[ii].time,
           profile->profiler_entries[ii].calls);
  }
}

int profiler_get_profile_entry(struct Profile* profile,
                               const char* entry_name) {
  for (int ii = 0; ii < profile->profiler_entry_count; ++ii) {
    if (strmatch(profile->profiler_entries[ii].name, entry_name)) return ii;
  }
  printf("Attempted to retrieve missing profile entry %s\n", entry_name);
  exit(1);
}

/* -------------------------------------------------------------- logging */
/* TeaLeaf/shared.c:5-111 */

void initialise_log(struct Settings* settings) {
  if (settings->rank != MASTER) return;
  printf("Opening %s as log file.\n", settings->tea_out_filename);
  settings->tea_out_fp = fopen(settings->tea_out_filename, "w");
  if (!settings->tea_out_fp) {
    die(__LINE__, __FILE__, "Could not open log %s\n",
        settings->tea_out_filename);
  }
}

void print_and_log(struct Settings* settings, const char* format, ...) {
  if (settings->rank != MASTER) return;
  va_list a1;
  va_start(a1, format);
  vprintf(format, a1);
  va_end(a1);
  if (!settings->tea_out_fp) {
    die(__LINE__, __FILE__,
        "Attempted to write to log before it was initialised\n");
  }
  va_list a2;
  va_start(a2, format);
  vfprintf(settings->tea_out_fp, format, a2);
  va_end(a2);
}

void print_to_log(struct Settings* settings, const char* format, ...) {
  if (settings->rank != MASTER) return;
  if (!settings->tea_out_fp) {
    die(__LINE__, __FILE__,
        "Attempted to write to log before it was initialised\n");
  }
  va_list a;
  va_start(a, format);
  vfprintf(settings->tea_out_fp, format, a);
  va_end(a);
}

void die(int lineNum, const char* file, const char* format, ...) {
  printf("\x1b[31m");
  printf("\nError at line %d in %s:", lineNum, file);
  printf("\x1b[0m \n");
  va_list a;
  va_start(a, format);
  vprintf(format, a);
  va_end(a);
  fflush(stdout);
  exit(1);
}

/* ------------------------------------------------------------- settings */
/* Defaults: TeaLeaf/settings.c:6-61 with the values of settings.h:11-45. */

static char* alloc_string(const char* init) {
  char* s = (char*)calloc(MAX_CHAR_LEN, 1);
  snprintf(s, MAX_CHAR_LEN, "%s", init);
  return s;
}

void set_default_settings(Settings* s) {
  memset(s, 0, sizeof(*s));
  s->test_problem_filename = alloc_string(DEF_TEST_PROBLEM_FILENAME);
  s->tea_in_filename = alloc_string(DEF_TEA_IN_FILENAME);
  s->tea_out_filename = alloc_string(DEF_TEA_OUT_FILENAME);
  s->tea_out_fp = NULL;
  s->grid_x_min = DEF_GRID_X_MIN;
  s->grid_y_min = DEF_GRID_Y_MIN;
  s->grid_x_max = DEF_GRID_X_MAX;
  s->grid_y_max = DEF_GRID_Y_MAX;
  s->grid_x_cells = DEF_GRID_X_CELLS;
  s->grid_y_cells = DEF_GRID_Y_CELLS;
  s->dt_init = DEF_DT_INIT;
  s->max_iters = DEF_MAX_ITERS;
  s->eps = DEF_EPS;
  s->end_time = DEF_END_TIME;
  s->end_step = DEF_END_STEP;
  s->summary_frequency = DEF_SUMMARY_FREQUENCY;
  s->solver = CG_SOLVER;
  s->coefficient = DEF_COEFFICIENT;
  s->error_switch = false;
  s->presteps = DEF_PRESTEPS;
  s->eps_lim = DEF_EPS_LIM;
  s->check_result = true;
  s->ppcg_inner_steps = DEF_PPCG_INNER_STEPS;
  s->preconditioner = false;
  s->num_states = 0;
  s->num_chunks = 1;
  s->num_chunks_per_rank = 1;
  s->num_ranks = 1;
  s->halo_depth = DEF_HALO_DEPTH;
  s->is_offload = false;
  s->kernel_language = C;
  s->kernel_profile = (struct Profile*)calloc(1, sizeof(struct Profile));
  s->application_profile = (struct Profile*)calloc(1, sizeof(struct Profile));
  s->wallclock_profile = (struct Profile*)calloc(1, sizeof(struct Profile));
  s->fields_to_exchange = (bool*)calloc(NUM_FIELDS, sizeof(bool));
  /* The reference leaves the name unset until a use_* key is read. */
  s->solver_name = alloc_string("CG");
}

void reset_fields_to_exchange(Settings* s) {
  for (int ii = 0; ii < NUM_FIELDS; ++ii) s->fields_to_exchange[ii] = false;
}

bool is_fields_to_exchange(Settings* s) {
  for (int ii = 0; ii < NUM_FIELDS; ++ii)
    if (s->fields_to_exchange[ii]) return true;
  return false;
}

/* ---------------------------------------------------------------- chunk */
/* TeaLeaf/chunk.c:4-45 */

void initialise_chunk(Chunk* chunk, Settings* settings, int x, int y) {
  chunk->x = x + settings->halo_depth * 2;
  chunk->y = y + settings->halo_depth * 2;
  chunk->dt_init = settings->dt_init;
  chunk->neighbours = (int*)malloc(sizeof(int) * NUM_FACES);
  size_t lr_len = (size_t)chunk->y * settings->halo_depth * NUM_FIELDS;
  chunk->left_send = (double*)malloc(sizeof(double) * lr_len);
  chunk->left_recv = (double*)malloc(sizeof(double) * lr_len);
  chunk->right_send = (double*)malloc(sizeof(double) * lr_len);
  chunk->right_recv = (double*)malloc(sizeof(double) * lr_len);
  size_t tb_len = (size_t)chunk->x * settings->halo_depth * NUM_FIELDS;
  chunk->top_send = (double*)malloc(sizeof(double) * tb_len);
  chunk->top_recv = (double*)malloc(sizeof(double) * tb_len);
  chunk->bottom_send = (double*)malloc(sizeof(double) * tb_len);
  chunk->bottom_recv = (double*)malloc(sizeof(double) * tb_len);
  chunk->ext = (ChunkExtension*)calloc(1, sizeof(ChunkExtension));
}

void finalise_chunk(Chunk* chunk) {
  free(chunk->neighbours);
  free(chunk->ext);
  free(chunk->left_send);
  free(chunk->left_recv);
  free(chunk->right_send);
  free(chunk->right_recv);
  free(chunk->top_send);
  free(chunk->top_recv);
  free(chunk->bottom_send);
  free(chunk->bottom_recv);
}

/* ----------------------------------------------------------- deck parser */
/* Key matching follows TeaLeaf/parse_config.c:288-366: a key matches when
 * the line, after leading blanks, starts with it; its value is the first
 * token that begins with a letter or digit after the first occurrence of
 * the key. (A leading '-' is therefore skipped, as in the reference.) */

static bool starts_with(const char* word, const char* line) {
  int matched = 0;
  int wlen = (int)strlen(word);
  int llen = (int)strlen(line);
  for (int ll = 0; ll < llen; ++ll) {
    if (!matched && isspace((unsigned char)line[ll])) continue;
    if (line[ll] != word[matched]) return false;
    if (++matched == wlen) return true;
  }
  return false;
}

static void read_value(const char* line, const char* word, char* value) {
  int matched = 0;
  int wlen = (int)strlen(word);
  int llen = (int)strlen(line);
  for (int ll = 0; ll < llen; ++ll) {
    if (matched == wlen) {
      if (isalpha((unsigned char)line[ll]) || isdigit((unsigned char)line[ll])) {
        sscanf(&line[ll], "%s", value);
        return;
      }
    } else {
      matched = (line[ll] == word[matched]) ? matched + 1 : 0;
    }
  }
  die(__LINE__, __FILE__, "Failed to find a value for key '%s'\n", word);
}

static bool starts_get_int(const char* key, const char* line, char* word,
                           int* value) {
  if (!starts_with(key, line)) return false;
  read_value(line, key, word);
  *value = atoi(word);
  return true;
}

static bool starts_get_double(const char* key, const char* line, char* word,
                              double* value) {
  if (!starts_with(key, line)) return false;
  read_value(line, key, word);
  *value = atof(word);
  return true;
}

static std::vector<std::string> read_lines(FILE* f) {
  std::vector<std::string> lines;
  char* line = NULL;
  size_t cap = 0;
  while (getline(&line, &cap, f) != -1) lines.push_back(line);
  free(line);
  return lines;
}

/* TeaLeaf/parse_config.c:77-192, in the same key order (so "epslim" is seen
 * before "eps", and x_cells/y_cells are taken only while still at their
 * default of 10). */
static void read_settings(const std::vector<std::string>& lines, Settings* s) {
  for (const std::string& ln : lines) {
    const char* line = ln.c_str();
    std::vector<char> wbuf(ln.size() + 2);
    char* word = wbuf.data();
    if (starts_get_double("initial_timestep", line, word, &s->dt_init)) continue;
    if (starts_get_double("end_time", line, word, &s->end_time)) continue;
    if (starts_get_int("end_step", line, word, &s->end_step)) continue;
    if (starts_get_double("xmin", line, word, &s->grid_x_min)) continue;
    if (starts_get_double("ymin", line, word, &s->grid_y_min)) continue;
    if (starts_get_double("xmax", line, word, &s->grid_x_max)) continue;
    if (starts_get_double("ymax", line, word, &s->grid_y_max)) continue;
    if (s->grid_x_cells == DEF_GRID_X_CELLS &&
        starts_get_int("x_cells", line, word, &s->grid_x_cells)) continue;
    if (s->grid_y_cells == DEF_GRID_Y_CELLS &&
        starts_get_int("y_cells", line, word, &s->grid_y_cells)) continue;
    if (starts_get_int("summary_frequency", line, word, &s->summary_frequency)) continue;
    if (starts_get_int("presteps", line, word, &s->presteps)) continue;
    if (starts_get_int("ppcg_inner_steps", line, word, &s->ppcg_inner_steps)) continue;
    if (starts_get_double("epslim", line, word, &s->eps_lim)) continue;
    if (starts_get_int("max_iters", line, word, &s->max_iters)) continue;
    if (starts_get_double("eps", line, word, &s->eps)) continue;
    if (starts_get_int("num_chunks_per_rank", line, word, &s->num_chunks_per_rank)) continue;
    if (starts_get_int("halo_depth", line, word, &s->halo_depth)) continue;
    if (starts_with("check_result", line)) { s->check_result = true; continue; }
    if (starts_with("errswitch", line)) { s->error_switch = true; continue; }
    if (starts_with("preconditioner_on", line)) { s->preconditioner = true; continue; }
    if (starts_with("use_fortran_kernels", line)) { s->kernel_language = FORTRAN; continue; }
    if (starts_with("use_c_kernels", line)) { s->kernel_language = C; continue; }
    if (starts_with("use_jacobi", line)) {
      s->solver = JACOBI_SOLVER; snprintf(s->solver_name, MAX_CHAR_LEN, "Jacobi"); continue;
    }
    if (starts_with("use_cg", line)) {
      s->solver = CG_SOLVER; snprintf(s->solver_name, MAX_CHAR_LEN, "CG"); continue;
    }
    if (starts_with("use_chebyshev", line)) {
      s->solver = CHEBY_SOLVER; snprintf(s->solver_name, MAX_CHAR_LEN, "Chebyshev"); continue;
    }
    if (starts_with("use_ppcg", line)) {
      s->solver = PPCG_SOLVER; snprintf(s->solver_name, MAX_CHAR_LEN, "PPCG"); continue;
    }
    if (starts_with("coefficient_density", line)) { s->coefficient = CONDUCTIVITY; continue; }
    if (starts_with("coefficient_inverse_density", line)) {
      s->coefficient = RECIP_CONDUCTIVITY; continue;
    }
  }
  s->dx = (s->grid_x_max - s->grid_x_min) / (double)s->grid_x_cells;
  s->dy = (s->grid_y_max - s->grid_y_min) / (double)s->grid_y_cells;
}

/* TeaLeaf/parse_config.c:195-286: state boundaries are pulled a hundredth of
 * a cell inwards so that a boundary on a cell edge cannot round into the
 * neighbouring cell. */
static int read_states(const std::vector<std::string>& lines, Settings* s,
                       State** states) {
  int num_states = 0;
  for (const std::string& ln : lines) {
    std::vector<char> wbuf(ln.size() + 2);
    int n = 0;
    if (starts_get_int("state", ln.c_str(), wbuf.data(), &n))
      num_states = MAX(num_states, n);
  }
  *states = (State*)calloc((size_t)MAX(num_states, 1), sizeof(State));
  for (const std::string& ln : lines) {
    const char* line = ln.c_str();
    std::vector<char> wbuf(ln.size() + 2);
    char* word = wbuf.data();
    int state_num = 0;
    if (!starts_get_int("state", line, word, &state_num)) continue;
    if (state_num < 1 || state_num > num_states) {
      die(__LINE__, __FILE__, "State number %d is out of range.\n", state_num);
    }
    State* st = &(*states)[state_num - 1];
    if (st->defined) {
      die(__LINE__, __FILE__, "State number %d defined twice.\n", state_num);
    }
    read_value(line, "density", word);
    st->density = atof(word);
    read_value(line, "energy", word);
    st->energy = atof(word);
    if (state_num > 1) {
      read_value(line, "xmin", word);
      st->x_min = atof(word) + s->dx / 100.0;
      read_value(line, "ymin", word);
      st->y_min = atof(word) + s->dy / 100.0;
      read_value(line, "xmax", word);
      st->x_max = atof(word) - s->dx / 100.0;
      read_value(line, "ymax", word);
      st->y_max = atof(word) - s->dy / 100.0;
      read_value(line, "geometry", word);
      if (strmatch(word, "rectangle")) {
        st->geometry = RECTANGULAR;
      } else if (strmatch(word, "circular")) {
        st->geometry = CIRCULAR;
        read_value(line, "radius", word);
        st->radius = atof(word);
      } else if (strmatch(word, "point")) {
        st->geometry = POINT;
      } else {
        die(__LINE__, __FILE__, "Unknown geometry '%s' for state %d.\n", word,
            state_num);
      }
    }
    st->defined = true;
  }
  return num_states;
}

/* TeaLeaf/parse_config.c:14-74 */
void read_config(Settings* settings, State** states) {
  FILE* tea_in = fopen(settings->tea_in_filename, "r");
  if (!tea_in) {
    die(__LINE__, __FILE__, "Could not open input file %s\n",
        settings->tea_in_filename);
  }
  std::vector<std::string> lines = read_lines(tea_in);
  fclose(tea_in);
  read_settings(lines, settings);
  settings->num_states = read_states(lines, settings, states);
  initialise_log(settings);

  print_to_log(settings, "Solution Parameters:\n");
  print_to_log(settings, "\tdt_init = %f\n", settings->dt_init);
  print_to_log(settings, "\tend_time = %f\n", settings->end_time);
  print_to_log(settings, "\tend_step = %d\n", settings->end_step);
  print_to_log(settings, "\tgrid_x_min = %f\n", settings->grid_x_min);
  print_to_log(settings, "\tgrid_y_min = %f\n", settings->grid_y_min);
  print_to_log(settings, "\tgrid_x_max = %f\n", settings->grid_x_max);
  print_to_log(settings, "\tgrid_y_max = %f\n", settings->grid_y_max);
  print_to_log(settings, "\tgrid_x_cells = %d\n", settings->grid_x_cells);
  print_to_log(settings, "\tgrid_y_cells = %d\n", settings->grid_y_cells);
  print_to_log(settings, "\tpresteps = %d\n", settings->presteps);
  print_to_log(settings, "\tppcg_inner_steps = %d\n", settings->ppcg_inner_steps);
  print_to_log(settings, "\teps_lim = %f\n", settings->eps_lim);
  print_to_log(settings, "\tmax_iters = %d\n", settings->max_iters);
  print_to_log(settings, "\teps = %f\n", settings->eps);
  print_to_log(settings, "\thalo_depth = %d\n", settings->halo_depth);
  print_to_log(settings, "\tcheck_result = %d\n", settings->check_result);
  print_to_log(settings, "\tcoefficient = %d\n", settings->coefficient);
  print_to_log(settings, "\tnum_chunks_per_rank = %d\n",
               settings->num_chunks_per_rank);
  print_to_log(settings, "\tsummary_frequency = %d\n",
               settings->summary_frequency);
  for (int ss = 0; ss < settings->num_states; ++ss) {
    print_to_log(settings, "\t\nstate %d\n", ss);
    print_to_log(settings, "\tdensity = %.12E\n", (*states)[ss].density);
    print_to_log(settings, "\tenergy= %.12E\n", (*states)[ss].energy);
    if (ss > 0) {
      print_to_log(settings, "\tx_min = %.12E\n", (*states)[ss].x_min);
      print_to_log(settings, "\ty_min = %.12E\n", (*states)[ss].y_min);
      print_to_log(settings, "\tx_max = %.12E\n", (*states)[ss].x_max);
      print_to_log(settings, "\ty_max = %.12E\n", (*states)[ss].y_max);
      print_to_log(settings, "\tradius = %.12E\n", (*states)[ss].radius);
      print_to_log(settings, "\tgeometry = %d\n", (*states)[ss].geometry);
    }
  }
}

/* --------------------------------------------------------------- drivers */

/* TeaLeaf/drivers/remote_halo_driver.c:132-184: packs (or unpacks) every
 * field marked for exchange into consecutive depth x offset slices of
 * `buffer`; returns the length used. */
static int invoke_pack_or_unpack(Chunk* chunk, Settings* settings, int face, int depth,
                                 int offset, bool pack, double* buffer) {
  int buffer_len = 0;
  for (int ii = 0; ii < NUM_FIELDS; ++ii) {
    if (!settings->fields_to_exchange[ii]) continue;
    FieldBufferType field;
    switch (ii) {
      case FIELD_DENSITY: field = chunk->density; break;
      case FIELD_ENERGY0: field = chunk->energy0; break;
      case FIELD_ENERGY1: field = chunk->energy; break;
      case FIELD_U: field = chunk->u; break;
      case FIELD_P: field = chunk->p; break;
      case FIELD_SD: field = chunk->sd; break;
      default: die(__LINE__, __FILE__, "Incorrect field provided: %d.\n", ii + 1);
    }
    double* offset_buffer = buffer + buffer_len;
    buffer_len += depth * offset;
    if (settings->kernel_language == C) {
      run_pack_or_unpack(chunk, settings, depth, face, pack, field, offset_buffer);
    }
  }
  return buffer_len;
}

/* The exchange of TeaLeaf/drivers/remote_halo_driver.c:11-129 between the
 * chunks of this rank (one rank: every neighbour is a local chunk, index =
 * chunk number). A chunk packs each face that has a neighbour into its send
 * buffer; the neighbour's receive buffer on the opposite face gets a copy,
 * which stands for the message; then every chunk unpacks. Left/right
 * first, then bottom/top, whose rows include the halo columns just filled. */
static void exchange_between_chunks(Chunk* chunks, Settings* settings, int depth) {
  const int n = settings->num_chunks_per_rank;
  if (n < 2) return;
  const int first = settings->rank * n;
  struct Pair { int face, opposite; };
  const Pair passes[2][2] = {{{CHUNK_LEFT, CHUNK_RIGHT}, {CHUNK_RIGHT, CHUNK_LEFT}},
                             {{CHUNK_BOTTOM, CHUNK_TOP}, {CHUNK_TOP, CHUNK_BOTTOM}}};
  auto send_buffer = [](Chunk* c, int face) {
    return face == CHUNK_LEFT ? c->left_send : face == CHUNK_RIGHT ? c->right_send
           : face == CHUNK_BOTTOM ? c->bottom_send : c->top_send;
  };
  auto recv_buffer = [](Chunk* c, int face) {
    return face == CHUNK_LEFT ? c->left_recv : face == CHUNK_RIGHT ? c->right_recv
           : face == CHUNK_BOTTOM ? c->bottom_recv : c->top_recv;
  };
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int> lens((size_t)n * 2, 0);
    for (int cc = 0; cc < n; ++cc) {
      for (int s = 0; s < 2; ++s) {
        const int face = passes[pass][s].face;
        if (chunks[cc].neighbours[face] == EXTERNAL_FACE) continue;
        const int offset = pass == 0 ? chunks[cc].y : chunks[cc].x;
        lens[(size_t)cc * 2 + s] = invoke_pack_or_unpack(&chunks[cc], settings, face, depth,
                                                         offset, true,
                                                         send_buffer(&chunks[cc], face));
      }
    }
    for (int cc = 0; cc < n; ++cc) {
      for (int s = 0; s < 2; ++s) {
        const int face = passes[pass][s].face;
        const int nb = chunks[cc].neighbours[face];
        if (nb == EXTERNAL_FACE) continue;
        const int local = nb - first;
        if (local < 0 || local >= n) {
          die(__LINE__, __FILE__, "Chunk %d's neighbour %d is not on this rank.\n",
              first + cc, nb);
        }
        /* the neighbour packed its opposite face, slot 1 - s of its pass */
        const int len = lens[(size_t)local * 2 + (1 - s)];
        if (len != lens[(size_t)cc * 2 + s]) {
          die(__LINE__, __FILE__, "Halo lengths of chunks %d and %d differ.\n", first + cc,
              nb);
        }
        memcpy(recv_buffer(&chunks[cc], face),
               send_buffer(&chunks[local], passes[pass][s].opposite),
               sizeof(double) * (size_t)len);
      }
    }
    for (int cc = 0; cc < n; ++cc) {
      for (int s = 0; s < 2; ++s) {
        const int face = passes[pass][s].face;
        if (chunks[cc].neighbours[face] == EXTERNAL_FACE) continue;
        const int offset = pass == 0 ? chunks[cc].y : chunks[cc].x;
        invoke_pack_or_unpack(&chunks[cc], settings, face, depth, offset, false,
                              recv_buffer(&chunks[cc], face));
      }
    }
  }
}

static void halo_update_driver(Chunk* chunks, Settings* settings, int depth) {
  /* TeaLeaf/drivers/halo_update_driver.c:6-25: the exchange between chunks
   * (remote_halo_driver.c), then the reflective halos of the external
   * faces. */
  if (!is_fields_to_exchange(settings)) return;
  exchange_between_chunks(chunks, settings, depth);
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_local_halos(&chunks[cc], settings, depth);
  }
}

/* A scalar that the backend overwrites rather than accumulates (r.r of
 * cg_calc_ur, the 2-norm, the Jacobi error and the field summary:
 * TeaLeaf/c_kernels/sycl/cg.cpp:253, solver_methods.cpp:116, jacobi.cpp:116,
 * field_summary.cpp:147-150) holds one chunk's value. With one chunk the
 * backend writes the driver's variable itself, as in the reference; with
 * several, the chunks' values are added in chunk order into `total`, which
 * starts from zero. `call(cc, out)` runs chunk cc's kernel into *out. */
template <class Call>
static void sum_chunk_scalars(Settings* settings, double* total, Call call) {
  if (settings->num_chunks_per_rank == 1) {
    call(0, total);
    return;
  }
  *total = 0.0;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    double v = 0.0;
    call(cc, &v);
    *total += v;
  }
}

/* TeaLeaf/drivers/cg_driver.c:31-66 */
static void cg_init_driver(Chunk* chunks, Settings* settings, double rx,
                           double ry, double* rro) {
  *rro = 0.0;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_cg_init(&chunks[cc], settings, rx, ry, rro);
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_U] = true;
  settings->fields_to_exchange[FIELD_P] = true;
  halo_update_driver(chunks, settings, 1);
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_copy_u(&chunks[cc], settings);
  }
}

/* TeaLeaf/drivers/cg_driver.c:69-124 */
static void cg_main_step_driver(Chunk* chunks, Settings* settings, int tt,
                                double* rro, double* error) {
  double pw = 0.0;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_cg_calc_w(&chunks[cc], settings, &pw);
  }
  double alpha = *rro / pw;
  double rrn = 0.0;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) chunks[cc].cg_alphas[tt] = alpha;
  if (settings->kernel_language == C) {
    sum_chunk_scalars(settings, &rrn, [&](int cc, double* out) {
      run_cg_calc_ur(&chunks[cc], settings, alpha, out);
    });
  }
  double beta = rrn / *rro;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    chunks[cc].cg_betas[tt] = beta;
    if (settings->kernel_language == C) run_cg_calc_p(&chunks[cc], settings, beta);
  }
  *error = rrn;
  *rro = rrn;
}

/* TeaLeaf/drivers/cg_driver.c:7-28: stop when sqrt(|rrn|) < eps. */
static void cg_driver(Chunk* chunks, Settings* settings, double rx, double ry,
                      double* error) {
  int tt;
  double rro = 0.0;
  cg_init_driver(chunks, settings, rx, ry, &rro);
  for (tt = 0; tt < settings->max_iters; ++tt) {
    cg_main_step_driver(chunks, settings, tt, &rro, error);
    halo_update_driver(chunks, settings, 1);
    if (std::sqrt(std::fabs(*error)) < settings->eps) break;
  }
  print_and_log(settings, "CG: \t\t\t%d iterations\n", tt);
}

/* Extreme eigenvalues of the symmetric tridiagonal matrix (d, e), where
 * e[i] couples rows i-1 and i (e[0] unused), by bisection on the Sturm
 * sequence count of eigenvalues below a shift (own implementation of the
 * classical method; see Golub & Van Loan, "Matrix Computations", 8.4). */
static int sturm_count_below(const double* d, const double* e, int n,
                             double lambda) {
  int count = 0;
  double q = 1.0;
  for (int i = 0; i < n; ++i) {
    double off = (i > 0) ? e[i] * e[i] : 0.0;
    q = d[i] - lambda - ((i > 0) ? off / q : 0.0);
    if (q == 0.0) q = -DBL_EPSILON * (fabs(d[i]) + fabs(lambda) + 1.0);
    if (q < 0.0) count++;
  }
  return count;
}

static double tridiag_eigenvalue(const double* d, const double* e, int n,
                                 int k /* 0-based rank from the bottom */) {
  double lo = d[0], hi = d[0];
  for (int i = 0; i < n; ++i) {
    double rad = (i > 0 ? fabs(e[i]) : 0.0) + (i + 1 < n ? fabs(e[i + 1]) : 0.0);
    lo = MIN(lo, d[i] - rad);
    hi = MAX(hi, d[i] + rad);
  }
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count_below(d, e, n, mid) > k) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

/* TeaLeaf/drivers/eigenvalue_driver.c:7-68: the Lanczos tridiagonal matrix
 * built from the CG alphas and betas, its extreme eigenvalues, then the
 * same 5 % widening. */
static void eigenvalue_driver_initialise(Chunk* chunks, Settings* settings,
                                         int num_cg_iters) {
  START_PROFILING(settings->kernel_profile);
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    std::vector<double> diag(num_cg_iters, 0.0), offdiag(num_cg_iters + 1, 0.0);
    for (int ii = 0; ii < num_cg_iters; ++ii) {
      diag[ii] = 1.0 / chunks[cc].cg_alphas[ii];
      if (ii > 0) diag[ii] += chunks[cc].cg_betas[ii - 1] / chunks[cc].cg_alphas[ii - 1];
      if (ii < num_cg_iters - 1)
        offdiag[ii + 1] = std::sqrt(chunks[cc].cg_betas[ii]) / chunks[cc].cg_alphas[ii];
    }
    double emin = tridiag_eigenvalue(diag.data(), offdiag.data(), num_cg_iters, 0);
    double emax = tridiag_eigenvalue(diag.data(), offdiag.data(), num_cg_iters,
                                     num_cg_iters - 1);
    chunks[cc].eigmin = emin;
    chunks[cc].eigmax = emax;
    if (chunks[cc].eigmin < 0.0 || chunks[cc].eigmax < 0.0) {
      die(__LINE__, __FILE__, "Calculated negative eigenvalues.\n");
    }
    chunks[cc].eigmin *= 0.95;
    chunks[cc].eigmax *= 1.05;
    print_and_log(settings, "Min. eigenvalue: \t%.12e\nMax. eigenvalue: \t%.12e\n",
                  chunks[cc].eigmin, chunks[cc].eigmax);
  }
  STOP_PROFILING(settings->kernel_profile, __func__);
}

/* TeaLeaf/drivers/cheby_driver.c:163-183 */
static void cheby_coef_driver(Chunk* chunks, Settings* settings, int max_iters) {
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    chunks[cc].theta = (chunks[cc].eigmax + chunks[cc].eigmin) / 2.0;
    double delta = (chunks[cc].eigmax - chunks[cc].eigmin) / 2.0;
    double sigma = chunks[cc].theta / delta;
    double rho_old = 1.0 / sigma;
    for (int ii = 0; ii < max_iters; ++ii) {
      double rho_new = 1.0 / (2.0 * sigma - rho_old);
      chunks[cc].cheby_alphas[ii] = rho_new * rho_old;
      chunks[cc].cheby_betas[ii] = 2.0 * rho_new / delta;
      rho_old = rho_new;
    }
  }
}

/* TeaLeaf/drivers/cheby_driver.c:80-107 */
static void cheby_init_driver(Chunk* chunks, Settings* settings,
                              int num_cg_iters, double* bb) {
  *bb = 0.0;
  eigenvalue_driver_initialise(chunks, settings, num_cg_iters);
  cheby_coef_driver(chunks, settings, settings->max_iters - num_cg_iters);
  if (settings->kernel_language == C) {
    sum_chunk_scalars(settings, bb, [&](int cc, double* out) {
      run_calculate_2norm(&chunks[cc], settings, chunks[cc].u0, out);
    });
    for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) run_cheby_init(&chunks[cc], settings);
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_U] = true;
  halo_update_driver(chunks, settings, 1);
}

/* TeaLeaf/drivers/cheby_driver.c:110-143 */
static void cheby_main_step_driver(Chunk* chunks, Settings* settings,
                                   int num_cheby_iters, bool is_calc_2norm,
                                   double* error) {
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C)
      run_cheby_iterate(&chunks[cc], settings, chunks[cc].cheby_alphas[num_cheby_iters],
                        chunks[cc].cheby_betas[num_cheby_iters]);
  }
  if (is_calc_2norm) {
    *error = 0.0;
    if (settings->kernel_language == C) {
      sum_chunk_scalars(settings, error, [&](int cc, double* out) {
        run_calculate_2norm(&chunks[cc], settings, chunks[cc].r, out);
      });
    }
  }
}

/* TeaLeaf/drivers/cheby_driver.c:146-160 */
static void cheby_calc_est_iterations(Chunk* chunks, double error, double bb,
                                      int* est_iterations) {
  double condition_number = chunks[0].eigmax / chunks[0].eigmin;
  double it_alpha = DBL_EPSILON * bb / (4.0 * error);
  double gamm = (std::sqrt(condition_number) - 1.0) /
                (std::sqrt(condition_number) + 1.0);
  *est_iterations = (int)roundf(logf((float)it_alpha) / (2.0f * logf((float)gamm)));
}

/* TeaLeaf/drivers/cheby_driver.c:10-77 */
static void cheby_driver(Chunk* chunks, Settings* settings, double rx,
                         double ry, double* error) {
  int tt;
  double rro = 0.0;
  int est_iterations = 0;
  int num_cheby_iters = 0;
  cg_init_driver(chunks, settings, rx, ry, &rro);
  for (tt = 0; tt < settings->max_iters; ++tt) {
    bool is_switch_to_cheby =
        (num_cheby_iters) ||
        (settings->error_switch
             ? (*error < settings->eps_lim) && (tt > CG_ITERS_FOR_EIGENVALUES)
             : (tt > settings->presteps) && (*error < ERROR_SWITCH_MAX));
    if (!is_switch_to_cheby) {
      cg_main_step_driver(chunks, settings, tt, &rro, error);
    } else {
      num_cheby_iters++;
      if (num_cheby_iters == 1) {
        double bb = 0.0;
        cheby_init_driver(chunks, settings, tt, &bb);
        cheby_main_step_driver(chunks, settings, num_cheby_iters, true, error);
        cheby_calc_est_iterations(chunks, *error, bb, &est_iterations);
      } else {
        bool is_calc_2norm = (num_cheby_iters >= est_iterations) && ((tt + 1) % 10 == 0);
        cheby_main_step_driver(chunks, settings, num_cheby_iters, is_calc_2norm, error);
      }
    }
    halo_update_driver(chunks, settings, 1);
    if (std::fabs(*error) < settings->eps) break;
  }
  print_and_log(settings, "CG: \t\t\t%d iterations\n", tt - num_cheby_iters + 1);
  print_and_log(settings, "Cheby: \t\t\t%d iterations (%d estimated)\n",
                num_cheby_iters, est_iterations);
}

/* TeaLeaf/drivers/ppcg_driver.c:66-84 */
static void ppcg_init_driver(Chunk* chunks, Settings* settings, double* rro) {
  (void)rro;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_calculate_residual(&chunks[cc], settings);
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_P] = true;
  halo_update_driver(chunks, settings, 1);
}

/* TeaLeaf/drivers/ppcg_driver.c:151-189 */
static void ppcg_inner_iterations(Chunk* chunks, Settings* settings) {
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_ppcg_init(&chunks[cc], settings);
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_SD] = true;
  for (int pp = 0; pp < settings->ppcg_inner_steps; ++pp) {
    halo_update_driver(chunks, settings, 1);
    for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
      if (settings->kernel_language == C)
        run_ppcg_inner_iteration(&chunks[cc], settings, chunks[cc].cheby_alphas[pp],
                                 chunks[cc].cheby_betas[pp]);
    }
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_P] = true;
}

/* TeaLeaf/drivers/ppcg_driver.c:87-149 */
static void ppcg_main_step_driver(Chunk* chunks, Settings* settings,
                                  double* rro, double* error) {
  double pw = 0.0;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_cg_calc_w(&chunks[cc], settings, &pw);
  }
  double alpha = *rro / pw;
  double rrn = 0.0;
  if (settings->kernel_language == C) {
    sum_chunk_scalars(settings, &rrn, [&](int cc, double* out) {
      run_cg_calc_ur(&chunks[cc], settings, alpha, out);
    });
  }
  ppcg_inner_iterations(chunks, settings);
  rrn = 0.0;
  if (settings->kernel_language == C) {
    sum_chunk_scalars(settings, &rrn, [&](int cc, double* out) {
      run_calculate_2norm(&chunks[cc], settings, chunks[cc].r, out);
    });
  }
  double beta = rrn / *rro;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_cg_calc_p(&chunks[cc], settings, beta);
  }
  *error = rrn;
  *rro = rrn;
}

/* TeaLeaf/drivers/ppcg_driver.c:10-63 */
static void ppcg_driver(Chunk* chunks, Settings* settings, double rx, double ry,
                        double* error) {
  int tt;
  double rro = 0.0;
  int num_ppcg_iters = 0;
  cg_init_driver(chunks, settings, rx, ry, &rro);
  for (tt = 0; tt < settings->max_iters; ++tt) {
    bool is_switch_to_ppcg =
        (num_ppcg_iters) ||
        (settings->error_switch
             ? (*error < settings->eps_lim) && (tt > CG_ITERS_FOR_EIGENVALUES)
             : (tt > settings->presteps) && (*error < ERROR_SWITCH_MAX));
    if (!is_switch_to_ppcg) {
      cg_main_step_driver(chunks, settings, tt, &rro, error);
    } else {
      num_ppcg_iters++;
      if (num_ppcg_iters == 1) {
        eigenvalue_driver_initialise(chunks, settings, tt);
        cheby_coef_driver(chunks, settings, settings->ppcg_inner_steps);
        ppcg_init_driver(chunks, settings, &rro);
      }
      ppcg_main_step_driver(chunks, settings, &rro, error);
    }
    halo_update_driver(chunks, settings, 1);
    if (std::fabs(*error) < settings->eps) break;
  }
  print_and_log(settings, "CG: \t\t\t%d iterations\n", tt - num_ppcg_iters + 1);
  print_and_log(settings, "PPCG: \t\t\t%d iterations (%d inner iterations per)\n",
                num_ppcg_iters, settings->ppcg_inner_steps);
}

/* TeaLeaf/drivers/jacobi_driver.c:7-84 */
static void jacobi_driver(Chunk* chunks, Settings* settings, double rx,
                          double ry, double* error) {
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) {
      run_jacobi_init(&chunks[cc], settings, rx, ry);
      run_copy_u(&chunks[cc], settings);
    }
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_U] = true;
  int tt;
  for (tt = 0; tt < settings->max_iters; ++tt) {
    if (settings->kernel_language == C) {
      sum_chunk_scalars(settings, error, [&](int cc, double* out) {
        run_jacobi_iterate(&chunks[cc], settings, out);
      });
    }
    if (tt % 50 == 0) {
      halo_update_driver(chunks, settings, 1);
      if (settings->kernel_language == C) {
        for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc)
          run_calculate_residual(&chunks[cc], settings);
        sum_chunk_scalars(settings, error, [&](int cc, double* out) {
          run_calculate_2norm(&chunks[cc], settings, chunks[cc].r, out);
        });
      }
    }
    halo_update_driver(chunks, settings, 1);
    if (std::fabs(*error) < settings->eps) break;
  }
  print_and_log(settings, "Jacobi: \t\t%d iterations\n", tt);
}

/* TeaLeaf/drivers/solve_finished_driver.c:7-43. The residual norm is
 * computed and, as in the reference, not reported; the ENERGY1 flag is
 * added to whatever flags the solver left set. */
static void solve_finished_driver(Chunk* chunks, Settings* settings) {
  double exact_error = 0.0;
  if (settings->check_result) {
    if (settings->kernel_language == C) {
      for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc)
        run_calculate_residual(&chunks[cc], settings);
      sum_chunk_scalars(settings, &exact_error, [&](int cc, double* out) {
        run_calculate_2norm(&chunks[cc], settings, chunks[cc].r, out);
      });
    }
  }
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_finalise(&chunks[cc], settings);
  }
  settings->fields_to_exchange[FIELD_ENERGY1] = true;
  halo_update_driver(chunks, settings, 1);
}

/* TeaLeaf/drivers/field_summary_driver.c:56-91 */
static void get_checking_value(Settings* settings, double* checking_value) {
  FILE* f = fopen(settings->test_problem_filename, "r");
  if (!f) {
    print_and_log(settings, "\nWARNING: Could not open the test problem file.\n");
    *checking_value = 1.0;
    return;
  }
  char* line = NULL;
  size_t len = 0;
  while (getline(&line, &len, f) != -1) {
    int x = 0, y = 0, num_steps = 0;
    double value = 1.0;
    if (sscanf(line, "%d %d %d %lf", &x, &y, &num_steps, &value) == 4 &&
        x == settings->grid_x_cells && y == settings->grid_y_cells &&
        num_steps == settings->end_step) {
      *checking_value = value;
      free(line);
      fclose(f);
      return;
    }
  }
  free(line);
  *checking_value = 1.0;
  print_and_log(settings, "\nWARNING: Problem was not found in the test problems file.\n");
  fclose(f);
}

/* TeaLeaf/drivers/field_summary_driver.c:8-53: PASS when the final
 * temperature is within 0.001 % of the tabulated value. */
static void field_summary_driver(Chunk* chunks, Settings* settings,
                                 bool is_solve_finished) {
  double vol = 0.0, ie = 0.0, temp = 0.0, mass = 0.0;
  if (settings->kernel_language == C && settings->num_chunks_per_rank == 1) {
    run_field_summary(&chunks[0], settings, &vol, &mass, &ie, &temp);
  } else if (settings->kernel_language == C) {
    /* the sums are overwritten per chunk (see sum_chunk_scalars) */
    for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
      double v = 0.0, m = 0.0, e = 0.0, t = 0.0;
      run_field_summary(&chunks[cc], settings, &v, &m, &e, &t);
      vol += v;
      mass += m;
      ie += e;
      temp += t;
    }
  }
  if (settings->rank == MASTER && settings->check_result && is_solve_finished) {
    print_and_log(settings, "\nChecking results...\n");
    double checking_value = 1.0;
    get_checking_value(settings, &checking_value);
    print_and_log(settings, "Expected %.15e\n", checking_value);
    print_and_log(settings, "Actual   %.15e\n", temp);
    double qa_diff = std::fabs(100.0 * (temp / checking_value) - 100.0);
    if (qa_diff < 0.001) print_and_log(settings, "This run \033[32mPASSED\033[0m");
    else print_and_log(settings, "This run \033[31mFAILED\033[0m");
    print_and_log(settings, " (Difference is within %.8lf%%)\n", qa_diff);
  }
}

/* ------------------------------------------------------ application init */

/* TeaLeaf/initialise.c:34-134, for one rank. */
static void decompose_field(Settings* settings, Chunk* chunks) {
  settings->num_chunks = settings->num_ranks * settings->num_chunks_per_rank;
  int num_chunks = settings->num_chunks;
  double best_metric = DBL_MAX;
  double x_cells = (double)settings->grid_x_cells;
  double y_cells = (double)settings->grid_y_cells;
  int x_chunks = 0, y_chunks = 0;
  for (int xx = 1; xx <= num_chunks; ++xx) {
    if (num_chunks % xx) continue;
    int yy = num_chunks / xx;
    if (num_chunks % yy) continue;
    double perimeter = ((x_cells / xx) * (x_cells / xx) + (y_cells / yy) * (y_cells / yy)) * 2;
    double area = (x_cells / xx) * (y_cells / yy);
    double metric = perimeter / area;
    if (metric < best_metric) {
      x_chunks = xx;
      y_chunks = yy;
      best_metric = metric;
    }
  }
  if (!x_chunks || !y_chunks) {
    die(__LINE__, __FILE__, "Failed to decompose the field with given parameters.\n");
  }
  int dx = settings->grid_x_cells / x_chunks;
  int dy = settings->grid_y_cells / y_chunks;
  int mod_x = settings->grid_x_cells % x_chunks;
  int mod_y = settings->grid_y_cells % y_chunks;
  int add_x_prev = 0, add_y_prev = 0;
  for (int yy = 0; yy < y_chunks; ++yy) {
    int add_y = (yy < mod_y);
    for (int xx = 0; xx < x_chunks; ++xx) {
      int add_x = (xx < mod_x);
      for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
        int chunk = xx + yy * x_chunks;
        int rank = cc + settings->rank * settings->num_chunks_per_rank;
        if (rank != chunk) continue;
        initialise_chunk(&chunks[cc], settings, dx + add_x, dy + add_y);
        chunks[cc].left = xx * dx + add_x_prev;
        chunks[cc].right = chunks[cc].left + dx + add_x;
        chunks[cc].bottom = yy * dy + add_y_prev;
        chunks[cc].top = chunks[cc].bottom + dy + add_y;
        chunks[cc].neighbours[CHUNK_LEFT] = (xx == 0) ? EXTERNAL_FACE : chunk - 1;
        chunks[cc].neighbours[CHUNK_RIGHT] = (xx == x_chunks - 1) ? EXTERNAL_FACE : chunk + 1;
        chunks[cc].neighbours[CHUNK_BOTTOM] = (yy == 0) ? EXTERNAL_FACE : chunk - x_chunks;
        chunks[cc].neighbours[CHUNK_TOP] = (yy == y_chunks - 1) ? EXTERNAL_FACE : chunk + x_chunks;
      }
      add_x_prev += add_x;
    }
    add_x_prev = 0;
    add_y_prev += add_y;
  }
}

/* TeaLeaf/initialise.c:11-31 */
static void initialise_application(Chunk** chunks, Settings* settings) {
  State* states = NULL;
  read_config(settings, &states);
  if (settings->num_chunks_per_rank < 1) {
    die(__LINE__, __FILE__, "num_chunks_per_rank=%d: at least one chunk is needed.\n",
        settings->num_chunks_per_rank);
  }
  if (settings->num_states < 1 || !states[0].defined) {
    die(__LINE__, __FILE__, "The deck defines no background state 1.\n");
  }
  *chunks = (Chunk*)calloc((size_t)settings->num_chunks_per_rank, sizeof(Chunk));
  decompose_field(settings, *chunks);
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_kernel_initialise(&(*chunks)[cc], settings);
  }
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_set_chunk_data(&(*chunks)[cc], settings);
  }
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_set_chunk_state(&(*chunks)[cc], settings, states);
  }
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_DENSITY] = true;
  settings->fields_to_exchange[FIELD_ENERGY0] = true;
  settings->fields_to_exchange[FIELD_ENERGY1] = true;
  halo_update_driver(*chunks, settings, 2);
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_store_energy(&(*chunks)[cc], settings);
  }
  free(states);
}

/* ------------------------------------------------------- timestep loop */

/* TeaLeaf/diffuse.c:23-78 */
static void solve(Chunk* chunks, Settings* settings, int tt,
                  double* wallclock_prev) {
  print_and_log(settings, "\nTimestep %d\n", tt + 1);
  profiler_start_timer(settings->wallclock_profile);
  double dt = settings->dt_init;
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (chunks[cc].dt_init < dt) dt = chunks[cc].dt_init;
  }
  double rx = dt / (settings->dx * settings->dx);
  double ry = dt / (settings->dy * settings->dy);
  reset_fields_to_exchange(settings);
  settings->fields_to_exchange[FIELD_ENERGY1] = true;
  settings->fields_to_exchange[FIELD_DENSITY] = true;
  halo_update_driver(chunks, settings, 2);
  double error = 1e+10;
  switch (settings->solver) {
    case JACOBI_SOLVER: jacobi_driver(chunks, settings, rx, ry, &error); break;
    case CG_SOLVER: cg_driver(chunks, settings, rx, ry, &error); break;
    case CHEBY_SOLVER: cheby_driver(chunks, settings, rx, ry, &error); break;
    case PPCG_SOLVER: ppcg_driver(chunks, settings, rx, ry, &error); break;
  }
  solve_finished_driver(chunks, settings);
  if (tt % settings->summary_frequency == 0) field_summary_driver(chunks, settings, false);
  profiler_end_timer(settings->wallclock_profile, "Wallclock");
  double wallclock = settings->wallclock_profile->profiler_entries[0].time;
  print_and_log(settings, "Wallclock: \t\t%.3lfs\n", wallclock);
  print_and_log(settings, "Avg. time per cell: \t%.6e\n",
                (wallclock - *wallclock_prev) /
                    ((double)settings->grid_x_cells * settings->grid_y_cells));
  print_and_log(settings, "Error: \t\t\t%.6e\n", error);
}

/* TeaLeaf/diffuse.c:10-20 */
static void diffuse(Chunk* chunks, Settings* settings) {
  double wallclock_prev = 0.0;
  for (int tt = 0; tt < settings->end_step; ++tt) solve(chunks, settings, tt, &wallclock_prev);
  field_summary_driver(chunks, settings, true);
}

/* Options that name files must be known before the deck is read. */
static void settings_files(Settings* settings, int argc, char** argv) {
  for (int aa = 1; aa + 1 < argc; ++aa) {
    if (strmatch(argv[aa], "-in")) snprintf(settings->tea_in_filename, MAX_CHAR_LEN, "%s", argv[aa + 1]);
    if (strmatch(argv[aa], "-out")) snprintf(settings->tea_out_filename, MAX_CHAR_LEN, "%s", argv[aa + 1]);
    if (strmatch(argv[aa], "-problems"))
      snprintf(settings->test_problem_filename, MAX_CHAR_LEN, "%s", argv[aa + 1]);
  }
}

/* TeaLeaf/main.c:61-99 (applied after initialisation, as there). */
static void settings_overload(Settings* settings, int argc, char** argv) {
  for (int aa = 1; aa < argc; ++aa) {
    if (strmatch(argv[aa], "-solver") || strmatch(argv[aa], "--solver") ||
        strmatch(argv[aa], "-s")) {
      if (aa + 1 == argc) break;
      if (strmatch(argv[aa + 1], "cg")) settings->solver = CG_SOLVER;
      if (strmatch(argv[aa + 1], "cheby")) settings->solver = CHEBY_SOLVER;
      if (strmatch(argv[aa + 1], "ppcg")) settings->solver = PPCG_SOLVER;
      if (strmatch(argv[aa + 1], "jacobi")) settings->solver = JACOBI_SOLVER;
    } else if (strmatch(argv[aa], "-help") || strmatch(argv[aa], "--help") ||
               strmatch(argv[aa], "-h")) {
      print_and_log(settings, "tealeaf <options>\n");
      print_and_log(settings, "options:\n");
      print_and_log(settings, "\t-solver, --solver, -s:\n");
      print_and_log(settings, "\t\tCan be 'cg', 'cheby', 'ppcg', or 'jacobi'\n");
      print_and_log(settings, "\t-in <file>, -out <file>, -problems <file>:\n");
      print_and_log(settings, "\t\tdeck, log and checking-value files\n");
      exit(0);
    }
  }
}

/* TeaLeaf/main.c:9-59 */
extern "C" int tl_main(int argc, char** argv) {
  Settings* settings = (Settings*)malloc(sizeof(Settings));
  set_default_settings(settings);
  settings->rank = MASTER;
  settings->num_ranks = 1;
  settings_files(settings, argc, argv);
  Chunk* chunks = NULL;
  initialise_application(&chunks, settings);
  settings_overload(settings, argc, argv);
  diffuse(chunks, settings);
  if (settings->rank == MASTER) {
    PRINT_PROFILING_RESULTS(settings->kernel_profile);
  }
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) {
    if (settings->kernel_language == C) run_kernel_finalise(&chunks[cc], settings);
  }
  for (int cc = 0; cc < settings->num_chunks_per_rank; ++cc) finalise_chunk(&chunks[cc]);
  free(chunks);
  if (settings->tea_out_fp) fclose(settings->tea_out_fp);
  free(settings->kernel_profile);
  free(settings->application_profile);
  free(settings->wallclock_profile);
  free(settings->fields_to_exchange);
  free(settings->solver_name);
  free(settings->tea_in_filename);
  free(settings->tea_out_filename);
  free(settings->test_problem_filename);
  free(settings);
  fflush(stdout);
  return 0;
}
