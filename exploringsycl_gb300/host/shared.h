/*
 * shared.h -- constants and logging shared by the driver and the backends.
 *
 * The numeric codes (faces, fields, coefficient kinds) are part of the
 * backend interface and keep the values the reference uses
 * (TeaLeaf/shared.h:31-55) so that a backend source compiles unchanged
 * against either driver.
 */
#pragma once
#include <stdarg.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cmath>

#include "profiler.h"

struct Settings;

void initialise_log(struct Settings* settings);
void print_to_log(struct Settings* settings, const char* format, ...);
void print_and_log(struct Settings* settings, const char* format, ...);
void die(int lineNum, const char* file, const char* format, ...);

#define MASTER 0

#define NUM_FACES 4
#define CHUNK_LEFT 0
#define CHUNK_RIGHT 1
#define CHUNK_BOTTOM 2
#define CHUNK_TOP 3
#define EXTERNAL_FACE -1

#define FIELD_DENSITY 0
#define FIELD_ENERGY0 1
#define FIELD_ENERGY1 2
#define FIELD_U 3
#define FIELD_P 4
#define FIELD_SD 5

#define CONDUCTIVITY 1
#define RECIP_CONDUCTIVITY 2

#define CG_ITERS_FOR_EIGENVALUES 20
#define ERROR_SWITCH_MAX 1.0

#define MIN(a, b) ((a < b) ? a : b)
#define MAX(a, b) ((a > b) ? a : b)
#define strmatch(a, b) (strcmp(a, b) == 0)
