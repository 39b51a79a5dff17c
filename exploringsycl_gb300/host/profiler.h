/*
 * profiler.h -- name-keyed wall-clock profiler used around every backend call.
 *
 * Same interface as the reference's profiler (TeaLeaf/profiler.h:8-71): a
 * Profile holds named accumulators, and START_PROFILING / STOP_PROFILING
 * compile to timer calls only when ENABLE_PROFILING is defined. Not thread
 * safe: the driver is single-threaded.
 */
#pragma once
#include <time.h>

#define PROFILER_MAX_NAME 128
#define PROFILER_MAX_ENTRIES 2048

struct ProfileEntry {
  int calls;
  double time;
  char name[PROFILER_MAX_NAME];
};

struct Profile {
  struct timespec profiler_start;
  struct timespec profiler_end;
  int profiler_entry_count;
  struct ProfileEntry profiler_entries[PROFILER_MAX_ENTRIES];
};

void profiler_start_timer(struct Profile* profile);
void profiler_end_timer(struct Profile* profile, const char* entry_name);
void profiler_print_simple_profile(struct Profile* profile);
void profiler_print_full_profile(struct Profile* profile);
int profiler_get_profile_entry(struct Profile* profile, const char* entry_name);

#ifdef ENABLE_PROFILING
#define START_PROFILING(profile) profiler_start_timer(profile)
#define STOP_PROFILING(profile, name) profiler_end_timer(profile, name)
#define PRINT_PROFILING_RESULTS(profile) profiler_print_full_profile(profile)
#else
#define START_PROFILING(profile) ;
#define STOP_PROFILING(profile, name) ;
#define PRINT_PROFILING_RESULTS(profile) ;
#endif
