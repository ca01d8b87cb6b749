// pt_output.h - the reference's output files, written on the host from a run's
// results: shared by the drop-in executable (one simulation) and the batch driver.
#pragma once
#include <cstddef>
#include <string>
#include <utility>
#include <vector>

#include "pandemic_gb300.h"

namespace pto {

std::string join(const std::string &dir, const char *name);

// daily_writeInfectedStats (PandemicSim.cu:2771-2825): header, then per day the
// susceptible / infectious / symptomatic / asymptomatic / recovered counts of each
// strain from the 16 status bins (counts: rows x 16).
bool write_infected_stats(const std::string &path, const int *counts, int rows);

// final_countReproduction (PandemicSim.cu:2227-2304): generation sizes and Rn from
// the per-generation counts, with the reference's lower-bound arithmetic (the last
// row's next generation includes the never-infected).
bool write_rn(const std::string &path, const int *gen_p, const int *gen_s, int max_days, int persons);

// logging_closeOutputStreams (PandemicSim.cu:855-866).
bool write_infected_max(const std::string &path, float proportion, int day);

// logging_pollMemoryUsage_done (resource_logging.cu:83-122): one line appended, the
// header written when the file is new.
bool append_resource_log(const std::string &path, const char *sim_type, const char *device, float people_scale,
                         float location_scale, int seed, double milliseconds, size_t bytes_used);

// CudaProfiler (profiler.cu:13, :72-76): one row per timed function, written when it
// ends (children before their parent).
struct ProfileRow {
    int day, depth;
    const char *name;
    int problem_size;
    double inclusive_ms, exclusive_ms;
};
bool write_profile_log(const std::string &path, const std::vector<ProfileRow> &rows);

// The rows of one day from the eight stage times of pt_get_day_stage_ms, under the
// reference's function names (runToCompletion's call tree, PandemicSim.cu:877-961).
void day_profile_rows(std::vector<ProfileRow> &rows, int day, bool weekend, int persons, int infected,
                      const float ms[8]);

// output_mem.csv (resource_logging.cu:31-81): the initial free/total bytes, then one
// sample (day, free bytes) per row.
bool write_mem_log(const std::string &path, size_t free0, size_t total0,
                   const std::vector<std::pair<int, size_t>> &samples);

}  // namespace pto
