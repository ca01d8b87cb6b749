// pt_output.cpp - the reference's output files (see pt_output.h).
#include "pt_output.h"

#include <cstdio>
#include <sys/stat.h>

namespace pto {

std::string join(const std::string &dir, const char *name) { return dir.empty() ? name : dir + "/" + name; }

bool write_infected_stats(const std::string &path, const int *counts, int rows)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "day,pandemic_susceptible,pandemic_infectious,pandemic_symptomatic,pandemic_asymptomatic,"
                    "pandemic_recovered,seasonal_susceptible,seasonal_infectious,seasonal_symptomatic,"
                    "seasonal_asymptomatic,seasonal_recovered\n");
    for (int day = 0; day < rows; day++) {
        const int *c = &counts[day * 16];
        const int sym_p = c[2] + c[3] + c[4], asym_p = c[5] + c[6] + c[7];
        const int sym_s = c[10] + c[11] + c[12], asym_s = c[13] + c[14] + c[15];
        std::fprintf(f, "%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d\n", day, c[1], sym_p + asym_p, sym_p, asym_p, c[0], c[9],
                     sym_s + asym_s, sym_s, asym_s, c[8]);
    }
    return std::fclose(f) == 0;
}

bool write_rn(const std::string &path, const int *gen_p, const int *gen_s, int max_days, int persons)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "gen,gen_size_p,rn_p,gen_size_s,rn_s\n");
    const int M = max_days;
    // lower bounds of generation g over the sorted generations, with offsets[M] = N
    std::vector<long> lbp(M + 1), lbs(M + 1);
    long ap = 0, as = 0;
    for (int g = 0; g < M; g++) {
        lbp[g] = ap;
        lbs[g] = as;
        if (g < 256) {
            ap += gen_p[g];
            as += gen_s[g];
        }
    }
    lbp[M] = persons;
    lbs[M] = persons;
    for (int g = 0; g < M - 1; g++) {
        const int size_p = (int)(lbp[g + 1] - lbp[g]), next_p = (int)(lbp[g + 2] - lbp[g + 1]);
        const int size_s = (int)(lbs[g + 1] - lbs[g]), next_s = (int)(lbs[g + 2] - lbs[g + 1]);
        const float rn_p = (float)next_p / (float)size_p;
        const float rn_s = (float)next_s / (float)size_s;
        std::fprintf(f, "%d,%d,%f,%d,%f\n", g, size_p, rn_p, size_s, rn_s);
    }
    return std::fclose(f) == 0;
}

bool write_infected_max(const std::string &path, float proportion, int day)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "max_proportion,day\n%f,%d\n", proportion, day);
    return std::fclose(f) == 0;
}

bool append_resource_log(const std::string &path, const char *sim_type, const char *device, float people_scale,
                         float location_scale, int seed, double milliseconds, size_t bytes_used)
{
    struct stat sb;
    const bool exists = ::stat(path.c_str(), &sb) == 0;
    FILE *f = std::fopen(path.c_str(), exists ? "a" : "w");
    if (!f) return false;
    if (!exists)
        std::fprintf(f, "sim_type,sim_device,people_sim_scale,location_sim_scale,seed,runtime_milliseconds,"
                        "runtime_seconds,bytes_used,megabytes_used\n");
    std::fprintf(f, "%s,%s,%f,%f,%d,%f,%f,%zu,%zu\n", sim_type, device, people_scale, location_scale, seed,
                 milliseconds, milliseconds / 1000.0, bytes_used, bytes_used >> 20);
    return std::fclose(f) == 0;
}

bool write_profile_log(const std::string &path, const std::vector<ProfileRow> &rows)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "day,stack_depth,function_name,problem_size,inclusive_time_milliseconds,exclusive_time_milliseconds\n");
    for (const ProfileRow &r : rows)
        std::fprintf(f, "%d, %d, %s, %d, %f, %lf\n", r.day, r.depth, r.name, r.problem_size, r.inclusive_ms,
                     r.exclusive_ms);
    return std::fclose(f) == 0;
}

// Stage order of pt_get_day_stage_ms: sweep, infected list, schedule, digit bases,
// radix sort, bucket offsets, infection, apply.
void day_profile_rows(std::vector<ProfileRow> &rows, int day, bool weekend, int persons, int infected,
                      const float ms[8])
{
    rows.push_back({day, 1, "daily_countAndRecover", persons, ms[0], ms[0]});
    rows.push_back({day, 1, "daily_buildInfectedArray_global", infected, ms[1], ms[1]});
    if (infected == 0) return;  // the reference breaks before the day's contacts
    const double sched = ms[2], sort = ms[3] + ms[4], search = ms[5], kernel = ms[6] + ms[7];
    if (weekend) {
        rows.push_back({day, 2, "weekend_assignErrands", persons, sched, sched});
        rows.push_back({day, 2, "doWeekend_wholeDay_setup_sort", persons, sort, sort});
        rows.push_back({day, 2, "doWeekend_wholeDay_setup_locationSearch", persons, search, search});
        rows.push_back({day, 2, "doWeekend_wholeDay_kernel", infected, kernel, kernel});
        rows.push_back({day, 1, "doWeekend_wholeDay", persons, sched + sort + search + kernel, 0.0});
    } else {
        rows.push_back({day, 2, "doWeekday_wholeDay_generateSchedulesKernel", persons, sched, sched});
        rows.push_back({day, 2, "doWeekday_wholeDay_setup_sort", persons, sort, sort});
        rows.push_back({day, 2, "doWeekday_wholeDay_setup_locationSearch", persons, search, search});
        rows.push_back({day, 2, "doWeekday_wholeDay_kernel", infected, kernel, kernel});
        rows.push_back({day, 1, "doWeekday_wholeDay", persons, sched + sort + search + kernel, 0.0});
    }
}

bool write_mem_log(const std::string &path, size_t free0, size_t total0,
                   const std::vector<std::pair<int, size_t>> &samples)
{
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "day,freeBytes,bytesUsed,totalBytes,megabytesUsed\n");
    std::fprintf(f, "INITIAL,%zu,0,%zu,0\n", free0, total0);
    for (const auto &s : samples) {
        const size_t used = free0 > s.second ? free0 - s.second : 0;
        std::fprintf(f, "%d,%zu,%zu,%zu,%zu\n", s.first, s.second, used, total0, used >> 20);
    }
    return std::fclose(f) == 0;
}

}  // namespace pto
