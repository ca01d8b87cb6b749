// pt_cli.cpp - drop-in executable for the reference's main.cu (PandemicThrust/
// PandemicThrust/main.cu:12-31): reads constants.csv and seed.txt from the working
// directory and writes output_infected_stats.csv, output_rn.csv, infected_max.txt and
// profile_log.csv, appends to output_resource_log.csv, and prints the reference's
// console lines.
//
//   pt_sim [--per-day] [--quiet] [--dir DIR] [--no-profile] [--mem-log]
//
// --per-day steps one day per call with a host synchronisation each day (the
// reference's flow); the default runs the whole day loop on the device.
// profile_log.csv holds the device time of each stage of each day under the
// reference's function names (the reference writes it when built with SIM_PROFILING,
// its default); --no-profile skips it, and then the day loop runs as one CUDA graph.
// --mem-log writes output_mem.csv (the reference's POLL_MEMORY_USAGE log).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pandemic_gb300.h"
#include "pt_output.h"

static int die(const char *what, pt_status st, const pt_sim *s)
{
    std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, pt_last_error(s));
    return 1;
}

static double ms_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

int main(int argc, char **argv)
{
    bool per_day = false, quiet = false, profile = true, mem_log = false;
    std::string dir;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--per-day")) per_day = true;
        else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
        else if (!std::strcmp(argv[i], "--no-profile")) profile = false;
        else if (!std::strcmp(argv[i], "--mem-log")) mem_log = true;
        else if (!std::strcmp(argv[i], "--dir") && i + 1 < argc) dir = argv[++i];
        else {
            std::fprintf(stderr, "usage: %s [--per-day] [--quiet] [--dir DIR] [--no-profile] [--mem-log]\n", argv[0]);
            return 2;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    size_t free0 = 0, total0 = 0;
    cudaMemGetInfo(&free0, &total0);

    // PandemicSim::setup_loadSeed / setup_loadParameters (PandemicSim.cu:2843-2862, :268-323)
    int core_seed = 0;
    pt_status st = pt_seed_from_file(pto::join(dir, "seed.txt").c_str(), &core_seed);
    if (st == PT_ERR_IO) {
        std::perror("Error opening seed file");
        return 1;
    }
    if (st != PT_OK) return die("seed.txt", st, nullptr);
    pt_params p;
    st = pt_params_from_csv(pto::join(dir, "constants.csv").c_str(), &p);
    if (st == PT_ERR_IO) {
        std::perror("Error opening constants file");
        return 1;
    }
    if (st != PT_OK) return die("constants.csv", st, nullptr);

    pt_sim *sim = nullptr;
    st = pt_create(&p, core_seed, nullptr, &sim);
    if (st != PT_OK) return die("pt_create", st, nullptr);
    pt_info info;
    pt_get_info(sim, &info);
    if (!quiet) {
        std::printf("seeds:\t%d\t%d\t%d\t%d\n", info.seeds[0], info.seeds[1], info.seeds[2], info.seeds[3]);
        std::printf("max days: %d\nr_p: %f\nr_s: %f\ninitial_pandemic: %d\ninitial_seasonal: %d\nnumber_households: %d\n",
                    p.max_days, p.r_pandemic, p.r_seasonal, p.initial_pandemic, p.initial_seasonal, 1000000);
    }
    const std::string stats_path = pto::join(dir, "output_infected_stats.csv");
    {
        // the reference opens the statistics file before setup (PandemicSim.cu:259-263)
        FILE *f = std::fopen(stats_path.c_str(), "w");
        if (!f) {
            std::perror("output_infected_stats.csv");
            return 1;
        }
        std::fclose(f);
    }

    // PandemicSim::setupSim
    const auto ts = std::chrono::steady_clock::now();
    st = pt_setup(sim);
    if (st != PT_OK) return die("pt_setup", st, sim);
    const double setup_ms = ms_since(ts);
    pt_get_info(sim, &info);
    size_t free1 = 0, total1 = 0;
    cudaMemGetInfo(&free1, &total1);
    if (!quiet)
        std::printf("%d people, %d households, %d workplaces\n", info.number_people, info.number_households,
                    info.number_workplaces);

    // PandemicSim::runToCompletion (PandemicSim.cu:877-967)
    if (profile) pt_set_timing(sim, 1);
    const auto tr = std::chrono::steady_clock::now();
    std::vector<int> counts(256 * 16), infected(256);
    int rows = 0;
    if (per_day) {
        for (;;) {
            int c16[16], I = 0;
            st = pt_step_day(sim, c16, &I);
            if (st == PT_FINISHED) break;
            if (st < 0) return die("pt_step_day", st, sim);
            std::memcpy(&counts[rows * 16], c16, sizeof(c16));
            infected[rows] = I;
            rows++;
            if (st == PT_DONE) break;
        }
    } else {
        st = pt_run(sim, counts.data(), infected.data(), &rows);
        if (st != PT_OK) return die("pt_run", st, sim);
    }
    if (!pto::write_infected_stats(stats_path, counts.data(), rows)) {
        std::perror("output_infected_stats.csv");
        return 1;
    }
    if (!quiet)
        for (int day = 0; day < rows; day++)
            if (infected[day] > 0) std::printf("Day %3d:\tinfected: %5d\n", day + 1, infected[day]);

    // final_countReproduction (PandemicSim.cu:2227-2304)
    const auto tf = std::chrono::steady_clock::now();
    int gp[256], gs[256];
    st = pt_final_gen_counts(sim, gp, gs);
    if (st != PT_OK) return die("pt_final_gen_counts", st, sim);
    pto::write_rn(pto::join(dir, "output_rn.csv"), gp, gs, p.max_days, info.number_people);
    const double final_ms = ms_since(tf), run_ms = ms_since(tr);
    // logging_closeOutputStreams (PandemicSim.cu:855-866)
    pt_get_info(sim, &info);
    pto::write_infected_max(pto::join(dir, "infected_max.txt"), info.max_infected_proportion, info.max_day_of_peak);

    if (profile) {
        std::vector<pto::ProfileRow> prow;
        prow.push_back({-1, 0, "setupSim", info.number_people, setup_ms, setup_ms});
        for (int day = 0; day < rows; day++) {
            float ms[8];
            pt_get_day_stage_ms(sim, day, ms);
            pto::day_profile_rows(prow, day, (day % 7) >= 5, info.number_people, infected[day], ms);
        }
        prow.push_back({-1, 1, "final_countReproduction", p.max_days, final_ms, final_ms});
        prow.push_back({-1, 0, "runToCompletion", info.number_people, run_ms, 0.0});
        pto::write_profile_log(pto::join(dir, "profile_log.csv"), prow);
    }
    if (mem_log) {
        // the day loop allocates nothing: every day's sample equals the one after setup
        std::vector<std::pair<int, size_t>> samples;
        for (int day = 0; day < rows; day++) samples.push_back({day, free1});
        pto::write_mem_log(pto::join(dir, "output_mem.csv"), free0, total0, samples);
    }
    // logging_pollMemoryUsage_done (resource_logging.cu:83-122): runtime and device
    // memory held, appended to output_resource_log.csv
    pto::append_resource_log(pto::join(dir, "output_resource_log.csv"), "gb300_native", "GB300", p.people_scaling,
                             p.location_scaling, core_seed, ms_since(t0), info.device_bytes);
    (void)total1;
    pt_destroy(sim);
    return 0;
}
