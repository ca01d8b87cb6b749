// pt_cli.cpp - drop-in executable for the reference's main.cu (PandemicThrust/
// PandemicThrust/main.cu:12-31): reads constants.csv and seed.txt from the working
// directory and writes output_infected_stats.csv, output_rn.csv, infected_max.txt and
// appends to output_resource_log.csv, with the reference's console lines.
//
//   pt_sim [--per-day] [--quiet] [--dir DIR]
//
// --per-day steps one day per call with a host synchronisation each day (the
// reference's flow); the default runs the whole day loop on the device.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include <cuda_runtime.h>

#include "pandemic_gb300.h"

static int die(const char *what, pt_status st, const pt_sim *s)
{
    std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, pt_last_error(s));
    return 1;
}

static std::string join(const std::string &dir, const char *name) { return dir.empty() ? name : dir + "/" + name; }

int main(int argc, char **argv)
{
    bool per_day = false, quiet = false;
    std::string dir;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--per-day")) per_day = true;
        else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
        else if (!std::strcmp(argv[i], "--dir") && i + 1 < argc) dir = argv[++i];
        else {
            std::fprintf(stderr, "usage: %s [--per-day] [--quiet] [--dir DIR]\n", argv[0]);
            return 2;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    size_t free0 = 0, total0 = 0;
    cudaMemGetInfo(&free0, &total0);

    // PandemicSim::setup_loadSeed / setup_loadParameters (PandemicSim.cu:2843-2862, :268-323)
    int core_seed = 0;
    pt_status st = pt_seed_from_file(join(dir, "seed.txt").c_str(), &core_seed);
    if (st == PT_ERR_IO) {
        std::perror("Error opening seed file");
        return 1;
    }
    if (st != PT_OK) return die("seed.txt", st, nullptr);
    pt_params p;
    st = pt_params_from_csv(join(dir, "constants.csv").c_str(), &p);
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
    FILE *fstats = std::fopen(join(dir, "output_infected_stats.csv").c_str(), "w");
    if (!fstats) {
        std::perror("output_infected_stats.csv");
        return 1;
    }
    std::fprintf(fstats, "day,pandemic_susceptible,pandemic_infectious,pandemic_symptomatic,pandemic_asymptomatic,"
                         "pandemic_recovered,seasonal_susceptible,seasonal_infectious,seasonal_symptomatic,"
                         "seasonal_asymptomatic,seasonal_recovered\n");

    // PandemicSim::setupSim
    st = pt_setup(sim);
    if (st != PT_OK) return die("pt_setup", st, sim);
    pt_get_info(sim, &info);
    if (!quiet)
        std::printf("%d people, %d households, %d workplaces\n", info.number_people, info.number_households,
                    info.number_workplaces);

    // PandemicSim::runToCompletion (PandemicSim.cu:877-967)
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
    for (int day = 0; day < rows; day++) {
        const int *c = &counts[day * 16];
        int sym_p = c[2] + c[3] + c[4], asym_p = c[5] + c[6] + c[7];
        int sym_s = c[10] + c[11] + c[12], asym_s = c[13] + c[14] + c[15];
        // daily_writeInfectedStats, PandemicSim.cu:2806-2818
        std::fprintf(fstats, "%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d\n", day, c[1], sym_p + asym_p, sym_p, asym_p, c[0],
                     c[9], sym_s + asym_s, sym_s, asym_s, c[8]);
        if (!quiet && infected[day] > 0) std::printf("Day %3d:\tinfected: %5d\n", day + 1, infected[day]);
    }
    std::fclose(fstats);

    // final_countReproduction (PandemicSim.cu:2227-2304)
    int gp[256], gs[256];
    st = pt_final_gen_counts(sim, gp, gs);
    if (st != PT_OK) return die("pt_final_gen_counts", st, sim);
    FILE *frn = std::fopen(join(dir, "output_rn.csv").c_str(), "w");
    if (frn) {
        std::fprintf(frn, "gen,gen_size_p,rn_p,gen_size_s,rn_s\n");
        const int M = p.max_days, N = info.number_people;
        std::vector<long> lbp(M + 1), lbs(M + 1);
        long ap = 0, as = 0;
        for (int g = 0; g < M; g++) {
            lbp[g] = ap;
            lbs[g] = as;
            if (g < 256) {
                ap += gp[g];
                as += gs[g];
            }
        }
        lbp[M] = N;
        lbs[M] = N;
        for (int g = 0; g < M - 1; g++) {
            int size_p = (int)(lbp[g + 1] - lbp[g]), next_p = (int)(lbp[g + 2] - lbp[g + 1]);
            int size_s = (int)(lbs[g + 1] - lbs[g]), next_s = (int)(lbs[g + 2] - lbs[g + 1]);
            float rn_p = (float)next_p / (float)size_p;
            float rn_s = (float)next_s / (float)size_s;
            std::fprintf(frn, "%d,%d,%f,%d,%f\n", g, size_p, rn_p, size_s, rn_s);
        }
        std::fclose(frn);
    }
    // logging_closeOutputStreams (PandemicSim.cu:855-866)
    pt_get_info(sim, &info);
    FILE *fmax = std::fopen(join(dir, "infected_max.txt").c_str(), "w");
    if (fmax) {
        std::fprintf(fmax, "max_proportion,day\n%f,%d\n", info.max_infected_proportion, info.max_day_of_peak);
        std::fclose(fmax);
    }
    // logging_pollMemoryUsage_done (resource_logging.cu:83-122): runtime and device
    // memory held, appended to output_resource_log.csv
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    size_t used = info.device_bytes;
    std::string rl = join(dir, "output_resource_log.csv");
    struct stat sb;
    bool exists = ::stat(rl.c_str(), &sb) == 0;
    FILE *fres = std::fopen(rl.c_str(), exists ? "a" : "w");
    if (fres) {
        if (!exists)
            std::fprintf(fres, "sim_type,sim_device,people_sim_scale,location_sim_scale,seed,runtime_milliseconds,"
                               "runtime_seconds,bytes_used,megabytes_used\n");
        std::fprintf(fres, "%s,%s,%f,%f,%d,%f,%f,%zu,%zu\n", "gb300_native", "GB300", p.people_scaling,
                     p.location_scaling, core_seed, ms, ms / 1000.0, used, used >> 20);
        std::fclose(fres);
    }
    (void)free0;
    (void)total0;
    pt_destroy(sim);
    return 0;
}
