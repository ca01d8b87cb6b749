// pt_batch_cli.cpp - batch driver for the reference's scenario grids.
//
// PythonBatcher/write_gpu_constants.py writes one directory per experiment with its
// constants.csv, and lists the constants.csv paths in experiment_files.txt; the
// reference executable is then run once per experiment (and seed) inside each
// directory.  This driver runs all of them as one batch (pt_batch_*) and writes each
// run's files where the reference's run would have written them:
//
//   pt_batch [--list FILE] [--seeds S1,S2,...] [--quiet]
//
// FILE (default experiment_files.txt) holds one constants.csv path per line.
// Without --seeds each experiment runs once with the seed in the seed.txt beside its
// constants.csv, and its output_infected_stats.csv, output_rn.csv and
// infected_max.txt go to that directory; with --seeds it runs once per seed, into
// <experiment dir>/seed_<S>/.  Each output directory also gets a line in its
// output_resource_log.csv (the batch's wall time and device memory).
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "pandemic_gb300.h"
#include "pt_output.h"

static std::string dirname_of(const std::string &path)
{
    const size_t slash = path.find_last_of('/');
    return slash == std::string::npos ? std::string() : path.substr(0, slash);
}

static bool parse_seeds(const char *arg, std::vector<int> &out)
{
    std::string s(arg);
    size_t pos = 0;
    while (pos <= s.size()) {
        const size_t comma = s.find(',', pos);
        const std::string tok = s.substr(pos, comma == std::string::npos ? std::string::npos : comma - pos);
        if (tok.empty()) return false;
        char *end = nullptr;
        errno = 0;
        const long v = std::strtol(tok.c_str(), &end, 10);
        if (errno || *end || v < -2147483647l - 1 || v > 2147483647l) return false;
        out.push_back((int)v);
        if (comma == std::string::npos) break;
        pos = comma + 1;
    }
    return !out.empty();
}

int main(int argc, char **argv)
{
    std::string list = "experiment_files.txt";
    std::vector<int> seeds;
    bool quiet = false;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--list") && i + 1 < argc) list = argv[++i];
        else if (!std::strcmp(argv[i], "--seeds") && i + 1 < argc) {
            if (!parse_seeds(argv[++i], seeds)) {
                std::fprintf(stderr, "bad --seeds list\n");
                return 2;
            }
        } else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
        else {
            std::fprintf(stderr, "usage: %s [--list FILE] [--seeds S1,S2,...] [--quiet]\n", argv[0]);
            return 2;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::ifstream in(list);
    if (!in) {
        std::perror(("Error opening " + list).c_str());
        return 1;
    }
    std::vector<pt_params> params;
    std::vector<int> core_seeds;
    std::vector<std::string> out_dirs;
    std::string line;
    while (std::getline(in, line)) {
        while (!line.empty() && (line.back() == '\r' || line.back() == ' ')) line.pop_back();
        if (line.empty()) continue;
        pt_params p;
        pt_status st = pt_params_from_csv(line.c_str(), &p);
        if (st != PT_OK) {
            std::fprintf(stderr, "%s: cannot read constants (%d)\n", line.c_str(), (int)st);
            return 1;
        }
        const std::string dir = dirname_of(line);
        if (seeds.empty()) {
            int s = 0;
            st = pt_seed_from_file(pto::join(dir, "seed.txt").c_str(), &s);
            if (st != PT_OK) {
                std::fprintf(stderr, "%s: cannot read seed.txt (%d)\n", dir.c_str(), (int)st);
                return 1;
            }
            params.push_back(p);
            core_seeds.push_back(s);
            out_dirs.push_back(dir);
        } else {
            for (int s : seeds) {
                const std::string od = pto::join(dir, ("seed_" + std::to_string(s)).c_str());
                if (::mkdir(od.c_str(), 0755) != 0 && errno != EEXIST) {
                    std::perror(od.c_str());
                    return 1;
                }
                params.push_back(p);
                core_seeds.push_back(s);
                out_dirs.push_back(od);
            }
        }
    }
    const int K = (int)params.size();
    if (K == 0) {
        std::fprintf(stderr, "%s lists no experiments\n", list.c_str());
        return 1;
    }
    pt_batch *b = nullptr;
    pt_status st = pt_batch_create(params.data(), core_seeds.data(), K, nullptr, &b);
    if (st == PT_OK) st = pt_batch_setup(b);
    if (st == PT_OK) st = pt_batch_run(b);
    std::vector<int> gp((size_t)K * 256), gs((size_t)K * 256);
    if (st == PT_OK) st = pt_batch_final_gen_counts(b, gp.data(), gs.data());
    if (st != PT_OK) {
        std::fprintf(stderr, "batch failed (%d): %s\n", (int)st, pt_batch_last_error(b));
        pt_batch_destroy(b);
        return 1;
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int failed = 0;
    for (int k = 0; k < K; k++) {
        std::vector<int> counts(256 * 16), infected(256);
        int rows = 0;
        pt_batch_counts(b, k, counts.data(), infected.data(), &rows);
        pt_info info;
        pt_batch_get_info(b, k, &info);
        const std::string &od = out_dirs[k];
        bool ok = pto::write_infected_stats(pto::join(od, "output_infected_stats.csv"), counts.data(), rows);
        ok = pto::write_rn(pto::join(od, "output_rn.csv"), &gp[(size_t)k * 256], &gs[(size_t)k * 256],
                           params[k].max_days, info.number_people) && ok;
        ok = pto::write_infected_max(pto::join(od, "infected_max.txt"), info.max_infected_proportion,
                                     info.max_day_of_peak) && ok;
        ok = pto::append_resource_log(pto::join(od, "output_resource_log.csv"), "gb300_native_batch", "GB300",
                                      params[k].people_scaling, params[k].location_scaling, core_seeds[k], ms,
                                      info.device_bytes) && ok;
        if (!ok) {
            std::fprintf(stderr, "%s: cannot write the outputs\n", od.c_str());
            failed++;
        }
        if (!quiet)
            std::printf("%s\tseed %d\t%d people\t%d days\tpeak %f on day %d\n", od.empty() ? "." : od.c_str(),
                        core_seeds[k], info.number_people, rows, info.max_infected_proportion, info.max_day_of_peak);
    }
    pt_batch_destroy(b);
    return failed ? 1 : 0;
}
