// pt_host.cpp - host-side logic: constants.csv / seed.txt parsing, the C library's
// rand() sequence and the constants PandemicSim derives before any kernel runs.
#include "pt_host.h"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace pth {

GlibcRand::GlibcRand(unsigned int seed)
{
    if (seed == 0) seed = 1;
    int32_t word = (int32_t)seed;
    r_[0] = word;
    for (int i = 1; i < 31; i++) {
        // r[i] = 16807 * r[i-1] mod (2^31 - 1), Schrage's method as glibc writes it
        long hi = word / 127773;
        long lo = word % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        word = (int32_t)w;
        r_[i] = word;
    }
    f_ = 3;
    b_ = 0;
    for (int i = 0; i < 310; i++) (void)next();
}

int GlibcRand::next()
{
    uint32_t v = (uint32_t)r_[f_] + (uint32_t)r_[b_];
    r_[f_] = (int32_t)v;
    f_ = (f_ + 1) % 31;
    b_ = (b_ + 1) % 31;
    return (int)(v >> 1);
}

// Base tables the scaling starts from (PandemicSim.cu:359-372, :486-555).
static const int kBaseTypeCount[14] = {1000, 7000, 2400, 300, 100, 200, 100, 100, 300, 500, 0, 300, 400, 100};
static const float kShedding[6][10] = {
    {0.007339835f, 0.332600216f, 0.501192066f, 0.142183447f, 0.015675154f, 0.000967407f,
     4.055E-05f, 1.29105E-06f, 3.34836E-08f, 7.41011E-10f},
    {0.002533572f, 0.348252834f, 0.498210218f, 0.130145145f, 0.018421298f, 0.002158374f,
     0.000245489f, 2.88922E-05f, 3.61113E-06f, 4.83901E-07f},
    {0.05927385f, 0.314171688f, 0.411588802f, 0.187010054f, 0.026934715f, 0.001013098f,
     7.78449E-06f, 9.29441E-09f, 1.29796E-12f, 0},
    {0.04687299f, 0.248505983f, 0.30307952f, 0.211008627f, 0.11087006f, 0.049241932f,
     0.019562658f, 0.007179076f, 0.002482875f, 0.000820094f},
    {0.028667712f, 0.283445338f, 0.319240133f, 0.190123057f, 0.093989959f, 0.044155659f,
     0.020682822f, 0.009841839f, 0.00479234f, 0.002393665f},
    {0.087866042f, 0.223005225f, 0.258992749f, 0.208637267f, 0.127489076f, 0.061148649f,
     0.023406737f, 0.007216643f, 0.001802145f, 0.00036581f}};

// roundHalfUp_toInt, PandemicSim.cu:1662-1665
static int round_half_up(double d) { return (int)std::floor(d + 0.5); }

pt_status derive(const pt_params &p, Derived &out, GlibcRand &rng, const char **why)
{
    if (p.max_days < 0 || p.max_days > 255) {
        *why = "max_days must be in 0..255 (the reference's day counter is an 8-bit day_t)";
        return PT_ERR_ARG;
    }
    if (p.initial_pandemic < 0 || p.initial_seasonal < 0) {
        *why = "initial infected counts must be non-negative";
        return PT_ERR_ARG;
    }
    if (!(p.people_scaling > 0.f) || !(p.location_scaling > 0.f) || !std::isfinite(p.people_scaling) ||
        !std::isfinite(p.location_scaling)) {
        *why = "people_scaling_factor and location_scaling_factor must be positive";
        return PT_ERR_ARG;
    }
    // setup_loadSeed, PandemicSim.cu:2856-2861
    for (int i = 0; i < 4; i++) out.seeds[i] = rng.next();
    out.key0 = (uint64_t)(int64_t)out.seeds[0];
    out.key1 = (uint64_t)(int64_t)out.seeds[1];
    // setup_scaleSimulation, PandemicSim.cu:1127-1162
    double hh = (double)p.people_scaling * 1000000.0;
    if (hh > 300000000.0) {
        *why = "people_scaling_factor too large (households would exceed 3e8)";
        return PT_ERR_ARG;
    }
    out.households = round_half_up(hh);
    int sum = 0;
    for (int t = 0; t < 14; t++) {
        int original = round_half_up(kBaseTypeCount[t]);
        float scaled = p.location_scaling * (float)original;  // float product, as the reference
        if ((double)scaled > 100000000.0) {
            *why = "location_scaling_factor too large";
            return PT_ERR_ARG;
        }
        int n = round_half_up((double)scaled);
        if (n == 0 && original > 0) n = 1;
        out.type_count[t] = n;
        sum += n;
    }
    out.workplaces = sum;
    int acc = 0;
    for (int t = 0; t < 14; t++) {
        out.type_offset[t] = acc;
        acc += out.type_count[t];
    }
    if (out.households <= 0) {
        *why = "people_scaling_factor gives zero households";
        return PT_ERR_ARG;
    }
    // setup_calculateInfectionData, PandemicSim.cu:2828-2840
    std::memcpy(out.shedding, kShedding, sizeof(kShedding));
    for (int i = 3; i < 6; i++)
        for (int j = 0; j < 10; j++) out.shedding[i][j] *= p.asymp_factor;
    volatile float denom = (1.0f - p.asymp_factor) * p.percent_symptomatic;
    out.infectiousness[0] = p.r_pandemic / denom;
    out.infectiousness[1] = p.r_seasonal / denom;
    return PT_OK;
}

std::vector<int32_t> unique_numbers(GlibcRand &rng, int n, int max)
{
    std::vector<int32_t> a((size_t)n);
    for (int i = 0; i < n; i++) {
        bool dup;
        do {
            a[i] = rng.next() % max;
            dup = false;
            for (int j = 0; j < i; j++)
                if (a[j] == a[i]) {
                    dup = true;
                    break;
                }
        } while (dup);
    }
    return a;
}

}  // namespace pth

extern "C" {

// setup_loadParameters, PandemicSim.cu:286-310: skip the header line and the first
// column, then read the nine values positionally.
pt_status pt_params_from_csv(const char *path, pt_params *out)
{
    if (!path || !out) return PT_ERR_ARG;
    FILE *f = std::fopen(path, "r");
    if (!f) return PT_ERR_IO;
    char line[512];
    pt_params p;
    std::memset(&p, 0, sizeof(p));
    int ok = 1;
    if (!std::fgets(line, sizeof(line), f)) ok = 0;
    if (ok && std::fscanf(f, "%*[^,]%*c") < 0) ok = 0;
    if (ok && std::fscanf(f, "%d%*c", &p.max_days) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f%*c", &p.r_pandemic) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f%*c", &p.r_seasonal) != 1) ok = 0;
    if (ok && std::fscanf(f, "%d%*c", &p.initial_pandemic) != 1) ok = 0;
    if (ok && std::fscanf(f, "%d%*c", &p.initial_seasonal) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f%*c", &p.people_scaling) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f%*c", &p.location_scaling) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f%*c", &p.percent_symptomatic) != 1) ok = 0;
    if (ok && std::fscanf(f, "%f", &p.asymp_factor) != 1) ok = 0;
    std::fclose(f);
    if (!ok) return PT_ERR_PARSE;
    *out = p;
    return PT_OK;
}

// setup_loadSeed, PandemicSim.cu:2845-2854
pt_status pt_seed_from_file(const char *path, int *core_seed)
{
    if (!path || !core_seed) return PT_ERR_ARG;
    FILE *f = std::fopen(path, "r");
    if (!f) return PT_ERR_IO;
    int v = 0;
    int n = std::fscanf(f, "%d", &v);
    std::fclose(f);
    if (n != 1) return PT_ERR_PARSE;
    *core_seed = v;
    return PT_OK;
}

}  // extern "C"
