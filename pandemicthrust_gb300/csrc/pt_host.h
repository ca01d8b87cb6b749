// pt_host.h - host-side logic of the simulation that needs no GPU: input parsing,
// the C library's rand() sequence, scaling and infection constants.
#pragma once
#include <cstdint>
#include <vector>
#include "pandemic_gb300.h"

namespace pth {

// glibc srand()/rand(): additive feedback generator of degree 31, separation 3,
// seeded by a Park-Miller sequence and warmed up by 310 outputs (glibc random_r.c).
// The reference draws its Random123 key with it after srand(seed)
// (PandemicSim.cu:2856-2861) and its initial infected with rand() % N (:1648).
class GlibcRand {
public:
    explicit GlibcRand(unsigned int seed);
    int next();
private:
    int32_t r_[31];
    int f_, b_;
};

struct Derived {
    int seeds[4];
    uint64_t key0, key1;
    int households;
    int type_count[14];
    int type_offset[14];
    int workplaces;
    float shedding[6][10];
    float infectiousness[2];
};

// Validates parameters and computes what PandemicSim's constructor derives from
// them (setup_loadSeed, setup_scaleSimulation, setup_calculateInfectionData).
// Returns PT_OK or PT_ERR_ARG with a message.
pt_status derive(const pt_params &p, Derived &out, GlibcRand &rng, const char **why);

// n_unique_numbers (PandemicSim.cu:1642-1659): n distinct rand() % max values.
std::vector<int32_t> unique_numbers(GlibcRand &rng, int n, int max);

}  // namespace pth
