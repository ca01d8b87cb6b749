/*
 * ref_harness.cpp - host harness that runs the reference's own simulation kernels on
 * the CPU (test infrastructure; see build_ref.py).
 *
 * The kernels and device functions come verbatim from PandemicSim.cu through the
 * generated ref_slices.inc.  This file supplies what the CUDA toolchain would:
 * qualifiers, a launch emulation (blockIdx/threadIdx/__syncthreads), atomics, and
 * host copies of the __constant__ tables.  It then restates the host methods of
 * class PandemicSim that orchestrate the kernels (setupSim, runToCompletion,
 * doWeekday_wholeDay, doWeekend_wholeDay, daily_countAndRecover,
 * daily_buildInfectedArray_global), replacing Thrust/CUB calls with sequential
 * standard algorithms of the same semantics.
 *
 * Kernels without block-level synchronisation run with one thread, so their
 * grid-stride loops visit items in ascending order: for kernel_doWeekday and
 * kernel_doWeekend that is the canonical infection order.  The counting kernel
 * uses __syncthreads() and shared memory, so it runs as 8 host threads with a
 * barrier, the smallest block for which it stores all 8 bins.
 */
#include <Random123/threefry.h>

#include <algorithm>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

/* ---- CUDA qualifier and runtime shims ---- */
#define __device__
#define __global__
#define __host__
#define __constant__
#define __shared__ static
struct ref_dim3 { unsigned x, y, z; };
static thread_local ref_dim3 threadIdx = {0, 0, 0};
static ref_dim3 blockIdx = {0, 0, 0};
static ref_dim3 blockDim = {1, 1, 1};
static ref_dim3 gridDim = {1, 1, 1};
static std::barrier<> *g_barrier = nullptr;
static inline void __syncthreads() { if (g_barrier) g_barrier->arrive_and_wait(); }
static inline unsigned int atomicCAS(unsigned int *a, unsigned int cmp, unsigned int val)
{
    unsigned int expected = cmp;
    __atomic_compare_exchange_n(a, &expected, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return expected;
}
static inline int atomicAdd(int *a, int v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
enum { cudaMemcpyHostToDevice = 1 };
#define cudaMemcpyToSymbolAsync(sym, src, n, ...) std::memcpy((void *)&(sym), (const void *)(src), (n))

namespace thrust {
template <class A, class R> struct unary_function { typedef A argument_type; typedef R result_type; };
template <class I, class O> O exclusive_scan(I first, I last, O out)
{
    typename std::iterator_traits<O>::value_type acc = 0;
    for (; first != last; ++first, ++out) {
        auto v = *first;
        *out = acc;
        acc += v;
    }
    return out;
}
}  // namespace thrust

/* ---- build-time switches of the shipped configuration (PandemicSim.h:9-66) ---- */
#define SIM_VALIDATION 0
#define SIM_PROFILING 0
#define CONSOLE_OUTPUT 0
#define COUNTING_GRID_THREADS 256
#ifndef __max
#define __max(a, b) (((a) > (b)) ? (a) : (b))
#endif
typedef int kval_t;                    /* indirect.h:41 */
typedef std::vector<int> h_vec;        /* indirect.h host_vector<int>, host side only */

#include "simParameters.h"
#include "host_functions.h"

struct ref_profiler_stub {
    void beginFunction(int, const char *) {}
    void endFunction(int, int) {}
};

/* The members of class PandemicSim (PandemicSim.h:68-281) that the extracted
 * parameter-loading methods touch. */
class PandemicSim {
public:
    randOffset_t rand_offset;
    int MAX_DAYS;
    day_t current_day;
    int core_seed;
    float people_scaling_factor, location_scaling_factor, asymp_factor;
    int number_people, number_households, number_workplaces;
    int INITIAL_INFECTED_PANDEMIC, INITIAL_INFECTED_SEASONAL;
    ref_profiler_stub profiler;
    void setup_loadParameters();
    void setup_loadSeed();
    void setup_scaleSimulation();
    void setup_calculateInfectionData();
    void setup_pushDeviceData();
};

#include "ref_slices.inc"

#include "pt_oracle.h"

/* ------------------------------------------------------------------ */
/* Harness state: the device vectors of PandemicSim.h:128-203          */
/* ------------------------------------------------------------------ */
namespace {
struct RefRun {
    PandemicSim sim;
    int N = 0, H = 0, L = 0, adults = 0, children = 0;
    std::vector<status_t> status_p, status_s;
    std::vector<day_t> day_p, day_s;
    std::vector<gen_t> gen_p, gen_s;
    std::vector<age_t> age;
    std::vector<locId_t> households, workplaces;
    std::vector<locOffset_t> hh_offsets, wp_offsets, errand_offsets;
    std::vector<personId_t> wp_people, infected, errand_people;
    std::vector<locId_t> errand_keys;
    int infected_count = 0;
    int errand_entries = 0, errand_buckets = 0;
    int max_days_run = 0;
    float max_prop = 0.f;
    int max_prop_day = 0;
    /* u8 mirrors of the u32 status arrays for the shared view struct */
    std::vector<uint8_t> sp8, ss8;
};
RefRun *g_run = nullptr;

void push_pointers(RefRun &r)
{
    /* setup_fetchVectorPtrs, PandemicSim.cu:2652-2673 */
    simArrayPtrStruct_t &p = device_arrayPtrStruct[0];
    p.people_status_pandemic = r.status_p.data();
    p.people_status_seasonal = r.status_s.data();
    p.people_days_pandemic = r.day_p.data();
    p.people_days_seasonal = r.day_s.data();
    p.people_gens_pandemic = r.gen_p.data();
    p.people_gens_seasonal = r.gen_s.data();
    p.people_ages = r.age.data();
    p.people_households = r.households.data();
    p.people_errands = r.errand_keys.data();
    p.household_locOffsets = r.hh_offsets.data();
    p.workplace_locOffsets = r.wp_offsets.data();
    p.errand_locOffsets = r.errand_offsets.data();
    p.workplace_people = r.wp_people.data();
}

/* Stable sort of (key, value) pairs + lower_bound offsets, as the reference's
 * CUB radix sort and thrust::lower_bound (PandemicSim.cu:1212-1248). */
void sort_and_offsets(std::vector<locId_t> &keys, std::vector<personId_t> &vals, int E, int B,
                      std::vector<locOffset_t> &offsets)
{
    std::vector<int> idx(E);
    for (int i = 0; i < E; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    std::vector<locId_t> k2(E);
    std::vector<personId_t> v2(E);
    for (int i = 0; i < E; i++) { k2[i] = keys[idx[i]]; v2[i] = vals[idx[i]]; }
    std::copy(k2.begin(), k2.end(), keys.begin());
    std::copy(v2.begin(), v2.end(), vals.begin());
    offsets.assign((size_t)B + 1, 0);
    for (int b = 0; b < B; b++)
        offsets[b] = (locOffset_t)(std::lower_bound(k2.begin(), k2.end(), b) - k2.begin());
    offsets[B] = E;
}

void launch_single(const std::function<void()> &k)
{
    blockDim = {1, 1, 1};
    gridDim = {1, 1, 1};
    blockIdx = {0, 0, 0};
    threadIdx = {0, 0, 0};
    k();
}

void launch_block(unsigned threads, const std::function<void()> &k)
{
    blockDim = {threads, 1, 1};
    gridDim = {1, 1, 1};
    blockIdx = {0, 0, 0};
    std::barrier<> bar((std::ptrdiff_t)threads);
    g_barrier = &bar;
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < threads; t++)
        ts.emplace_back([t, &k]() { threadIdx = {t, 0, 0}; k(); });
    for (auto &t : ts) t.join();
    g_barrier = nullptr;
    threadIdx = {0, 0, 0};
}
}  // namespace

extern "C" {

/* Threefry from the vendored header (threefry.h:726-735). */
void ptref_threefry2x64(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2])
{
    threefry2x64_ctr_t c = {{ctr[0], ctr[1]}};
    threefry2x64_key_t k = {{key[0], key[1]}};
    threefry2x64_ctr_t r = threefry2x64(c, k);
    out[0] = r.v[0];
    out[1] = r.v[1];
}

void ptref_threefry2x32(const uint32_t ctr[2], const uint32_t key[2], uint32_t out[2])
{
    threefry2x32_ctr_t c = {{ctr[0], ctr[1]}};
    threefry2x32_key_t k = {{key[0], key[1]}};
    threefry2x32_ctr_t r = threefry2x32(c, k);
    out[0] = r.v[0];
    out[1] = r.v[1];
}

/* The host C library's srand()/rand(). */
void ptref_libc_rand(unsigned int seed, int n, int *out)
{
    srand(seed);
    for (int i = 0; i < n; i++) out[i] = rand();
}

/* PandemicSim() constructor + setupSim() (PandemicSim.cu:98-208) reading
 * constants.csv and seed.txt from dir. */
int ptref_create(const char *dir)
{
    if (g_run) { delete g_run; g_run = nullptr; }
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) return -1;
    if (chdir(dir) != 0) return -1;
    RefRun *r = new RefRun();
    PandemicSim &s = r->sim;
    s.setup_loadParameters();
    s.setup_scaleSimulation();
    s.setup_calculateInfectionData();
    s.setup_pushDeviceData();
    if (chdir(cwd) != 0) { delete r; return -1; }
    g_run = r;
    return 0;
}

void ptref_destroy(void)
{
    delete g_run;
    g_run = nullptr;
}

int ptref_setup(void)
{
    if (!g_run) return -1;
    RefRun &r = *g_run;
    PandemicSim &s = r.sim;
    s.rand_offset = 0;
    s.current_day = 0;
    r.H = s.number_households;
    r.L = s.number_workplaces;
    /* setup_calcPopulationSize_thrust, PandemicSim.cu:3634-3651 */
    {
        hh_peopleCount_functor f;
        f.number_households = s.number_households;
        int p = 0;
        for (randOffset_t c = 0; c < (randOffset_t)(s.number_households / 4) + 1; c++) p += f(c);
        s.number_people = p;
    }
    const int N = s.number_people, H = r.H, L = r.L;
    r.N = N;
    /* setup_sizeGlobalArrays, PandemicSim.cu:1047-1107 */
    r.status_p.assign(N, 0); r.status_s.assign(N, 0);
    r.day_p.assign(N, 0); r.day_s.assign(N, 0);
    r.gen_p.assign(N, 0); r.gen_s.assign(N, 0);
    r.age.assign(N, 0); r.households.assign(N, 0);
    r.hh_offsets.assign((size_t)H + 1, 0);
    r.wp_offsets.assign((size_t)L + 1, 0);
    r.wp_people.assign(N, 0);
    r.infected.assign(N, 0);
    r.errand_keys.assign((size_t)3 * N, 0);
    r.errand_people.assign((size_t)3 * N, 0);
    r.errand_offsets.assign((size_t)10 * L + 1, 0);
    r.workplaces.assign(N, 0);
    host_simSizeStruct[0].number_people = N;
    host_simSizeStruct[0].number_households = H;
    host_simSizeStruct[0].number_workplaces = L;
    device_simSizeStruct[0] = host_simSizeStruct[0];
    push_pointers(r);

    /* setup_generateHouseholds, PandemicSim.cu:2552-2622 */
    std::vector<householdType_t> types((size_t)H + 1, 0);
    launch_single([&]() { kernel_householdTypeAssignment(types.data(), H, s.rand_offset); });
    s.rand_offset += H / 4;
    std::vector<int> ascan((size_t)H + 1), cscan((size_t)H + 1);
    {
        hh_adult_count_functor fa;
        hh_child_count_functor fc;
        int a = 0, c = 0;
        for (int h = 0; h <= H; h++) {
            ascan[h] = a; cscan[h] = c;
            a += fa(types[h]); c += fc(types[h]);
        }
    }
    r.adults = ascan[H];
    r.children = cscan[H];
    launch_single([&]() {
        kernel_generateHouseholds(types.data(), ascan.data(), cscan.data(), H, r.hh_offsets.data(),
                                  r.age.data(), r.households.data());
    });
    r.hh_offsets[H] = N;

    /* setup_assignWorkplaces, PandemicSim.cu:3812-3869 */
    host_randOffsetsStruct->workplace_randOffset = s.rand_offset;
    {
        assignWorkplaceFunctor f;
        f.functor_rand_offset = s.rand_offset;
        f.number_people = N;
        f.people_workplaces_arr = r.workplaces.data();
        f.people_ages_arr = r.age.data();
        for (int g = 0; g < N / 4 + 1; g++) f(g);
    }
    s.rand_offset += N / 4;
    {
        std::vector<locId_t> keys(r.workplaces);
        std::vector<personId_t> vals(N);
        for (int i = 0; i < N; i++) vals[i] = i;
        sort_and_offsets(keys, vals, N, L, r.wp_offsets);
        r.wp_people = vals;
    }
    push_pointers(r);

    /* setup_initializeStatusArrays, PandemicSim.cu:3654-3664 */
    std::fill(r.status_p.begin(), r.status_p.end(), STATUS_SUSCEPTIBLE);
    std::fill(r.status_s.begin(), r.status_s.end(), STATUS_SUSCEPTIBLE);
    std::fill(r.day_p.begin(), r.day_p.end(), DAY_NOT_INFECTED);
    std::fill(r.day_s.begin(), r.day_s.end(), DAY_NOT_INFECTED);
    std::fill(r.gen_p.begin(), r.gen_p.end(), GENERATION_NOT_INFECTED);
    std::fill(r.gen_s.begin(), r.gen_s.end(), GENERATION_NOT_INFECTED);

    /* setup_initialInfected, PandemicSim.cu:708-758 */
    int P = s.INITIAL_INFECTED_PANDEMIC, S = s.INITIAL_INFECTED_SEASONAL;
    h_vec init(P + S);
    n_unique_numbers(&init, P + S, N);
    for (int i = 0; i < P; i++) {
        r.status_p[init[i]] = STATUS_INFECTED; r.day_p[init[i]] = INITIAL_DAY; r.gen_p[init[i]] = INITIAL_GEN;
    }
    for (int i = P; i < P + S; i++) {
        r.status_s[init[i]] = STATUS_INFECTED; r.day_s[init[i]] = INITIAL_DAY; r.gen_s[init[i]] = INITIAL_GEN;
    }
    return 0;
}

/* One iteration of runToCompletion, PandemicSim.cu:882-954.  Returns 0 when the
 * day ran, 1 when the infected count was zero, 2 when max_days is reached. */
int ptref_step_day(int counts16[16], int *infected_count)
{
    if (!g_run) return -1;
    RefRun &r = *g_run;
    PandemicSim &s = r.sim;
    if ((int)s.current_day >= s.MAX_DAYS) return 2;
    const day_t current_day = s.current_day;
    /* daily_countAndRecover, PandemicSim.cu:2738-2768 */
    int counts[16] = {0};
    launch_block(8, [&]() {
        kernel_countInfectedStatusAndRecover(r.status_p.data(), r.status_s.data(), r.day_p.data(),
                                             r.day_s.data(), r.N, current_day, counts, counts + 8);
    });
    std::memcpy(counts16, counts, sizeof(counts));
    /* daily_buildInfectedArray_global, PandemicSim.cu:2207-2224 */
    int I = 0;
    for (int i = 0; i < r.N; i++)
        if (person_is_infected(r.status_p[i], r.status_s[i])) r.infected[I++] = i;
    r.infected_count = I;
    if (infected_count) *infected_count = I;
    if (I == 0) return 1;
    /* PandemicSim.cu:923-931 */
    float prop = (float)I / r.N;
    if (prop > r.max_prop) { r.max_prop = prop; r.max_prop_day = current_day; }
    std::vector<personId_t> vals((size_t)3 * r.N);
    if ((current_day % 7) < 5) {
        /* doWeekday_wholeDay, PandemicSim.cu:1186-1291 */
        host_randOffsetsStruct->errand_randOffset = s.rand_offset;
        device_randOffsetsStruct[0] = host_randOffsetsStruct[0];
        launch_single([&]() {
            kernel_assignWeekdayAfterschoolAndErrands(r.age.data(), r.N, r.L, r.errand_keys.data(),
                                                      vals.data(), s.rand_offset);
        });
        s.rand_offset += r.N / 2;
        int E = 2 * r.N, B = NUM_WEEKDAY_ERRAND_HOURS * r.L;
        std::vector<locId_t> keys(r.errand_keys.begin(), r.errand_keys.begin() + E);
        std::vector<personId_t> v(vals.begin(), vals.begin() + E);
        sort_and_offsets(keys, v, E, B, r.errand_offsets);
        std::copy(v.begin(), v.end(), r.errand_people.begin());
        r.errand_entries = E;
        r.errand_buckets = B;
        launch_single([&]() {
            kernel_doWeekday(I, r.infected.data(), r.errand_offsets.data(), r.errand_people.data(),
                             current_day, s.rand_offset);
        });
        s.rand_offset += 6 * I;
    } else {
        /* doWeekend_wholeDay, PandemicSim.cu:1294-1401 */
        host_randOffsetsStruct->errand_randOffset = s.rand_offset;
        device_randOffsetsStruct[0] = host_randOffsetsStruct[0];
        launch_single([&]() {
            kernel_assignWeekendErrands(vals.data(), r.errand_keys.data(), r.N, r.L, s.rand_offset);
        });
        s.rand_offset += 2 * r.N;
        int E = 3 * r.N, B = NUM_WEEKEND_ERRAND_HOURS * r.L;
        std::vector<locId_t> keys(r.errand_keys.begin(), r.errand_keys.begin() + E);
        std::vector<personId_t> v(vals.begin(), vals.begin() + E);
        sort_and_offsets(keys, v, E, B, r.errand_offsets);
        std::copy(v.begin(), v.end(), r.errand_people.begin());
        r.errand_entries = E;
        r.errand_buckets = B;
        launch_single([&]() {
            kernel_doWeekend(I, r.infected.data(), r.errand_offsets.data(), r.errand_people.data(),
                             current_day, s.rand_offset);
        });
        s.rand_offset += I * 6;
    }
    s.current_day++;
    return 0;
}

void ptref_get_view(ptor_view *v)
{
    std::memset(v, 0, sizeof(*v));
    if (!g_run) return;
    RefRun &r = *g_run;
    r.sp8.resize(r.N);
    r.ss8.resize(r.N);
    for (int i = 0; i < r.N; i++) { r.sp8[i] = (uint8_t)r.status_p[i]; r.ss8[i] = (uint8_t)r.status_s[i]; }
    v->N = r.N; v->H = r.H; v->L = r.L;
    v->adults = r.adults; v->children = r.children;
    v->infected_count = r.infected_count;
    v->current_day = r.sim.current_day;
    v->rand_offset = r.sim.rand_offset;
    v->workplace_rand_offset = host_randOffsetsStruct->workplace_randOffset;
    v->errand_rand_offset = host_randOffsetsStruct->errand_randOffset;
    for (int i = 0; i < 4; i++) v->seeds[i] = SEED_HOST[i];
    for (int t = 0; t < NUM_BUSINESS_TYPES; t++) {
        v->type_count[t] = WORKPLACE_TYPE_COUNT_HOST[t];
        v->type_offset[t] = WORKPLACE_TYPE_OFFSET_HOST[t];
    }
    v->infectiousness[0] = INFECTIOUSNESS_FACTOR_HOST[0];
    v->infectiousness[1] = INFECTIOUSNESS_FACTOR_HOST[1];
    std::memcpy(v->shedding, VIRAL_SHEDDING_PROFILES_HOST, sizeof(v->shedding));
    v->status_p = r.sp8.data(); v->status_s = r.ss8.data();
    v->day_p = r.day_p.data(); v->day_s = r.day_s.data();
    v->gen_p = r.gen_p.data(); v->gen_s = r.gen_s.data();
    v->age = r.age.data();
    v->household = r.households.data();
    v->household_offset = r.hh_offsets.data();
    v->workplace = r.workplaces.data();
    v->workplace_people = r.wp_people.data();
    v->workplace_offset = r.wp_offsets.data();
    v->infected = r.infected.data();
    v->errand_keys = r.errand_keys.data();
    v->errand_people = r.errand_people.data();
    v->errand_offset = r.errand_offsets.data();
    v->errand_entries = r.errand_entries;
    v->errand_buckets = r.errand_buckets;
}

/* Counts per generation (the sorted-generation lower bounds of
 * final_countReproduction, PandemicSim.cu:2236-2260, are prefix sums of these). */
void ptref_gen_counts(int gen_p[256], int gen_s[256])
{
    std::memset(gen_p, 0, 256 * sizeof(int));
    std::memset(gen_s, 0, 256 * sizeof(int));
    if (!g_run) return;
    for (int i = 0; i < g_run->N; i++) { gen_p[g_run->gen_p[i]]++; gen_s[g_run->gen_s[i]]++; }
}

/* host_functions.cpp wrappers: the reference's own CPU regeneration path. */
int ptref_host_recalc_workplace(int idx, int age)
{
    return host_recalcWorkplace(idx, (age_t)age);
}

int ptref_host_recalc_weekday(uint64_t errand_offset, int idx, int age, int *d1, int *d2)
{
    host_randOffsetsStruct->errand_randOffset = errand_offset;
    locId_t a, b;
    int prof = host_recalc_weekdayErrandDests_assignProfile(idx, (age_t)age, &a, &b);
    *d1 = a;
    *d2 = b;
    return prof;
}

void ptref_host_recalc_weekend(uint64_t errand_offset, int idx, int out[3])
{
    host_randOffsetsStruct->errand_randOffset = errand_offset;
    locId_t d[3];
    host_recalc_weekendErrandDests(idx, d);
    out[0] = d[0]; out[1] = d[1]; out[2] = d[2];
}

}  // extern "C"
