// pt_sim.cpp - C ABI of the simulation: lifecycle, the PandemicSim host flow
// (setupSim / runToCompletion / doWeekday|doWeekend / final_countReproduction) and
// device-memory ownership, for one simulation (pt_sim) and for a batch of
// independent simulations (pt_batch).  Both are an Engine: K instances whose persons,
// households, locations and buckets share batch-wide arrays, each instance in its own
// range.  A pt_sim is an Engine with one instance.  All device memory of an engine
// lives in two allocations (a small one and an arena).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "pandemic_gb300.h"
#include "pt_host.h"
#include "pt_kernels.h"

namespace {

struct Arena {
    char *base = nullptr;
    size_t size = 0, used = 0;
    template <typename T>
    T *take(size_t count)
    {
        size_t bytes = ((count * sizeof(T)) + 255) & ~(size_t)255;
        T *p = reinterpret_cast<T *>(base + used);
        used += bytes;
        return p;
    }
};

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

thread_local std::string g_create_error;

// One simulation of an engine: its inputs and the host mirror of its results.
struct Instance {
    pt_params params;
    int core_seed = 0;
    pth::Derived derived;
    std::unique_ptr<pth::GlibcRand> rng;
    std::vector<int32_t> seed_list;   // the instance's person numbers
    ptk::SimConst c;
    int adults = 0;
    pt_interventions iv{};            // all zero: the reference's model
    int day = 0;                      // next day to run
    bool stopped = false;             // a day counted zero infected
    int days_run = 0;
    std::vector<int> counts;          // kMaxDays * 16
    std::vector<int> infected;        // kMaxDays
    float max_prop = 0.f;
    int max_prop_day = 0;
};

// Stage boundaries recorded per day when timing is on.
enum { kStSweep, kStInfectedList, kStSchedule, kStDigits, kStRadix, kStOffsets, kStInfect, kStApply, kStages };
static_assert(kStages == 8, "eight stages per day type in pt_get_stage_ms");

}  // namespace

struct Engine {
    std::vector<Instance> inst;
    std::vector<ptk::InstConst> ic;   // host copy of the device array
    ptk::DevArrays d;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    char *setup_mem = nullptr;        // household types/sizes during setup
    char *small_mem = nullptr;        // scalars, instance records, look-back words, histograms, household offsets
    size_t small_bytes = 0;
    char *arena_mem = nullptr;
    size_t arena_bytes = 0;
    int32_t *d_seeds = nullptr;
    int seeds_p = 0, seeds_s = 0;     // pandemic / seasonal seeds over all instances
    std::vector<int32_t> seed_global; // global person ids: all pandemic seeds, then all seasonal ones
    int *d_hist = nullptr;            // K x 512
    int64_t persons = 0;              // real persons over all instances
    bool setup_done = false;
    int next_day = 0;                 // next global day to run
    int max_days = 0;                 // longest max_days of the instances
    std::string err;
    bool timing = false;
    bool full_tables = false;             // materialise every bucket (tables complete for inspection)
    std::vector<cudaEvent_t> day_events;  // kMaxDays x (stages + 1), created on demand
    std::vector<int> timed_days;
    float stage_ms[16] = {0};             // [weekday stages 0..7, weekend stages 8..15]
    int stage_days[2] = {0, 0};
    std::vector<float> day_stage_ms;      // kMaxDays x kStages: the last timed run of each day
    mutable uint64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device copies issued
    // The whole day loop (days 0..max_days-1) captured once and replayed by run().
    // Every per-day decision (early stop, counters, offsets) reads device state, so
    // the same graph serves every run after a reset.
    cudaGraphExec_t run_graph = nullptr;
    uint64_t graph_kernels = 0;

    int K() const { return (int)inst.size(); }
    ~Engine();
};

struct pt_sim : Engine {};
struct pt_batch : Engine {};

// Every host<->device copy of the library goes through these, so the bytes a call
// moves across PCIe/C2C can be reported (pt_transfer_bytes).
// Engines take their device memory from one stream-ordered pool per device that keeps
// the blocks engines free (release threshold at its maximum): creating and destroying
// engines of similar sizes, as replicate loops and scenario sweeps do, reuses memory
// instead of mapping and unmapping gigabytes each time.  pt_trim_device_memory hands
// the unused part back to the device.
static std::mutex g_pool_mu;
static std::map<int, cudaMemPool_t> g_pools;

static cudaError_t engine_pool(cudaMemPool_t *out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(g_pool_mu);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
        cudaMemPoolDestroy(p);
        return e;
    }
    g_pools[dev] = p;
    *out = p;
    return cudaSuccess;
}

// Device memory for an engine, ordered on its stream; freed with cudaFreeAsync.
static cudaError_t engine_alloc(void **ptr, size_t bytes, cudaStream_t st)
{
    cudaMemPool_t pool = nullptr;
    cudaError_t e = engine_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(ptr, bytes, pool, st);
}

static cudaError_t pt_memcpy(const Engine *s, void *dst, const void *src, size_t n, cudaMemcpyKind k, cudaStream_t st)
{
    if (k == cudaMemcpyHostToDevice) s->h2d_bytes += n;
    else if (k == cudaMemcpyDeviceToHost) s->d2h_bytes += n;
    return cudaMemcpyAsync(dst, src, n, k, st);
}

static cudaError_t pt_memcpy_sync(const Engine *s, void *dst, const void *src, size_t n, cudaMemcpyKind k)
{
    cudaError_t e = pt_memcpy(s, dst, src, n, k, s->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s->stream);
}

static pt_status fail(Engine *s, pt_status st, const std::string &msg)
{
    if (s) s->err = msg;
    else g_create_error = msg;
    return st;
}

static pt_status cuda_fail(Engine *s, cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(s, e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA, m);
}

#define CK(expr, where)                                   \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_fail(s, _e, where); \
    } while (0)

Engine::~Engine()
{
    if (stream) cudaStreamSynchronize(stream);
    if (run_graph) cudaGraphExecDestroy(run_graph);
    // back to the pool, in stream order
    if (arena_mem) cudaFreeAsync(arena_mem, stream);
    if (setup_mem) cudaFreeAsync(setup_mem, stream);
    if (small_mem) cudaFreeAsync(small_mem, stream);
    if (stream) cudaStreamSynchronize(stream);
    for (auto &e : day_events)
        if (e) cudaEventDestroy(e);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

// PandemicSim::PandemicSim() for each instance: seeds, scaling, infection data.
// Needs no device: parameters and derived sizes can be inspected before setup.
static pt_status engine_create(Engine *s, const pt_params *params, const int *core_seeds, int K, void *cuda_stream)
{
    s->inst.resize(K);
    for (int k = 0; k < K; k++) {
        Instance &in = s->inst[k];
        in.params = params[k];
        in.core_seed = core_seeds[k];
        in.rng.reset(new pth::GlibcRand((unsigned int)in.core_seed));
        const char *why = nullptr;
        pt_status st = pth::derive(in.params, in.derived, *in.rng, &why);
        if (st != PT_OK) {
            std::string m = why ? why : "invalid parameters";
            if (K > 1) m = "instance " + std::to_string(k) + ": " + m;
            return fail(nullptr, st, m);
        }
        ptk::SimConst &c = in.c;
        std::memset(&c, 0, sizeof(c));
        c.H = in.derived.households;
        c.L = in.derived.workplaces;
        for (int t = 0; t < ptk::kTypes; t++) {
            c.type_count[t] = in.derived.type_count[t];
            c.type_offset[t] = in.derived.type_offset[t];
        }
        std::memcpy(c.shedding, in.derived.shedding, sizeof(c.shedding));
        c.infectiousness[0] = in.derived.infectiousness[0];
        c.infectiousness[1] = in.derived.infectiousness[1];
        c.pct_sympt = in.params.percent_symptomatic;
        c.key0 = in.derived.key0;
        c.key1 = in.derived.key1;
        if ((long long)c.L * 10 + 1 > 0x7FFFFFFFll) return fail(nullptr, PT_ERR_ARG, "too many locations");
        in.counts.assign(ptk::kMaxDays * 16, 0);
        in.infected.assign(ptk::kMaxDays, 0);
        s->max_days = std::max(s->max_days, in.params.max_days);
    }
    // The CUDA stream and events are created by setup.
    s->stream = (cudaStream_t)cuda_stream;
    return PT_OK;
}

static pt_status engine_reset(Engine *s);

// A fraction in [0, 1] as a threshold on a 32-bit hash value: hash < threshold with
// probability `fraction`.
static uint64_t fraction_threshold(float fraction)
{
    const double t = (double)fraction * 4294967296.0;
    return t <= 0.0 ? 0ull : (t >= 4294967296.0 ? 4294967296ull : (uint64_t)(t + 0.5));
}

static void apply_interventions(ptk::InstConst &r, const pt_interventions &iv)
{
    r.closure_start = iv.school_closure_start;
    r.closure_end = iv.school_closure_days > 0 ? iv.school_closure_start + iv.school_closure_days : 0;
    r.absent_thr = fraction_threshold(iv.workplace_absenteeism);
    r.vacc_thr = fraction_threshold(iv.vaccination_coverage);
}

static const char *check_interventions(const pt_interventions &iv)
{
    if (iv.school_closure_start < 0 || iv.school_closure_days < 0 || iv.school_closure_days > 256)
        return "school closure start and days must be >= 0 (days <= 256)";
    if (!(iv.workplace_absenteeism >= 0.f && iv.workplace_absenteeism <= 1.f))
        return "workplace absenteeism must be in [0, 1]";
    if (!(iv.vaccination_coverage >= 0.f && iv.vaccination_coverage <= 1.f))
        return "vaccination coverage must be in [0, 1]";
    return nullptr;
}

// Sets instance k's interventions; after setup the device record is updated at once
// (vaccination takes effect at the next reset).
static pt_status engine_set_interventions(Engine *s, int k, const pt_interventions &iv)
{
    if (const char *why = check_interventions(iv)) return fail(s, PT_ERR_ARG, why);
    s->inst[k].iv = iv;
    if (s->setup_done) {
        apply_interventions(s->ic[k], iv);
        CK(pt_memcpy_sync(s, (void *)(s->d.ic + k), &s->ic[k], sizeof(ptk::InstConst), cudaMemcpyHostToDevice),
           "instance record");
    }
    return PT_OK;
}

// PandemicSim::setupSim (PandemicSim.cu:146-208) for every instance: population,
// households, workplaces and schools, the workplace table, status arrays, initial
// infected.  Household types and workplace draws run per instance (each has its own
// counter stream); scans, the household scatter and the workplace table cover all
// instances at once.
static pt_status engine_setup(Engine *s)
{
    if (s->setup_done) return fail(s, PT_ERR_STATE, "setup called twice");
    if (!s->stream) {
        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        s->own_stream = true;
    }
    const int K = s->K();
    ptk::DevArrays &d = s->d;
    // household slots (H + 1 per instance: the last holds its padding persons),
    // locations and an upper bound of the persons
    std::vector<int> hbase(K), lbase(K), bbase0(K), bbase1(K);
    long long HS = 0, LT = 0, maxP = 0, B0 = 0, B1 = 0;
    for (int k = 0; k < K; k++) {
        const ptk::SimConst &c = s->inst[k].c;
        hbase[k] = (int)HS;
        lbase[k] = (int)LT;
        bbase0[k] = (int)B0;
        bbase1[k] = (int)B1;
        HS += (long long)c.H + 1;
        LT += c.L;
        B0 += ptk::day_buckets(c, false) + 1;  // each instance's buckets and its end slot
        B1 += ptk::day_buckets(c, true) + 1;
        maxP += 5ll * c.H + ptk::kPersonTile;  // the largest household type holds 5 persons
        if (HS + 1 > INT_MAX / 2 || LT + 2 > INT_MAX / 2 || B1 + 1 > INT_MAX / 2 || maxP > INT_MAX)
            return fail(s, PT_ERR_ARG, "batch too large for 32-bit ids");
    }
    const long long Bday = std::max(B0, B1), Bmax = std::max(Bday, LT + 1);
    const long long tiles_cap = std::max({maxP, Bmax + 1, HS + 1}) / ptk::kScanTileEntries + 4;

    // small block: scalars, look-back tiles and control words, instance records and
    // state, generation histograms, household offsets, setup counters
    const size_t small_bytes = round256(sizeof(ptk::Scalars)) +
                               round256((tiles_cap + 4) * sizeof(unsigned long long)) +
                               round256((size_t)K * sizeof(ptk::InstConst)) + round256((size_t)K * sizeof(ptk::InstState)) +
                               round256((size_t)K * 512 * sizeof(int)) + round256(((size_t)HS + 1) * 4) +
                               round256((size_t)2 * K * sizeof(int));
    CK(engine_alloc((void **)&s->small_mem, small_bytes, s->stream), "device memory (small)");
    s->small_bytes = small_bytes;
    Arena a0{s->small_mem, small_bytes, 0};
    d.sc = a0.take<ptk::Scalars>(1);
    d.tiles = a0.take<unsigned long long>(tiles_cap + 4);
    d.tiles_cap = (int)tiles_cap;
    ptk::InstConst *ic_dev = a0.take<ptk::InstConst>(K);
    d.ic = ic_dev;
    d.is = a0.take<ptk::InstState>(K);
    s->d_hist = a0.take<int>((size_t)K * 512);
    d.hh_offset = a0.take<int32_t>((size_t)HS + 1);
    int *d_counts = a0.take<int>((size_t)2 * K);  // adults, persons per instance
    // setup-only block: household types and sizes
    const size_t setup_bytes = round256((size_t)HS) + round256((size_t)HS * 4);
    CK(engine_alloc((void **)&s->setup_mem, setup_bytes, s->stream), "device memory (setup)");
    Arena a1{s->setup_mem, setup_bytes, 0};
    uint8_t *types = a1.take<uint8_t>((size_t)HS);
    int32_t *sizes = a1.take<int32_t>((size_t)HS);
    CK(cudaMemsetAsync(d.sc, 0, sizeof(ptk::Scalars), s->stream), "memset scalars");
    CK(cudaMemsetAsync(d.tiles, 0, (tiles_cap + 4) * sizeof(unsigned long long), s->stream), "memset tiles");
    CK(cudaMemsetAsync(d_counts, 0, (size_t)2 * K * sizeof(int), s->stream), "memset counters");
    int *ctl = (int *)(d.tiles + tiles_cap);

    // household types and sizes, persons and adults of each instance
    for (int k = 0; k < K; k++)
        CK(ptk::launch_household_types(s->inst[k].c, types + hbase[k], sizes + hbase[k], d_counts + k,
                                       d_counts + K + k, s->stream), "household_types");
    std::vector<int> hcounts((size_t)2 * K);
    CK(pt_memcpy_sync(s, hcounts.data(), d_counts, hcounts.size() * sizeof(int), cudaMemcpyDeviceToHost),
       "population counts");
    long long P = 0;
    std::vector<int> pbase(K);
    for (int k = 0; k < K; k++) {
        Instance &in = s->inst[k];
        const int N = hcounts[K + k];
        if (N <= 0) return fail(s, PT_ERR_STATE, "population is empty");
        in.c.N = N;
        in.adults = hcounts[k];
        in.c.workplace_offset = (uint64_t)(in.c.H / 4);
        if ((long long)in.params.initial_pandemic + in.params.initial_seasonal > N)
            return fail(s, PT_ERR_ARG, "more initial infected than persons");
        if ((long long)N * 3 >= (1ll << 30))
            return fail(s, PT_ERR_ARG, "population too large (3N must stay below 2^30)");
        pbase[k] = (int)P;
        P += ((long long)N + ptk::kPersonTile - 1) / ptk::kPersonTile * ptk::kPersonTile;
        s->persons += N;
    }
    if (3 * P >= (long long)INT_MAX) return fail(s, PT_ERR_ARG, "batch too large (3 x persons must stay below 2^31)");
    s->ic.resize(K);
    d.bucket_max[0] = d.bucket_max[1] = 1;
    for (int k = 0; k < K; k++) {
        ptk::InstConst &r = s->ic[k];
        std::memset(&r, 0, sizeof(r));
        r.c = s->inst[k].c;
        r.pbase = pbase[k];
        r.pend = k + 1 < K ? pbase[k + 1] : (int)P;
        r.hbase = hbase[k];
        r.lbase = lbase[k];
        r.bbase[0] = bbase0[k];
        r.bbase[1] = bbase1[k];
        r.bcount[0] = ptk::day_buckets(r.c, false);
        r.bcount[1] = ptk::day_buckets(r.c, true);
        d.bucket_max[0] = std::max(d.bucket_max[0], r.bcount[0]);
        d.bucket_max[1] = std::max(d.bucket_max[1], r.bcount[1]);
        r.max_days = s->inst[k].params.max_days;
        r.kbase = 3ll * pbase[k];
        apply_interventions(r, s->inst[k].iv);
    }
    CK(pt_memcpy(s, ic_dev, s->ic.data(), (size_t)K * sizeof(ptk::InstConst), cudaMemcpyHostToDevice, s->stream),
       "instance records");
    d.K = K;
    d.P = (int)P;
    d.buckets[0] = (int)B0;
    d.buckets[1] = (int)B1;
    d.locations = (int)LT;
    // padding slots, then one scan of all household slots: offsets and person bases
    CK(ptk::launch_batch_padding(d, types, sizes, 0, false, s->stream), "padding slots");
    CK(ptk::launch_scan_exclusive(sizes, d.hh_offset, (int)HS, 0, d.tiles, ctl, &d.sc->error, nullptr, 0, nullptr,
                                  s->stream), "household scan");

    // arena of per-person and per-location arrays
    const size_t n = (size_t)P, ntiles = n / ptk::kPersonTile;
    const size_t radix_tiles =  // segments round up to whole tiles
        (3 * n + ptk::kRadixTileEntries - 1) / ptk::kRadixTileEntries + 1 + (size_t)K;
    int nseeds = 0;
    for (const Instance &in : s->inst) nseeds += in.params.initial_pandemic + in.params.initial_seasonal;
    size_t bytes = 0;
    bytes += round256(n * 4);                   // state
    bytes += 3 * round256(n);                   // gen_p, gen_s, age
    bytes += round256(n * 4) * 3;               // household, workplace, wp_people
    bytes += round256(n * 16);                  // packed person records
    bytes += round256(((size_t)LT + 2) * 4);    // wp_offset
    bytes += round256(3 * n * 4) * 6;           // keys, bkt_people, radix k0/v0/k1/v1
    bytes += round256(((size_t)Bday + 1) * 4);  // bkt_offset
    bytes += round256((size_t)Bmax * 4);        // bkt_count (also the workplace histogram)
    bytes += round256(radix_tiles * 256 * 8);   // radix look-back words
    bytes += round256(8 * 4);                                                      // radix ctl
    bytes += round256((size_t)K * ptk::kDigitStripes * 4 * 256 * 4);               // digit histograms
    bytes += round256((size_t)K * 4 * 256 * 4) + 2 * round256(((size_t)K + 1) * 4);  // digit bases, tile prefixes
    bytes += round256(((size_t)Bday / 32 + 1) * 4);        // bucket mark bitmap
    bytes += round256(n * 4) * 2;               // infected, infected_inst
    bytes += round256(n / 16 * 2) + round256((ntiles + 1) * 4);  // sweep masks, sweep tile counts
    bytes += round256(2 * n * 8);               // claim
    bytes += round256(2 * n * 4);               // new_list
    bytes += round256((size_t)(nseeds + 1) * 4);  // seeds
    bytes += round256(ntiles * 4);              // tile_inst
    CK(engine_alloc((void **)&s->arena_mem, bytes, s->stream), "device memory (arena)");
    s->arena_bytes = bytes;
    Arena a{s->arena_mem, bytes, 0};
    d.state = a.take<uint32_t>(n);
    d.gen_p = a.take<uint8_t>(n);
    d.gen_s = a.take<uint8_t>(n);
    d.age = a.take<uint8_t>(n);
    d.household = a.take<int32_t>(n);
    d.workplace = a.take<int32_t>(n);
    d.wp_people = a.take<int32_t>(n);
    d.wp_offset = a.take<int32_t>((size_t)LT + 2);
    d.prec = a.take<uint4>(n);
    d.keys = a.take<int32_t>(3 * n);
    d.bkt_people = a.take<int32_t>(3 * n);
    d.rk0 = a.take<uint32_t>(3 * n);
    d.rv0 = a.take<uint32_t>(3 * n);
    d.rk1 = a.take<uint32_t>(3 * n);
    d.rv1 = a.take<uint32_t>(3 * n);
    d.bkt_offset = a.take<int32_t>((size_t)Bday + 1);
    d.bkt_count = a.take<int32_t>((size_t)Bmax);
    d.radix_status = a.take<unsigned long long>(radix_tiles * 256);
    d.radix_ctl = a.take<int>(8);
    d.digit_hist = a.take<int>((size_t)K * ptk::kDigitStripes * 4 * 256);
    d.digit_base = a.take<int>((size_t)K * 4 * 256);
    d.tile_prefix = a.take<int32_t>((size_t)K + 1);
    d.tile_prefix0 = a.take<int32_t>((size_t)K + 1);
    d.mark = a.take<uint32_t>((size_t)Bday / 32 + 1);
    d.infected = a.take<int32_t>(n);
    d.infected_inst = a.take<int32_t>(n);
    d.sweep_flags = a.take<uint16_t>(n / 16);
    d.sweep_tiles = a.take<int32_t>(ntiles + 1);
    d.claim = a.take<unsigned long long>(2 * n);
    d.new_list = a.take<int32_t>(2 * n);
    s->d_seeds = a.take<int32_t>((size_t)(nseeds + 1));
    int32_t *tile_inst = a.take<int32_t>(ntiles);
    d.tile_inst = tile_inst;
    {
        std::vector<int32_t> ti(ntiles);
        for (int k = 0; k < K; k++) {
            const size_t t0 = (size_t)pbase[k] / ptk::kPersonTile;
            const size_t t1 = k + 1 < K ? (size_t)pbase[k + 1] / ptk::kPersonTile : ntiles;
            for (size_t t = t0; t < t1; t++) ti[t] = k;
        }
        CK(pt_memcpy(s, tile_inst, ti.data(), ntiles * 4, cudaMemcpyHostToDevice, s->stream), "tile map");
        CK(cudaStreamSynchronize(s->stream), "tile map sync");
    }
    CK(cudaMemsetAsync(d.bkt_count, 0, (size_t)Bmax * 4, s->stream), "memset counts");
    CK(cudaMemsetAsync(d.radix_ctl, 0, 8 * 4, s->stream), "memset radix ctl");
    CK(cudaMemsetAsync(d.radix_status, 0, radix_tiles * 256 * 8, s->stream), "memset radix words");
    CK(cudaMemsetAsync(d.digit_hist, 0, (size_t)K * ptk::kDigitStripes * 4 * 256 * 4, s->stream), "memset digit hist");

    // households -> persons, padding persons, then workplaces and schools (setup_assignWorkplaces)
    CK(ptk::launch_generate_households(types, d.hh_offset, (int)HS, d.household, d.age, s->stream), "households");
    CK(ptk::launch_batch_padding(d, types, sizes, (int)LT, true, s->stream), "padding persons");
    for (int k = 0; k < K; k++)
        CK(ptk::launch_assign_workplaces(s->inst[k].c, d.age + pbase[k], d.workplace + pbase[k], lbase[k], s->stream),
           "workplaces");
    // workplace table: person ids stably sorted by workplace, with offsets
    // (setup_assignWorkplaces' radix sort + lower_bound, PandemicSim.cu:3835-3862);
    // padding persons sit in the spare location LT, behind every instance's persons
    {
        ptk::RadixArgs r;
        r.keys = (const uint32_t *)d.workplace;
        r.E = (int)P;
        r.buckets = (int)LT + 1;
        r.N = (int)P;
        r.person_mode = 0;
        r.k0 = d.rk0; r.v0 = d.rv0; r.k1 = d.rk1; r.v1 = d.rv1;
        r.out = (uint32_t *)d.wp_people;
        r.digit_base = d.digit_base;
        r.status = d.radix_status;
        r.ctl = d.radix_ctl;
        r.error = &d.sc->error;
        r.skip = nullptr;
        CK(ptk::launch_bucket_table(r, d.bkt_count, true, d.wp_offset, d.tiles, ctl, d.digit_hist, s->stream),
           "workplace table");
    }
    CK(ptk::launch_person_records(d, s->stream), "person records");
    // initial infected: rand() % N draws continue each instance's seed sequence
    // (PandemicSim.cu:708-758); the first P of an instance get the pandemic strain
    s->seed_global.clear();
    std::vector<int32_t> seasonal;
    for (int k = 0; k < K; k++) {
        Instance &in = s->inst[k];
        const int np = in.params.initial_pandemic, ns = in.params.initial_seasonal;
        in.seed_list = pth::unique_numbers(*in.rng, np + ns, in.c.N);
        for (int i = 0; i < np + ns; i++) (i < np ? s->seed_global : seasonal).push_back(pbase[k] + in.seed_list[i]);
    }
    s->seeds_p = (int)s->seed_global.size();
    s->seeds_s = (int)seasonal.size();
    s->seed_global.insert(s->seed_global.end(), seasonal.begin(), seasonal.end());
    int derr = 0;
    CK(pt_memcpy(s, &derr, &d.sc->error, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "error flag");
    CK(cudaStreamSynchronize(s->stream), "setup sync");
    cudaFreeAsync(s->setup_mem, s->stream);
    s->setup_mem = nullptr;
    if (derr) return fail(s, PT_ERR_TIMEOUT, "a device-side wait gave up during setup");
    pt_status st = engine_reset(s);
    if (st != PT_OK) return st;
    s->setup_done = true;
    return PT_OK;
}

static pt_status engine_reset(Engine *s)
{
    ptk::DevArrays &d = s->d;
    CK(ptk::launch_init_status(d.P, d.state, d.gen_p, d.gen_s, d.claim, s->stream), "init_status");
    bool vaccination = false;
    for (const ptk::InstConst &r : s->ic) vaccination |= r.vacc_thr != 0;
    if (vaccination) CK(ptk::launch_vaccinate(d, s->stream), "vaccinate");
    if (!s->seed_global.empty()) {
        CK(pt_memcpy(s, s->d_seeds, s->seed_global.data(), sizeof(int32_t) * s->seed_global.size(),
                     cudaMemcpyHostToDevice, s->stream), "seed copy");
        CK(ptk::launch_seed_infected(s->d_seeds, s->seeds_p, s->seeds_s, d.state, d.gen_p, d.gen_s, s->stream), "seed");
    }
    CK(cudaMemsetAsync(d.sc, 0, sizeof(ptk::Scalars), s->stream), "memset scalars");
    CK(ptk::launch_reset_instances(d, s->stream), "reset instances");
    CK(cudaStreamSynchronize(s->stream), "reset sync");
    s->next_day = 0;
    for (Instance &in : s->inst) {
        in.day = 0;
        in.stopped = false;
        in.days_run = 0;
        in.max_prop = 0.f;
        in.max_prop_day = 0;
        std::fill(in.counts.begin(), in.counts.end(), 0);
        std::fill(in.infected.begin(), in.infected.end(), 0);
    }
    return PT_OK;
}

static cudaEvent_t stage_event(Engine *s, int day, int k)
{
    return s->day_events[(size_t)day * (kStages + 1) + k];
}

// Enqueues one day of every instance: sweep, schedule, bucket build (scan, radix
// sort), infection, apply.  Every kernel after the sweep skips an instance that
// counted no infected, and skips itself once no instance has infected left.
static pt_status enqueue_day(Engine *s, int day)
{
    const bool weekend = (day % 7) >= 5;  // PandemicSim.h:283-284
    const ptk::DevArrays &d = s->d;
    cudaStream_t st = s->stream;
    const bool t = s->timing;
    if (t) cudaEventRecord(stage_event(s, day, kStSweep), st);
    CK(ptk::launch_sweep(d, day, st), "sweep");
    if (t) cudaEventRecord(stage_event(s, day, kStInfectedList), st);
    CK(ptk::launch_infected_list(d, st), "infected list");
    if (t) cudaEventRecord(stage_event(s, day, kStSchedule), st);
    CK(ptk::launch_schedule(d, weekend, day, s->full_tables, st), "schedule");
    if (t) cudaEventRecord(stage_event(s, day, kStDigits), st);
    CK(ptk::launch_bucket_scan(d, weekend, st), "digit bases");
    if (t) cudaEventRecord(stage_event(s, day, kStRadix), st);
    CK(ptk::launch_bucket_sort(d, weekend, st), "bucket sort");
    if (t) cudaEventRecord(stage_event(s, day, kStOffsets), st);
    CK(ptk::launch_bucket_offsets(d, weekend, s->full_tables, st), "bucket offsets");
    if (t) cudaEventRecord(stage_event(s, day, kStInfect), st);
    CK(ptk::launch_infect(d, weekend, day, st), "infect");
    if (t) cudaEventRecord(stage_event(s, day, kStApply), st);
    CK(ptk::launch_apply(d, day, st), "apply");
    if (t) cudaEventRecord(stage_event(s, day, kStages), st);
    if (t) s->timed_days.push_back(day);
    return PT_OK;
}

static void accumulate_timing(Engine *s)
{
    if (!s->timing) return;
    cudaStreamSynchronize(s->stream);
    for (int day : s->timed_days) {
        const bool weekend = (day % 7) >= 5;
        if (s->day_stage_ms.empty()) s->day_stage_ms.assign((size_t)ptk::kMaxDays * kStages, 0.f);
        for (int k = 0; k < kStages; k++) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, stage_event(s, day, k), stage_event(s, day, k + 1)) == cudaSuccess)
                s->stage_ms[(weekend ? 8 : 0) + k] += ms;
            s->day_stage_ms[(size_t)day * kStages + k] = ms;
        }
        s->stage_days[weekend ? 1 : 0]++;
    }
    s->timed_days.clear();
}

static void track_peak(Engine *s, Instance &in, int day, int I)
{
    (void)s;
    // PandemicSim.cu:923-931: strictly greater proportions only
    float prop = (float)I / (float)in.c.N;
    if (prop > in.max_prop) {
        in.max_prop = prop;
        in.max_prop_day = day;
    }
}

// Copies every instance's rows of days [lo, hi) (strided copies out of the device
// state records), checks the device error word and updates the host mirrors.
static pt_status fetch_rows(Engine *s, int lo, int hi)
{
    const int K = s->K();
    const size_t pitch = sizeof(ptk::InstState);
    const int days = std::max(0, hi - lo);
    std::vector<int> hc((size_t)K * 16 * std::max(days, 1)), hi_((size_t)K * std::max(days, 1)), rows(K);
    char *base = reinterpret_cast<char *>(s->d.is);
    if (days > 0) {
        const size_t wc = (size_t)days * 16 * sizeof(int), wi = (size_t)days * sizeof(int);
        s->d2h_bytes += (uint64_t)K * (wc + wi);
        CK(cudaMemcpy2DAsync(hc.data(), wc, base + offsetof(ptk::InstState, counts) + (size_t)lo * 16 * sizeof(int),
                             pitch, wc, K, cudaMemcpyDeviceToHost, s->stream), "counts");
        CK(cudaMemcpy2DAsync(hi_.data(), wi, base + offsetof(ptk::InstState, infected_per_day) + (size_t)lo * sizeof(int),
                             pitch, wi, K, cudaMemcpyDeviceToHost, s->stream), "infected");
    }
    s->d2h_bytes += (uint64_t)K * sizeof(int);
    CK(cudaMemcpy2DAsync(rows.data(), sizeof(int), base + offsetof(ptk::InstState, days_run), pitch, sizeof(int), K,
                         cudaMemcpyDeviceToHost, s->stream), "rows");
    int e = 0;
    CK(pt_memcpy(s, &e, &s->d.sc->error, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "error flag");
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (e) return fail(s, PT_ERR_TIMEOUT, "a device-side wait gave up (look-back ordering)");
    accumulate_timing(s);
    for (int k = 0; k < K; k++) {
        Instance &in = s->inst[k];
        if (in.stopped) continue;
        for (int day = in.days_run; day < rows[k]; day++) {
            if (day < lo || day >= hi) continue;  // outside the rows copied
            const size_t r = (size_t)k * days + (day - lo);
            std::memcpy(&in.counts[(size_t)day * 16], &hc[r * 16], 16 * sizeof(int));
            in.infected[day] = hi_[r];
            if (hi_[r] == 0) {
                in.stopped = true;
                break;
            }
            track_peak(s, in, day, hi_[r]);
        }
        in.days_run = rows[k];
        in.day = in.stopped ? rows[k] - 1 : rows[k];
    }
    return PT_OK;
}

static int instances_running(const Engine *s)
{
    int n = 0;
    for (const Instance &in : s->inst)
        if (!in.stopped && in.day < in.params.max_days) n++;
    return n;
}

static bool all_zero_stopped(const Engine *s)
{
    for (const Instance &in : s->inst)
        if (!in.stopped) return false;
    return true;
}

// One day of every running instance (runToCompletion's loop body, PandemicSim.cu:882-954).
static pt_status engine_step(Engine *s, int *running)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "step before setup");
    if (instances_running(s) == 0) return all_zero_stopped(s) ? PT_DONE : PT_FINISHED;
    const int day = s->next_day;
    pt_status st = enqueue_day(s, day);
    if (st != PT_OK) return st;
    s->next_day = day + 1;
    st = fetch_rows(s, day, day + 1);
    if (st != PT_OK) return st;
    if (running) *running = instances_running(s);
    return all_zero_stopped(s) ? PT_DONE : PT_OK;
}

// The remaining days of every instance on the device, then one copy of the rows.
static pt_status engine_run(Engine *s)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "run before setup");
    const int first = s->next_day, M = s->max_days;
    if (instances_running(s) > 0 && first < M) {
        if (first == 0 && !s->timing) {
            if (!s->run_graph) {
                const uint64_t before = ptk::launches();
                CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
                pt_status st = PT_OK;
                for (int day = 0; day < M && st == PT_OK; day++) st = enqueue_day(s, day);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(s->stream, &g);
                if (st != PT_OK) {
                    if (g) cudaGraphDestroy(g);
                    return st;
                }
                CK(e, "end capture");
                e = cudaGraphInstantiate(&s->run_graph, g, 0);
                cudaGraphDestroy(g);
                CK(e, "graph instantiate");
                s->graph_kernels = ptk::launches() - before;
                ptk::add_launches(-(int64_t)s->graph_kernels);  // counted when the graph runs
            }
            CK(cudaGraphLaunch(s->run_graph, s->stream), "graph launch");
            ptk::add_launches((int64_t)s->graph_kernels);
        } else {
            for (int day = first; day < M; day++) {
                pt_status st = enqueue_day(s, day);
                if (st != PT_OK) return st;
            }
        }
        s->next_day = M;
    }
    return fetch_rows(s, first, std::max(first, M));
}

static pt_status engine_gen_counts(Engine *s, int *gen_p, int *gen_s)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "generation counts before setup");
    const int K = s->K();
    CK(ptk::launch_gen_hist(s->d, s->d_hist, s->stream), "gen hist");
    std::vector<int> h((size_t)K * 512);
    CK(pt_memcpy_sync(s, h.data(), s->d_hist, h.size() * sizeof(int), cudaMemcpyDeviceToHost), "hist copy");
    for (int k = 0; k < K; k++) {
        std::memcpy(gen_p + (size_t)k * 256, &h[(size_t)k * 512], 256 * sizeof(int));
        std::memcpy(gen_s + (size_t)k * 256, &h[(size_t)k * 512 + 256], 256 * sizeof(int));
    }
    return PT_OK;
}

static pt_status engine_info(const Engine *cs, int k, pt_info *out)
{
    Engine *s = const_cast<Engine *>(cs);
    std::memset(out, 0, sizeof(*out));
    const Instance &in = s->inst[k];
    out->number_people = in.c.N;
    out->number_households = in.c.H;
    out->number_workplaces = in.c.L;
    out->number_adults = in.adults;
    out->number_children = in.c.N - in.adults;
    out->current_day = in.day;
    out->days_run = in.days_run;
    out->infected_count = in.days_run > 0 ? in.infected[in.days_run - 1] : 0;
    for (int i = 0; i < 4; i++) out->seeds[i] = in.derived.seeds[i];
    for (int t = 0; t < ptk::kTypes; t++) {
        out->type_count[t] = in.c.type_count[t];
        out->type_offset[t] = in.c.type_offset[t];
    }
    out->infectiousness[0] = in.c.infectiousness[0];
    out->infectiousness[1] = in.c.infectiousness[1];
    out->max_day_of_peak = in.max_prop_day;
    out->max_infected_proportion = in.max_prop;
    out->sm_count = ptk::sm_count();
    out->device_bytes = s->arena_bytes + s->small_bytes;
    if (s->setup_done) {
        unsigned long long ro = 0, mat = 0;
        CK(pt_memcpy(s, &ro, &s->d.is[k].rand_offset, sizeof(ro), cudaMemcpyDeviceToHost, s->stream), "offset");
        CK(pt_memcpy_sync(s, &mat, &s->d.sc->materialised_sum, sizeof(mat), cudaMemcpyDeviceToHost), "materialised");
        out->rand_offset = ro;
        out->bucket_entries_materialised = mat;  // over all instances of the engine
        uint64_t total = 0;
        for (int day = 0; day < in.days_run; day++)
            if (in.infected[day] > 0) total += (uint64_t)((day % 7) >= 5 ? 3 : 2) * (uint64_t)in.c.N;
        out->bucket_entries_scheduled = total;
    }
    return PT_OK;
}

static pt_status engine_person_state(Engine *s, int k, uint8_t *status_p, uint8_t *status_s, uint8_t *day_p,
                                     uint8_t *day_s, uint8_t *gen_p, uint8_t *gen_s, uint8_t *age)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "state before setup");
    const size_t N = (size_t)s->inst[k].c.N, pb = (size_t)s->ic[k].pbase;
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (status_p || status_s || day_p || day_s) {
        std::vector<uint32_t> st(N);
        CK(pt_memcpy_sync(s, st.data(), s->d.state + pb, N * 4, cudaMemcpyDeviceToHost), "state copy");
        for (size_t i = 0; i < N; i++) {
            if (status_p) status_p[i] = (uint8_t)(st[i] & 0xFF);
            if (status_s) status_s[i] = (uint8_t)((st[i] >> 8) & 0xFF);
            if (day_p) day_p[i] = (uint8_t)((st[i] >> 16) & 0xFF);
            if (day_s) day_s[i] = (uint8_t)(st[i] >> 24);
        }
    }
    if (gen_p) CK(pt_memcpy_sync(s, gen_p, s->d.gen_p + pb, N, cudaMemcpyDeviceToHost), "gen copy");
    if (gen_s) CK(pt_memcpy_sync(s, gen_s, s->d.gen_s + pb, N, cudaMemcpyDeviceToHost), "gen copy");
    if (age) CK(pt_memcpy_sync(s, age, s->d.age + pb, N, cudaMemcpyDeviceToHost), "age copy");
    return PT_OK;
}

// Setup tables of instance k in its own numbering (global ids minus its bases).
static pt_status engine_population(Engine *s, int k, int32_t *household, int32_t *household_offset,
                                   int32_t *workplace, int32_t *workplace_people, int32_t *workplace_offset)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "population before setup");
    const ptk::InstConst &r = s->ic[k];
    const size_t N = (size_t)r.c.N, H = (size_t)r.c.H, L = (size_t)r.c.L;
    CK(cudaStreamSynchronize(s->stream), "sync");
    auto rebase = [](int32_t *v, size_t n, int32_t by) {
        if (by)
            for (size_t i = 0; i < n; i++) v[i] -= by;
    };
    if (household) {
        CK(pt_memcpy_sync(s, household, s->d.household + r.pbase, N * 4, cudaMemcpyDeviceToHost), "copy");
        rebase(household, N, r.hbase);
    }
    if (household_offset) {
        CK(pt_memcpy_sync(s, household_offset, s->d.hh_offset + r.hbase, (H + 1) * 4, cudaMemcpyDeviceToHost), "copy");
        rebase(household_offset, H + 1, r.pbase);
    }
    if (workplace) {
        CK(pt_memcpy_sync(s, workplace, s->d.workplace + r.pbase, N * 4, cudaMemcpyDeviceToHost), "copy");
        rebase(workplace, N, r.lbase);
    }
    if (workplace_people || workplace_offset) {
        std::vector<int32_t> off(L + 1);
        CK(pt_memcpy_sync(s, off.data(), s->d.wp_offset + r.lbase, (L + 1) * 4, cudaMemcpyDeviceToHost), "copy");
        const int32_t first = off[0];
        if (workplace_people) {
            CK(pt_memcpy_sync(s, workplace_people, s->d.wp_people + first, N * 4, cudaMemcpyDeviceToHost), "copy");
            rebase(workplace_people, N, r.pbase);
        }
        if (workplace_offset) {
            for (size_t i = 0; i <= L; i++) workplace_offset[i] = off[i] - first;
        }
    }
    return PT_OK;
}

static pt_status engine_set_timing(Engine *s, int enabled)
{
    if (enabled && s->day_events.empty()) {
        s->day_events.resize((size_t)ptk::kMaxDays * (kStages + 1));
        for (auto &e : s->day_events) CK(cudaEventCreate(&e), "cudaEventCreate");
    }
    s->timing = enabled != 0;
    std::memset(s->stage_ms, 0, sizeof(s->stage_ms));
    s->stage_days[0] = s->stage_days[1] = 0;
    return PT_OK;
}

static pt_status engine_stage_ms(Engine *s, float ms[16], int days[2])
{
    accumulate_timing(s);
    std::memcpy(ms, s->stage_ms, sizeof(s->stage_ms));
    if (days) {
        days[0] = s->stage_days[0];
        days[1] = s->stage_days[1];
    }
    std::memset(s->stage_ms, 0, sizeof(s->stage_ms));
    s->stage_days[0] = s->stage_days[1] = 0;
    return PT_OK;
}

// ------------------------------------------------------------------ launch shapes
static pt_tuning to_public(const ptk::Tuning &t)
{
    pt_tuning o;
    o.infect_coop = t.infect_coop;
    o.infect_blocks_per_sm = t.infect_blocks_per_sm;
    o.radix_blocks_per_sm = t.radix_blocks_per_sm;
    o.sched_tf = t.sched_tf;
    o.dense_level = t.dense_level;
    o.radix_threads = t.radix_threads;
    return o;
}

static pt_status engine_set_tuning(Engine *s, const pt_tuning *t)
{
    if (!t || (t->infect_coop != 0 && t->infect_coop != 1) || t->infect_blocks_per_sm < 1 ||
        t->infect_blocks_per_sm > 32 || t->radix_blocks_per_sm < 1 || t->radix_blocks_per_sm > 4 ||
        t->sched_tf < 0 || t->sched_tf > 2 || t->dense_level < 0 || t->dense_level > 3 ||
        (t->radix_threads != 256 && t->radix_threads != 512) ||
        (t->radix_threads == 512 && t->radix_blocks_per_sm > 2))
        return fail(s, PT_ERR_ARG, "launch shape outside its range");
    ptk::Tuning n;
    n.infect_coop = t->infect_coop;
    n.infect_blocks_per_sm = t->infect_blocks_per_sm;
    n.radix_blocks_per_sm = t->radix_blocks_per_sm;
    n.sched_tf = t->sched_tf;
    n.dense_level = t->dense_level;
    n.radix_threads = t->radix_threads;
    if (n.infect_coop != s->d.tune.infect_coop || n.infect_blocks_per_sm != s->d.tune.infect_blocks_per_sm ||
        n.radix_blocks_per_sm != s->d.tune.radix_blocks_per_sm || n.sched_tf != s->d.tune.sched_tf ||
        n.dense_level != s->d.tune.dense_level || n.radix_threads != s->d.tune.radix_threads) {
        // the captured day loop holds the old launch shapes
        if (s->stream) cudaStreamSynchronize(s->stream);
        if (s->run_graph) cudaGraphExecDestroy(s->run_graph);
        s->run_graph = nullptr;
    }
    s->d.tune = n;
    return PT_OK;
}

// Shapes already chosen in this process, by engine size.
static std::mutex g_tune_mutex;
static std::map<std::vector<long long>, pt_tuning> g_tune_cache;

static std::vector<long long> tune_key(const Engine *s)
{
    return {s->K(), s->d.P, s->d.bucket_max[0], s->d.bucket_max[1], s->d.buckets[0], s->d.buckets[1],
            s->max_days, ptk::sm_count()};
}

// The tuner.  The infection, radix and schedule stages are timed separately (per-stage
// CUDA events around every day), so one run measures one candidate of each: run i
// uses infection candidate i, radix candidate i % 3 and Threefry form (i + 1) % 3.
// Two more runs then try the dense-day sort levels 2 and 3 with the shapes chosen.
static pt_status engine_autotune(Engine *s, int days, pt_tuning *chosen)
{
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "autotune before setup");
    if (days < 0) return fail(s, PT_ERR_ARG, "negative day count");
    const std::vector<long long> key = tune_key(s);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            pt_status st = engine_set_tuning(s, &it->second);
            if (st == PT_OK && chosen) *chosen = it->second;
            return st;
        }
    }
    struct Cand { int coop, bps; };
    // thread-per-infector kernel: 9 resident 128-thread blocks per SM at 56 registers;
    // warp-cooperative kernel: 6 resident 256-thread blocks per SM at 40 registers
    const Cand infect[] = {{0, 8}, {0, 4}, {1, 6}, {1, 12}, {1, 3}, {0, 16}};
    // radix passes: (blocks per SM, threads per block)
    const int radix[] = {3, 4, 2};
    const int radix_threads[] = {256, 256, 512};
    const int tfs[] = {0, 1, 2};
    const int runs = (int)(sizeof(infect) / sizeof(infect[0]));
    float best_inf = 1e30f, best_rad[3] = {1e30f, 1e30f, 1e30f}, best_tf[3] = {1e30f, 1e30f, 1e30f};
    int best_i = 0;
    const int saved_max = s->max_days;
    const int trial = days > 0 ? std::min(days, saved_max) : saved_max;
    for (int i = 0; i < runs; i++) {
        pt_tuning t;
        t.infect_coop = infect[i].coop;
        t.infect_blocks_per_sm = infect[i].bps;
        t.radix_blocks_per_sm = radix[i % 3];
        t.radix_threads = radix_threads[i % 3];
        t.sched_tf = tfs[(i + 1) % 3];
        t.dense_level = 0;
        pt_status st = engine_set_tuning(s, &t);
        if (st == PT_OK) st = engine_reset(s);
        if (st == PT_OK) st = engine_set_timing(s, 1);
        if (st != PT_OK) return st;
        s->max_days = trial;
        st = engine_run(s);
        s->max_days = saved_max;
        if (st != PT_OK) return st;
        float ms[16];
        engine_stage_ms(s, ms, nullptr);
        const float inf = ms[kStInfect] + ms[8 + kStInfect];
        const float rad = ms[kStRadix] + ms[8 + kStRadix];
        const float sch = ms[kStSchedule] + ms[8 + kStSchedule];
        best_tf[(i + 1) % 3] = std::min(best_tf[(i + 1) % 3], sch);
        if (inf < best_inf) {
            best_inf = inf;
            best_i = i;
        }
        best_rad[i % 3] = std::min(best_rad[i % 3], rad);
    }
    int rbest = 0, tbest = 0;
    for (int r = 1; r < 3; r++) {
        if (best_rad[r] < best_rad[rbest]) rbest = r;
        if (best_tf[r] < best_tf[tbest]) tbest = r;
    }
    pt_tuning t;
    t.infect_coop = infect[best_i].coop;
    t.infect_blocks_per_sm = infect[best_i].bps;
    t.radix_blocks_per_sm = radix[rbest];
    t.radix_threads = radix_threads[rbest];
    t.sched_tf = tfs[tbest];
    t.dense_level = 0;
    // the dense-day sort changes both the schedule and the sort stage: its levels are
    // timed after the others are chosen, against their schedule + sort time
    float best_dense = best_rad[rbest] + best_tf[tbest];
    for (int lv = 2; lv <= 3; lv++) {
        pt_tuning c = t;
        c.dense_level = lv;
        pt_status st = engine_set_tuning(s, &c);
        if (st == PT_OK) st = engine_reset(s);
        if (st == PT_OK) st = engine_set_timing(s, 1);
        if (st != PT_OK) return st;
        s->max_days = trial;
        st = engine_run(s);
        s->max_days = saved_max;
        if (st != PT_OK) return st;
        float ms[16];
        engine_stage_ms(s, ms, nullptr);
        const float cost = ms[kStRadix] + ms[8 + kStRadix] + ms[kStSchedule] + ms[8 + kStSchedule];
        if (cost < best_dense) {
            best_dense = cost;
            t.dense_level = lv;
        }
    }
    pt_status st = engine_set_timing(s, 0);
    if (st == PT_OK) st = engine_set_tuning(s, &t);
    if (st == PT_OK) st = engine_reset(s);
    if (st != PT_OK) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = t;
    }
    if (chosen) *chosen = t;
    return PT_OK;
}

extern "C" {

// ------------------------------------------------------------------ one simulation
pt_status pt_create(const pt_params *params, int core_seed, void *cuda_stream, pt_sim **out)
{
    if (!params || !out) return fail(nullptr, PT_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<pt_sim> s(new pt_sim());
    pt_status st = engine_create(s.get(), params, &core_seed, 1, cuda_stream);
    if (st != PT_OK) return st;
    *out = s.release();
    return PT_OK;
}

pt_status pt_setup(pt_sim *s)
{
    if (!s) return PT_ERR_ARG;
    if (s->setup_done) return fail(s, PT_ERR_STATE, "pt_setup called twice");
    return engine_setup(s);
}

pt_status pt_reset_epidemic(pt_sim *s)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_reset_epidemic before pt_setup");
    return engine_reset(s);
}

pt_status pt_step_day(pt_sim *s, int counts16[16], int *infected_count)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_step_day before pt_setup");
    const Instance &in = s->inst[0];
    const int day = in.day;
    const bool ran = !in.stopped && day < in.params.max_days;
    pt_status st = engine_step(s, nullptr);
    if (!ran || st < 0) return st;
    if (counts16) std::memcpy(counts16, &in.counts[(size_t)day * 16], 16 * sizeof(int));
    if (infected_count) *infected_count = in.infected[day];
    return st;
}

pt_status pt_run(pt_sim *s, int *counts, int *infected, int *days_run)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_run before pt_setup");
    pt_status st = engine_run(s);
    if (st != PT_OK) return st;
    const Instance &in = s->inst[0];
    if (counts) std::memcpy(counts, in.counts.data(), (size_t)in.days_run * 16 * sizeof(int));
    if (infected) std::memcpy(infected, in.infected.data(), (size_t)in.days_run * sizeof(int));
    if (days_run) *days_run = in.days_run;
    return PT_OK;
}

pt_status pt_final_gen_counts(pt_sim *s, int gen_p[256], int gen_s[256])
{
    if (!s || !gen_p || !gen_s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_final_gen_counts before pt_setup");
    return engine_gen_counts(s, gen_p, gen_s);
}

pt_status pt_get_info(const pt_sim *s, pt_info *out)
{
    if (!s || !out) return PT_ERR_ARG;
    return engine_info(s, 0, out);
}

pt_status pt_get_person_state(pt_sim *s, uint8_t *status_p, uint8_t *status_s, uint8_t *day_p, uint8_t *day_s,
                              uint8_t *gen_p, uint8_t *gen_s, uint8_t *age)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "state before pt_setup");
    return engine_person_state(s, 0, status_p, status_s, day_p, day_s, gen_p, gen_s, age);
}

pt_status pt_get_population(pt_sim *s, int32_t *household, int32_t *household_offset, int32_t *workplace,
                            int32_t *workplace_people, int32_t *workplace_offset)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "population before pt_setup");
    return engine_population(s, 0, household, household_offset, workplace, workplace_people, workplace_offset);
}

// The device keeps each day's buckets in compact form: errand destinations of a
// day all lie in [lo, L) (lo = first location of type 8 on weekdays, type 9 on
// weekends), so bucket hour*R + dest - lo (R = L - lo) replaces the reference's key
// hour*L + dest.  This copies the tables back in the reference's layout: keys
// hour*L + dest and offsets over all 2L (10L) keys, offsets[k] = number of entries
// with a smaller key.
pt_status pt_get_day_tables(pt_sim *s, int32_t *infected, int32_t *keys, int32_t *people, int32_t *offsets,
                            int *entries, int *buckets)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "tables before pt_setup");
    CK(cudaStreamSynchronize(s->stream), "sync");
    int dayinf[2] = {0, 0};
    CK(pt_memcpy(s, &dayinf[0], &s->d.is[0].day, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "day");
    CK(pt_memcpy_sync(s, &dayinf[1], &s->d.is[0].infected, sizeof(int), cudaMemcpyDeviceToHost), "infected");
    const int day = dayinf[0], I = dayinf[1];
    const bool weekend = (day % 7) >= 5;
    const ptk::SimConst &c = s->inst[0].c;
    const int L = c.L, hours = weekend ? 10 : 2;
    const int lo = c.type_offset[weekend ? 9 : 8], R = L - lo;
    const int E = (weekend ? 3 : 2) * c.N, B = hours * L;
    const int Bc = ptk::day_buckets(c, weekend);
    if (entries) *entries = E;
    if (buckets) *buckets = B;
    if (infected && I > 0)
        CK(pt_memcpy_sync(s, infected, s->d.infected, (size_t)I * 4, cudaMemcpyDeviceToHost), "copy");
    if (keys) {
        CK(pt_memcpy_sync(s, keys, s->d.keys, (size_t)E * 4, cudaMemcpyDeviceToHost), "copy");
        for (int i = 0; i < E; i++) {
            int h = keys[i] / R, loc = keys[i] % R + lo;
            keys[i] = h * L + loc;
        }
    }
    if (people) CK(pt_memcpy_sync(s, people, s->d.bkt_people, (size_t)E * 4, cudaMemcpyDeviceToHost), "copy");
    if (offsets) {
        std::vector<int32_t> co((size_t)Bc + 1);
        CK(pt_memcpy_sync(s, co.data(), s->d.bkt_offset, ((size_t)Bc + 1) * 4, cudaMemcpyDeviceToHost), "copy");
        for (int h = 0; h < hours; h++)
            for (int loc = 0; loc < L; loc++)
                offsets[(size_t)h * L + loc] = loc < lo ? co[(size_t)h * R] : co[(size_t)h * R + loc - lo];
        offsets[B] = E;
    }
    return PT_OK;
}

pt_status pt_set_interventions(pt_sim *s, const pt_interventions *iv)
{
    if (!s || !iv) return PT_ERR_ARG;
    return engine_set_interventions(s, 0, *iv);
}

pt_status pt_set_full_tables(pt_sim *s, int enabled)
{
    if (!s) return PT_ERR_ARG;
    const bool v = enabled != 0;
    if (v != s->full_tables && s->run_graph) {
        // the captured day loop bakes this choice in; capture again on the next run
        cudaGraphExecDestroy(s->run_graph);
        s->run_graph = nullptr;
    }
    s->full_tables = v;
    return PT_OK;
}

pt_status pt_set_timing(pt_sim *s, int enabled)
{
    if (!s) return PT_ERR_ARG;
    return engine_set_timing(s, enabled);
}

pt_status pt_set_tuning(pt_sim *s, const pt_tuning *t)
{
    if (!s || !t) return PT_ERR_ARG;
    return engine_set_tuning(s, t);
}

pt_status pt_get_tuning(const pt_sim *s, pt_tuning *t)
{
    if (!s || !t) return PT_ERR_ARG;
    *t = to_public(s->d.tune);
    return PT_OK;
}

pt_status pt_autotune(pt_sim *s, int days, pt_tuning *chosen)
{
    if (!s) return PT_ERR_ARG;
    return engine_autotune(s, days, chosen);
}

pt_status pt_get_stage_ms(pt_sim *s, float ms[16], int days[2])
{
    if (!s || !ms) return PT_ERR_ARG;
    return engine_stage_ms(s, ms, days);
}

pt_status pt_get_day_stage_ms(pt_sim *s, int day, float ms[8])
{
    if (!s || !ms || day < 0 || day >= ptk::kMaxDays) return PT_ERR_ARG;
    accumulate_timing(s);
    for (int k = 0; k < kStages; k++)
        ms[k] = s->day_stage_ms.empty() ? 0.f : s->day_stage_ms[(size_t)day * kStages + k];
    return PT_OK;
}

uint64_t pt_launch_count(void) { return ptk::launches(); }

pt_status pt_transfer_bytes(const pt_sim *s, uint64_t *h2d, uint64_t *d2h)
{
    if (!s) return PT_ERR_ARG;
    if (h2d) *h2d = s->h2d_bytes;
    if (d2h) *d2h = s->d2h_bytes;
    return PT_OK;
}

pt_status pt_selftest_bounded_wait(int publish_predecessor, int64_t spin_limit, uint32_t *prefix)
{
    if (spin_limit < 0 || spin_limit > ptk::max_spin_limit()) {
        g_create_error = "spin_limit outside [0, the simulation's own limit]";
        return PT_ERR_ARG;
    }
    // two look-back words, the error word and the returned prefix, all zero
    void *mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, 64);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc(probe)");
    unsigned long long *tiles = (unsigned long long *)mem;
    int *error = (int *)(tiles + 2);
    unsigned *out = (unsigned *)(error + 1);
    int h_error = 0;
    unsigned h_prefix = 0;
    e = cudaMemset(mem, 0, 64);
    if (e == cudaSuccess) e = ptk::launch_wait_probe(tiles, error, publish_predecessor ? 1 : 0, spin_limit, out, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(&h_error, error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&h_prefix, out, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "bounded-wait probe");
    if (prefix) *prefix = h_prefix;
    if (h_error) {
        g_create_error = "a device-side wait gave up (bounded-wait probe)";
        return PT_ERR_TIMEOUT;
    }
    return PT_OK;
}

pt_status pt_selftest_errand_lookup(uint64_t counts[4])
{
    if (!counts) return PT_ERR_ARG;
    unsigned long long *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc(errand self-test)");
    unsigned long long h[4] = {0, 0, 0, 0};
    e = cudaMemset(d, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = ptk::launch_errand_selftest(d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "errand self-test");
    for (int i = 0; i < 4; i++) counts[i] = h[i];
    return PT_OK;
}

pt_status pt_trim_device_memory(void)
{
    cudaMemPool_t pool = nullptr;
    cudaError_t e = engine_pool(&pool);
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "trim device memory");
    return PT_OK;
}

void pt_destroy(pt_sim *s) { delete s; }

const char *pt_last_error(const pt_sim *s)
{
    if (!s) return g_create_error.c_str();
    return s->err.c_str();
}

// ------------------------------------------------------------------ batches
pt_status pt_batch_create(const pt_params *params, const int *core_seeds, int instances, void *cuda_stream,
                          pt_batch **out)
{
    if (!params || !core_seeds || !out) return fail(nullptr, PT_ERR_ARG, "null argument");
    *out = nullptr;
    if (instances < 1 || instances > PT_BATCH_MAX_INSTANCES)
        return fail(nullptr, PT_ERR_ARG, "instances must be in 1.." + std::to_string(PT_BATCH_MAX_INSTANCES));
    std::unique_ptr<pt_batch> b(new pt_batch());
    pt_status st = engine_create(b.get(), params, core_seeds, instances, cuda_stream);
    if (st != PT_OK) return st;
    *out = b.release();
    return PT_OK;
}

pt_status pt_batch_setup(pt_batch *b)
{
    if (!b) return PT_ERR_ARG;
    return engine_setup(b);
}

pt_status pt_batch_run(pt_batch *b)
{
    if (!b) return PT_ERR_ARG;
    return engine_run(b);
}

pt_status pt_batch_step_day(pt_batch *b, int *running)
{
    if (!b) return PT_ERR_ARG;
    return engine_step(b, running);
}

pt_status pt_batch_reset_epidemic(pt_batch *b)
{
    if (!b) return PT_ERR_ARG;
    if (!b->setup_done) return fail(b, PT_ERR_STATE, "reset before setup");
    return engine_reset(b);
}

pt_status pt_batch_set_interventions(pt_batch *b, const pt_interventions *iv)
{
    if (!b || !iv) return PT_ERR_ARG;
    for (int k = 0; k < b->K(); k++)
        if (const char *why = check_interventions(iv[k]))
            return fail(b, PT_ERR_ARG, "instance " + std::to_string(k) + ": " + why);
    for (int k = 0; k < b->K(); k++) {
        pt_status st = engine_set_interventions(b, k, iv[k]);
        if (st != PT_OK) return st;
    }
    return PT_OK;
}

pt_status pt_batch_size(const pt_batch *b, int *instances, int64_t *persons, int64_t *padded_persons)
{
    if (!b) return PT_ERR_ARG;
    if (instances) *instances = b->K();
    if (persons) *persons = b->persons;
    if (padded_persons) *padded_persons = b->setup_done ? b->d.P : 0;
    return PT_OK;
}

static bool bad_instance(const pt_batch *b, int k) { return !b || k < 0 || k >= b->K(); }

pt_status pt_batch_counts(const pt_batch *b, int k, int *counts, int *infected, int *days_run)
{
    if (bad_instance(b, k)) return PT_ERR_ARG;
    const Instance &in = b->inst[k];
    if (counts) std::memcpy(counts, in.counts.data(), (size_t)in.days_run * 16 * sizeof(int));
    if (infected) std::memcpy(infected, in.infected.data(), (size_t)in.days_run * sizeof(int));
    if (days_run) *days_run = in.days_run;
    return PT_OK;
}

pt_status pt_batch_final_gen_counts(pt_batch *b, int *gen_p, int *gen_s)
{
    if (!b || !gen_p || !gen_s) return PT_ERR_ARG;
    return engine_gen_counts(b, gen_p, gen_s);
}

pt_status pt_batch_get_info(const pt_batch *b, int k, pt_info *out)
{
    if (bad_instance(b, k) || !out) return PT_ERR_ARG;
    return engine_info(b, k, out);
}

pt_status pt_batch_get_person_state(pt_batch *b, int k, uint8_t *status_p, uint8_t *status_s, uint8_t *day_p,
                                    uint8_t *day_s, uint8_t *gen_p, uint8_t *gen_s, uint8_t *age)
{
    if (bad_instance(b, k)) return PT_ERR_ARG;
    return engine_person_state(b, k, status_p, status_s, day_p, day_s, gen_p, gen_s, age);
}

pt_status pt_batch_get_population(pt_batch *b, int k, int32_t *household, int32_t *household_offset,
                                  int32_t *workplace, int32_t *workplace_people, int32_t *workplace_offset)
{
    if (bad_instance(b, k)) return PT_ERR_ARG;
    return engine_population(b, k, household, household_offset, workplace, workplace_people, workplace_offset);
}

pt_status pt_batch_set_timing(pt_batch *b, int enabled)
{
    if (!b) return PT_ERR_ARG;
    return engine_set_timing(b, enabled);
}

pt_status pt_batch_set_tuning(pt_batch *b, const pt_tuning *t)
{
    if (!b || !t) return PT_ERR_ARG;
    return engine_set_tuning(b, t);
}

pt_status pt_batch_get_tuning(const pt_batch *b, pt_tuning *t)
{
    if (!b || !t) return PT_ERR_ARG;
    *t = to_public(b->d.tune);
    return PT_OK;
}

pt_status pt_batch_autotune(pt_batch *b, int days, pt_tuning *chosen)
{
    if (!b) return PT_ERR_ARG;
    return engine_autotune(b, days, chosen);
}

pt_status pt_batch_get_stage_ms(pt_batch *b, float ms[16], int days[2])
{
    if (!b || !ms) return PT_ERR_ARG;
    return engine_stage_ms(b, ms, days);
}

pt_status pt_batch_transfer_bytes(const pt_batch *b, uint64_t *h2d, uint64_t *d2h)
{
    if (!b) return PT_ERR_ARG;
    if (h2d) *h2d = b->h2d_bytes;
    if (d2h) *d2h = b->d2h_bytes;
    return PT_OK;
}

void pt_batch_destroy(pt_batch *b) { delete b; }

const char *pt_batch_last_error(const pt_batch *b)
{
    if (!b) return g_create_error.c_str();
    return b->err.c_str();
}

}  // extern "C"
