// pt_sim.cpp - C ABI of the simulation: lifecycle, the PandemicSim host flow
// (setupSim / runToCompletion / doWeekday|doWeekend / final_countReproduction) and
// device-memory ownership.  All device memory of a simulation lives in one arena.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
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

}  // namespace

struct pt_sim {
    pt_params params;
    int core_seed = 0;
    pth::Derived derived;
    std::unique_ptr<pth::GlibcRand> rng;
    std::vector<int32_t> seed_list;
    ptk::SimConst c;
    ptk::DevArrays d;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    char *setup_mem = nullptr;      // household types/sizes during setup
    char *small_mem = nullptr;      // scalars, look-back words, histogram, household offsets
    size_t small_bytes = 0;
    char *arena_mem = nullptr;
    size_t arena_bytes = 0;
    int32_t *d_seeds = nullptr;
    int *d_hist = nullptr;
    int adults = 0;
    bool setup_done = false;
    int day = 0;                    // next day to run
    bool stopped = false;           // a day counted zero infected
    int days_run = 0;
    std::string err;
    bool timing = false;
    bool full_tables = false;             // materialise every bucket (tables complete for inspection)
    std::vector<cudaEvent_t> day_events;  // kMaxDays x (stages + 1), created on demand
    std::vector<int> timed_days;
    float stage_ms[16] = {0};             // [weekday stages 0..7, weekend stages 8..15]
    int stage_days[2] = {0, 0};
    // per-day results mirrored on the host
    std::vector<int> counts;        // kMaxDays * 16
    std::vector<int> infected;      // kMaxDays
    float max_prop = 0.f;
    int max_prop_day = 0;
    mutable uint64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device copies issued
    // The whole day loop (days 0..max_days-1) captured once and replayed by pt_run.
    // Every per-day decision (early stop, counters, offsets) reads device scalars,
    // so the same graph serves every run after pt_reset_epidemic.
    cudaGraphExec_t run_graph = nullptr;
    uint64_t graph_kernels = 0;
};

// Every host<->device copy of the library goes through these, so the bytes a call
// moves across PCIe/C2C can be reported (pt_transfer_bytes).
static cudaError_t pt_memcpy(const pt_sim *s, void *dst, const void *src, size_t n, cudaMemcpyKind k,
                             cudaStream_t st)
{
    if (k == cudaMemcpyHostToDevice) s->h2d_bytes += n;
    else if (k == cudaMemcpyDeviceToHost) s->d2h_bytes += n;
    return cudaMemcpyAsync(dst, src, n, k, st);
}

static cudaError_t pt_memcpy_sync(const pt_sim *s, void *dst, const void *src, size_t n, cudaMemcpyKind k)
{
    cudaError_t e = pt_memcpy(s, dst, src, n, k, s->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s->stream);
}

static pt_status fail(pt_sim *s, pt_status st, const std::string &msg)
{
    if (s) s->err = msg;
    else g_create_error = msg;
    return st;
}

static pt_status cuda_fail(pt_sim *s, cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(s, e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA, m);
}

#define CK(expr, where)                                   \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_fail(s, _e, where); \
    } while (0)

extern "C" {

pt_status pt_create(const pt_params *params, int core_seed, void *cuda_stream, pt_sim **out)
{
    if (!params || !out) return fail(nullptr, PT_ERR_ARG, "null argument");
    *out = nullptr;
    std::unique_ptr<pt_sim> s(new pt_sim());
    s->params = *params;
    s->core_seed = core_seed;
    s->rng.reset(new pth::GlibcRand((unsigned int)core_seed));
    const char *why = nullptr;
    pt_status st = pth::derive(*params, core_seed, s->derived, *s->rng, &why);
    if (st != PT_OK) return fail(nullptr, st, why ? why : "invalid parameters");
    ptk::SimConst &c = s->c;
    std::memset(&c, 0, sizeof(c));
    c.H = s->derived.households;
    c.L = s->derived.workplaces;
    for (int t = 0; t < 14; t++) {
        c.type_count[t] = s->derived.type_count[t];
        c.type_offset[t] = s->derived.type_offset[t];
    }
    std::memcpy(c.shedding, s->derived.shedding, sizeof(c.shedding));
    c.infectiousness[0] = s->derived.infectiousness[0];
    c.infectiousness[1] = s->derived.infectiousness[1];
    c.pct_sympt = params->percent_symptomatic;
    c.key0 = s->derived.key0;
    c.key1 = s->derived.key1;
    if ((long long)c.L * 10 + 1 > 0x7FFFFFFFll) return fail(nullptr, PT_ERR_ARG, "too many locations");
    // The CUDA stream and events are created by pt_setup, so parameters, seeds and
    // scaling can be inspected without a device.
    s->stream = (cudaStream_t)cuda_stream;
    s->counts.assign(ptk::kMaxDays * 16, 0);
    s->infected.assign(ptk::kMaxDays, 0);
    *out = s.release();
    return PT_OK;
}

static pt_status reset_epidemic(pt_sim *s)
{
    const int N = s->c.N;
    ptk::DevArrays &d = s->d;
    CK(ptk::launch_init_status(N, d.state, d.gen_p, d.gen_s, d.claim, s->stream), "init_status");
    const int P = s->params.initial_pandemic, S = s->params.initial_seasonal;
    if (P + S > 0) {
        CK(pt_memcpy(s, s->d_seeds, s->seed_list.data(), sizeof(int32_t) * (P + S), cudaMemcpyHostToDevice,
                           s->stream), "seed copy");
        CK(ptk::launch_seed_infected(s->d_seeds, P, S, d.state, d.gen_p, d.gen_s, s->stream), "seed");
    }
    ptk::Scalars z;
    std::memset(&z, 0, sizeof(z));
    // rand_offset after setup: H/4 (household types) + N/4 (workplaces)
    z.rand_offset = (unsigned long long)(s->c.H / 4) + (unsigned long long)(N / 4);
    z.adults = s->adults;
    CK(pt_memcpy(s, d.sc, &z, sizeof(z), cudaMemcpyHostToDevice, s->stream), "scalars");
    CK(cudaStreamSynchronize(s->stream), "reset sync");
    s->day = 0;
    s->stopped = false;
    s->days_run = 0;
    s->max_prop = 0.f;
    s->max_prop_day = 0;
    std::fill(s->counts.begin(), s->counts.end(), 0);
    std::fill(s->infected.begin(), s->infected.end(), 0);
    return PT_OK;
}

pt_status pt_setup(pt_sim *s)
{
    if (!s) return PT_ERR_ARG;
    if (s->setup_done) return fail(s, PT_ERR_STATE, "pt_setup called twice");
    if (!s->stream) {
        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        s->own_stream = true;
    }
    ptk::SimConst &c = s->c;
    const int H = c.H, L = c.L;
    const long long maxN = 5ll * H;  // the largest household type holds 5 persons
    const long long tiles_cap = std::max({maxN, 10ll * L + 1, (long long)H + 1}) / 4096 + 4;

    // persistent small block: scalars, look-back tiles and control words, the
    // generation histogram and the household offsets (H+1)
    size_t small_bytes = round256(sizeof(ptk::Scalars)) + round256((tiles_cap + 4) * sizeof(unsigned long long)) +
                         round256(512 * sizeof(int)) + round256(((size_t)H + 1) * 4);
    CK(cudaMalloc(&s->small_mem, small_bytes), "cudaMalloc(small)");
    Arena a0{s->small_mem, small_bytes, 0};
    ptk::DevArrays &d = s->d;
    d.sc = a0.take<ptk::Scalars>(1);
    d.tiles = a0.take<unsigned long long>(tiles_cap + 4);
    d.tiles_cap = (int)tiles_cap;
    s->d_hist = a0.take<int>(512);
    d.hh_offset = a0.take<int32_t>((size_t)H + 1);
    s->small_bytes = small_bytes;
    // setup-only block: household types and sizes
    size_t setup_bytes = round256((size_t)H) + round256((size_t)H * 4);
    CK(cudaMalloc(&s->setup_mem, setup_bytes), "cudaMalloc(setup)");
    Arena a1{s->setup_mem, setup_bytes, 0};
    uint8_t *types = a1.take<uint8_t>(H);
    int32_t *sizes = a1.take<int32_t>(H);
    CK(cudaMemsetAsync(d.sc, 0, sizeof(ptk::Scalars), s->stream), "memset scalars");
    CK(cudaMemsetAsync(d.tiles, 0, (tiles_cap + 4) * sizeof(unsigned long long), s->stream), "memset tiles");
    int *ctl = (int *)(d.tiles + tiles_cap);

    // households: types and sizes, exclusive scan -> offsets and N
    CK(ptk::launch_household_types(c, types, sizes, &d.sc->adults, s->stream), "household_types");
    CK(ptk::launch_scan_exclusive(sizes, d.hh_offset, H, 0, d.tiles, ctl, &d.sc->error, nullptr, 0, nullptr,
                                  s->stream), "household scan");
    int hN = 0, hA = 0;
    CK(pt_memcpy(s, &hN, d.hh_offset + H, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "N copy");
    CK(pt_memcpy(s, &hA, &d.sc->adults, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "adults copy");
    CK(cudaStreamSynchronize(s->stream), "setup sync");
    if (hN <= 0) return fail(s, PT_ERR_STATE, "population is empty");
    const int N = hN;
    c.N = N;
    s->adults = hA;
    c.workplace_offset = (uint64_t)(H / 4);
    const int P = s->params.initial_pandemic, S = s->params.initial_seasonal;
    if ((long long)P + S > N) return fail(s, PT_ERR_ARG, "more initial infected than persons");

    if ((long long)N * 3 >= (1ll << 30)) return fail(s, PT_ERR_ARG, "population too large (3N must stay below 2^30)");

    // arena of per-person and per-location arrays
    const size_t n = (size_t)N, B = 10 * (size_t)L;
    const size_t radix_tiles = (3 * n + 4095) / 4096 + 1;
    size_t bytes = 0;
    bytes += round256(n * 4);                 // state
    bytes += 3 * round256(n);                 // gen_p, gen_s, age
    bytes += round256(n * 4) * 3;             // household, workplace, wp_people
    bytes += round256(((size_t)L + 1) * 4);   // wp_offset
    bytes += round256(3 * n * 4) * 6;         // keys, bkt_people, radix k0/v0/k1/v1
    bytes += round256((B + 1) * 4);           // bkt_offset
    bytes += round256(B * 4);                 // bkt_count
    bytes += round256(radix_tiles * 256 * 8); // radix look-back words
    bytes += round256(8 * 4) + 2 * round256(4 * 256 * 4);  // radix ctl, digit hist/base
    bytes += round256((B / 32 + 1) * 4);      // bucket mark bitmap
    bytes += round256(n * 4);                 // infected
    bytes += round256(2 * n * 8);             // claim
    bytes += round256(2 * n * 4);             // new_list
    bytes += round256((size_t)(P + S + 1) * 4);  // seeds
    CK(cudaMalloc(&s->arena_mem, bytes), "cudaMalloc(arena)");
    s->arena_bytes = bytes;
    Arena a{s->arena_mem, bytes, 0};
    d.state = a.take<uint32_t>(n);
    d.gen_p = a.take<uint8_t>(n);
    d.gen_s = a.take<uint8_t>(n);
    d.age = a.take<uint8_t>(n);
    d.household = a.take<int32_t>(n);
    d.workplace = a.take<int32_t>(n);
    d.wp_people = a.take<int32_t>(n);
    d.wp_offset = a.take<int32_t>((size_t)L + 1);
    d.keys = a.take<int32_t>(3 * n);
    d.bkt_people = a.take<int32_t>(3 * n);
    d.rk0 = a.take<uint32_t>(3 * n);
    d.rv0 = a.take<uint32_t>(3 * n);
    d.rk1 = a.take<uint32_t>(3 * n);
    d.rv1 = a.take<uint32_t>(3 * n);
    d.bkt_offset = a.take<int32_t>(B + 1);
    d.bkt_count = a.take<int32_t>(B);
    d.radix_status = a.take<unsigned long long>(radix_tiles * 256);
    d.radix_ctl = a.take<int>(8);
    d.digit_hist = a.take<int>(4 * 256);
    d.digit_base = a.take<int>(4 * 256);
    d.mark = a.take<uint32_t>(B / 32 + 1);
    d.infected = a.take<int32_t>(n);
    d.claim = a.take<unsigned long long>(2 * n);
    d.new_list = a.take<int32_t>(2 * n);
    s->d_seeds = a.take<int32_t>((size_t)(P + S + 1));
    CK(cudaMemsetAsync(d.bkt_count, 0, B * 4, s->stream), "memset counts");
    CK(cudaMemsetAsync(d.radix_ctl, 0, 8 * 4, s->stream), "memset radix ctl");
    CK(cudaMemsetAsync(d.radix_status, 0, radix_tiles * 256 * 8, s->stream), "memset radix words");
    CK(cudaMemsetAsync(d.digit_hist, 0, 4 * 256 * 4, s->stream), "memset digit hist");

    // households -> persons, then workplaces and schools (setup_assignWorkplaces)
    CK(ptk::launch_generate_households(c, types, d.hh_offset, d.household, d.age, s->stream), "households");
    CK(ptk::launch_assign_workplaces(c, d.age, d.workplace, s->stream), "workplaces");
    // workplace table: person ids stably sorted by workplace, with offsets
    // (setup_assignWorkplaces' radix sort + lower_bound, PandemicSim.cu:3835-3862)
    {
        ptk::RadixArgs r;
        r.keys = (const uint32_t *)d.workplace;
        r.E = N;
        r.buckets = L;
        r.N = N;
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
    // initial infected: rand() % N draws continue the seed sequence (PandemicSim.cu:708-758)
    s->seed_list = pth::unique_numbers(*s->rng, P + S, N);
    int derr = 0;
    CK(pt_memcpy(s, &derr, &d.sc->error, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "error flag");
    CK(cudaStreamSynchronize(s->stream), "setup sync");
    cudaFree(s->setup_mem);
    s->setup_mem = nullptr;
    if (derr) return fail(s, PT_ERR_TIMEOUT, "a device-side wait gave up during setup");
    pt_status st = reset_epidemic(s);
    if (st != PT_OK) return st;
    s->setup_done = true;
    return PT_OK;
}

pt_status pt_reset_epidemic(pt_sim *s)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_reset_epidemic before pt_setup");
    return reset_epidemic(s);
}

// Stage boundaries recorded per day when timing is on.
enum { kStSweep, kStSchedule, kStScan, kStRadix, kStInfect, kStApply, kStages };

static cudaEvent_t stage_event(pt_sim *s, int day, int k)
{
    return s->day_events[(size_t)day * (kStages + 1) + k];
}

// Enqueues one day: sweep, schedule, bucket build (scan, radix sort), infection,
// apply.  Every kernel after the sweep skips itself on the device when the day
// counted no infected.
static pt_status enqueue_day(pt_sim *s, int day)
{
    const bool weekend = (day % 7) >= 5;  // PandemicSim.h:283-284
    const ptk::SimConst &c = s->c;
    const ptk::DevArrays &d = s->d;
    cudaStream_t st = s->stream;
    const bool t = s->timing;
    if (t) cudaEventRecord(stage_event(s, day, 0), st);
    CK(ptk::launch_sweep(c, d, day, st), "sweep");
    if (t) cudaEventRecord(stage_event(s, day, 1), st);
    CK(ptk::launch_schedule(c, d, weekend, s->full_tables, st), "schedule");
    if (t) cudaEventRecord(stage_event(s, day, 2), st);
    CK(ptk::launch_bucket_scan(c, d, weekend, st), "bucket scan");
    if (t) cudaEventRecord(stage_event(s, day, 3), st);
    CK(ptk::launch_bucket_sort(c, d, weekend, st), "bucket sort");
    if (t) cudaEventRecord(stage_event(s, day, 4), st);
    CK(ptk::launch_infect(c, d, weekend, day, st), "infect");
    if (t) cudaEventRecord(stage_event(s, day, 5), st);
    CK(ptk::launch_apply(d, day, st), "apply");
    if (t) cudaEventRecord(stage_event(s, day, 6), st);
    if (t) s->timed_days.push_back(day);
    return PT_OK;
}

static void accumulate_timing(pt_sim *s)
{
    if (!s->timing) return;
    cudaStreamSynchronize(s->stream);
    for (int day : s->timed_days) {
        const bool weekend = (day % 7) >= 5;
        for (int k = 0; k < kStages; k++) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, stage_event(s, day, k), stage_event(s, day, k + 1)) == cudaSuccess)
                s->stage_ms[(weekend ? 8 : 0) + k] += ms;
        }
        s->stage_days[weekend ? 1 : 0]++;
    }
    s->timed_days.clear();
}

static pt_status check_device_error(pt_sim *s)
{
    int e = 0;
    CK(pt_memcpy(s, &e, &s->d.sc->error, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "error flag");
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (e) return fail(s, PT_ERR_TIMEOUT, "a device-side wait gave up (look-back ordering)");
    return PT_OK;
}

static void track_peak(pt_sim *s, int day, int I)
{
    // PandemicSim.cu:923-931: strictly greater proportions only
    float prop = (float)I / (float)s->c.N;
    if (prop > s->max_prop) {
        s->max_prop = prop;
        s->max_prop_day = day;
    }
}

pt_status pt_step_day(pt_sim *s, int counts16[16], int *infected_count)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_step_day before pt_setup");
    if (s->stopped) return PT_DONE;
    if (s->day >= s->params.max_days) return PT_FINISHED;
    const int day = s->day;
    pt_status st = enqueue_day(s, day);
    if (st != PT_OK) return st;
    int buf[17];
    CK(pt_memcpy(s, buf, s->d.sc->counts[day], 16 * sizeof(int), cudaMemcpyDeviceToHost, s->stream), "counts");
    CK(pt_memcpy(s, buf + 16, &s->d.sc->infected_per_day[day], sizeof(int), cudaMemcpyDeviceToHost, s->stream),
       "infected");
    st = check_device_error(s);
    if (st != PT_OK) return st;
    accumulate_timing(s);
    std::memcpy(&s->counts[day * 16], buf, 16 * sizeof(int));
    s->infected[day] = buf[16];
    if (counts16) std::memcpy(counts16, buf, 16 * sizeof(int));
    if (infected_count) *infected_count = buf[16];
    s->days_run = day + 1;
    if (buf[16] == 0) {
        s->stopped = true;
        return PT_DONE;
    }
    track_peak(s, day, buf[16]);
    s->day = day + 1;
    return PT_OK;
}

pt_status pt_run(pt_sim *s, int *counts, int *infected, int *days_run)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_run before pt_setup");
    const int first = s->day, M = s->params.max_days;
    if (!s->stopped) {
        if (first == 0 && !s->timing && M > 0) {
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
    }
    // one copy of all per-day results
    std::vector<int> hc(ptk::kMaxDays * 16), hi(ptk::kMaxDays);
    int rows = 0;
    CK(pt_memcpy(s, hc.data(), s->d.sc->counts, hc.size() * sizeof(int), cudaMemcpyDeviceToHost, s->stream),
       "counts");
    CK(pt_memcpy(s, hi.data(), s->d.sc->infected_per_day, hi.size() * sizeof(int), cudaMemcpyDeviceToHost,
                       s->stream), "infected");
    CK(pt_memcpy(s, &rows, &s->d.sc->days_run, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "rows");
    pt_status st = check_device_error(s);
    if (st != PT_OK) return st;
    accumulate_timing(s);
    if (!s->stopped) {
        for (int day = first; day < rows; day++) {
            std::memcpy(&s->counts[day * 16], &hc[day * 16], 16 * sizeof(int));
            s->infected[day] = hi[day];
            if (hi[day] == 0) {
                s->stopped = true;
                break;
            }
            track_peak(s, day, hi[day]);
        }
        s->days_run = rows;
        s->day = s->stopped ? rows - 1 : rows;
    }
    if (counts) std::memcpy(counts, s->counts.data(), (size_t)s->days_run * 16 * sizeof(int));
    if (infected) std::memcpy(infected, s->infected.data(), (size_t)s->days_run * sizeof(int));
    if (days_run) *days_run = s->days_run;
    return PT_OK;
}

pt_status pt_final_gen_counts(pt_sim *s, int gen_p[256], int gen_s[256])
{
    if (!s || !gen_p || !gen_s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "pt_final_gen_counts before pt_setup");
    CK(ptk::launch_gen_hist(s->d.gen_p, s->d.gen_s, s->c.N, s->d_hist, s->stream), "gen hist");
    int h[512];
    CK(pt_memcpy(s, h, s->d_hist, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "hist copy");
    CK(cudaStreamSynchronize(s->stream), "sync");
    std::memcpy(gen_p, h, 256 * sizeof(int));
    std::memcpy(gen_s, h + 256, 256 * sizeof(int));
    return PT_OK;
}

pt_status pt_get_info(const pt_sim *s, pt_info *out)
{
    if (!s || !out) return PT_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    out->number_people = s->c.N;
    out->number_households = s->c.H;
    out->number_workplaces = s->c.L;
    out->number_adults = s->adults;
    out->number_children = s->c.N - s->adults;
    out->current_day = s->day;
    out->days_run = s->days_run;
    out->infected_count = s->days_run > 0 ? s->infected[s->days_run - 1] : 0;
    for (int i = 0; i < 4; i++) out->seeds[i] = s->derived.seeds[i];
    for (int t = 0; t < 14; t++) {
        out->type_count[t] = s->c.type_count[t];
        out->type_offset[t] = s->c.type_offset[t];
    }
    out->infectiousness[0] = s->c.infectiousness[0];
    out->infectiousness[1] = s->c.infectiousness[1];
    out->max_day_of_peak = s->max_prop_day;
    out->max_infected_proportion = s->max_prop;
    out->sm_count = ptk::sm_count();
    out->device_bytes = s->arena_bytes + s->small_bytes;
    if (s->setup_done) {
        unsigned long long v[2] = {0, 0};
        pt_memcpy_sync(s, v, &s->d.sc->rand_offset, sizeof(v), cudaMemcpyDeviceToHost);
        out->rand_offset = v[0];
        out->bucket_entries_materialised = v[1];
        uint64_t total = 0;
        for (int day = 0; day < s->days_run; day++)
            if (s->infected[day] > 0) total += (uint64_t)((day % 7) >= 5 ? 3 : 2) * (uint64_t)s->c.N;
        out->bucket_entries_scheduled = total;
    }
    return PT_OK;
}

pt_status pt_get_person_state(pt_sim *s, uint8_t *status_p, uint8_t *status_s, uint8_t *day_p, uint8_t *day_s,
                              uint8_t *gen_p, uint8_t *gen_s, uint8_t *age)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "state before pt_setup");
    const size_t N = (size_t)s->c.N;
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (status_p || status_s || day_p || day_s) {
        std::vector<uint32_t> st(N);
        CK(pt_memcpy_sync(s, st.data(), s->d.state, N * 4, cudaMemcpyDeviceToHost), "state copy");
        for (size_t i = 0; i < N; i++) {
            if (status_p) status_p[i] = (uint8_t)(st[i] & 0xFF);
            if (status_s) status_s[i] = (uint8_t)((st[i] >> 8) & 0xFF);
            if (day_p) day_p[i] = (uint8_t)((st[i] >> 16) & 0xFF);
            if (day_s) day_s[i] = (uint8_t)(st[i] >> 24);
        }
    }
    if (gen_p) CK(pt_memcpy_sync(s, gen_p, s->d.gen_p, N, cudaMemcpyDeviceToHost), "gen copy");
    if (gen_s) CK(pt_memcpy_sync(s, gen_s, s->d.gen_s, N, cudaMemcpyDeviceToHost), "gen copy");
    if (age) CK(pt_memcpy_sync(s, age, s->d.age, N, cudaMemcpyDeviceToHost), "age copy");
    return PT_OK;
}

pt_status pt_get_population(pt_sim *s, int32_t *household, int32_t *household_offset, int32_t *workplace,
                            int32_t *workplace_people, int32_t *workplace_offset)
{
    if (!s) return PT_ERR_ARG;
    if (!s->setup_done) return fail(s, PT_ERR_STATE, "population before pt_setup");
    const size_t N = (size_t)s->c.N;
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (household) CK(pt_memcpy_sync(s, household, s->d.household, N * 4, cudaMemcpyDeviceToHost), "copy");
    if (household_offset)
        CK(pt_memcpy_sync(s, household_offset, s->d.hh_offset, ((size_t)s->c.H + 1) * 4, cudaMemcpyDeviceToHost), "copy");
    if (workplace) CK(pt_memcpy_sync(s, workplace, s->d.workplace, N * 4, cudaMemcpyDeviceToHost), "copy");
    if (workplace_people) CK(pt_memcpy_sync(s, workplace_people, s->d.wp_people, N * 4, cudaMemcpyDeviceToHost), "copy");
    if (workplace_offset)
        CK(pt_memcpy_sync(s, workplace_offset, s->d.wp_offset, ((size_t)s->c.L + 1) * 4, cudaMemcpyDeviceToHost), "copy");
    return PT_OK;
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
    ptk::Scalars sc;
    CK(pt_memcpy_sync(s, &sc, s->d.sc, sizeof(sc), cudaMemcpyDeviceToHost), "scalars");
    const int day = sc.day;
    const bool weekend = (day % 7) >= 5;
    const int L = s->c.L, hours = weekend ? 10 : 2;
    const int lo = s->c.type_offset[weekend ? 9 : 8], R = L - lo;
    const int E = (weekend ? 3 : 2) * s->c.N, B = hours * L;
    const int Bc = ptk::day_buckets(s->c, weekend);
    if (entries) *entries = E;
    if (buckets) *buckets = B;
    if (infected && sc.infected > 0)
        CK(pt_memcpy_sync(s, infected, s->d.infected, (size_t)sc.infected * 4, cudaMemcpyDeviceToHost), "copy");
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
    if (enabled && s->day_events.empty()) {
        s->day_events.resize((size_t)ptk::kMaxDays * (kStages + 1));
        for (auto &e : s->day_events) CK(cudaEventCreate(&e), "cudaEventCreate");
    }
    s->timing = enabled != 0;
    std::memset(s->stage_ms, 0, sizeof(s->stage_ms));
    s->stage_days[0] = s->stage_days[1] = 0;
    return PT_OK;
}

pt_status pt_get_stage_ms(pt_sim *s, float ms[16], int days[2])
{
    if (!s || !ms) return PT_ERR_ARG;
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

uint64_t pt_launch_count(void) { return ptk::launches(); }

pt_status pt_transfer_bytes(const pt_sim *s, uint64_t *h2d, uint64_t *d2h)
{
    if (!s) return PT_ERR_ARG;
    if (h2d) *h2d = s->h2d_bytes;
    if (d2h) *d2h = s->d2h_bytes;
    return PT_OK;
}

void pt_destroy(pt_sim *s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->run_graph) cudaGraphExecDestroy(s->run_graph);
    cudaFree(s->arena_mem);
    cudaFree(s->setup_mem);
    cudaFree(s->small_mem);
    for (auto &e : s->day_events)
        if (e) cudaEventDestroy(e);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

const char *pt_last_error(const pt_sim *s)
{
    if (!s) return g_create_error.c_str();
    return s->err.c_str();
}

}  // extern "C"
