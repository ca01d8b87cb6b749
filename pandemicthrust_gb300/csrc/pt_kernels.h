// pt_kernels.h - kernel launchers and the device data model of the simulation.
// Shared by the CUDA translation unit (pt_kernels.cu) and the host orchestration
// (pt_sim.cpp); no CUDA-specific types beyond cudaStream_t appear here.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ptk {

constexpr int kTypes = 14;
constexpr int kMaxDays = 256;

constexpr int kPersonTile = 4096;  // persons per sweep / schedule tile
constexpr int kRadixTileEntries = 4096;  // entries per radix-pass tile (256 look-back words each)
constexpr int kScanTileEntries = 4096;   // values per scan tile (one look-back word each)
constexpr int kDigitStripes = 16;  // copies of the day's radix digit histograms (spreads the updates)

// Constants of one simulation (setup kernels take them by value; the day kernels
// read them from the InstConst array).
struct SimConst {
    int N, H, L;
    int type_count[kTypes];
    int type_offset[kTypes];
    float shedding[6][10];
    float infectiousness[2];
    float pct_sympt;
    uint64_t key0, key1;           // {(long)SEED[0], (long)SEED[1]}
    uint64_t workplace_offset;     // W0: counter base of the workplace draws
};

// One simulation of a batch and where its rows sit in the batch-wide arrays.  Every
// instance's persons start on a person-tile boundary, so a sweep or schedule tile
// belongs to exactly one instance; the persons up to the next boundary are padding
// (never infected, never counted, in no table).
struct InstConst {
    SimConst c;            // c.N = the instance's persons
    int pbase;             // first global person (a multiple of kPersonTile)
    int pend;              // end of its persons and padding (the next instance's pbase)
    int hbase;             // first global household slot; H + 1 slots, the last one
                           // holds the padding persons
    int lbase;             // first global location
    int bbase[2];          // first global bucket of the weekday / weekend errand tables
    int bcount[2];         // the instance's weekday / weekend buckets; one more global
                           // slot follows them (the end offset of its last bucket)
    int max_days;
    long long kbase;       // first schedule-key slot (3 * pbase)
    // interventions (build-defined extensions; all zero reproduces the reference)
    int closure_start, closure_end;  // school-type locations closed on days [start, end)
    uint64_t absent_thr;             // an adult is absent from work when intervention_hash < this
    uint64_t vacc_thr;               // a person starts vaccinated when intervention_hash < this
};

constexpr uint64_t kTagAbsent = 1, kTagVaccinated = 2;

// Device-resident state of one simulation.  The day loop reads and updates it on
// the device, so a whole run needs no host round trip.
struct InstState {
    unsigned long long rand_offset;     // next free Random123 counter
    unsigned long long errand_offset;   // E0 of the current day's schedule
    unsigned long long infect_offset;   // R0 of the current day's contacts
    int infected;                       // infected count of the current day
    int start;                          // their first position in the batch's infected list
    int list_end;                       // one past their last position
    int marked;                         // today's schedule entries in materialised buckets
    int dense;                          // today's sort reads the schedule keys directly (most
                                        // buckets are read) instead of entries the schedule appended
    int done;                           // set once a day counts zero infected
    int days_run;                       // statistics rows written
    int day;                            // last day run
    int counts[kMaxDays][16];           // per-day status bins
    int infected_per_day[kMaxDays];
};

// Batch-wide device scalars.
struct Scalars {
    unsigned long long materialised_sum;  // schedule entries written to bucket tables, all days
    int infected;                         // length of today's infected list (all instances)
    int done;                             // set once a day finds no instance with infected
    int day;                              // current day index
    int new_count;                        // entries in the new-infection list
    int error;                            // nonzero: a bounded device wait gave up
    int error_site;
    int pad;
};

// Launch shapes chosen at run time (the engine's tuner picks them per engine; every
// choice gives bit-identical results, only the speed differs).
struct Tuning {
    int infect_coop = 0;            // 1: warp-cooperative contacts (8 lanes per infector)
    int infect_blocks_per_sm = 8;   // infection grid: 256-thread blocks per SM (twice as
                                    // many 128-thread blocks for the thread-per-infector kernels)
    int radix_blocks_per_sm = 4;    // persistent blocks of a day's radix pass per SM (1..4)
    int sched_tf = 0;               // schedule kernel's Threefry arithmetic: 0 ALU adds and
                                    // shifts, 1 multiply-add adds, 2 also multiply rotations
    int dense_level = 0;            // when a day's sort reads the schedule keys directly:
                                    // 0 never; 1, 2, 3: infected >= buckets / 4, x 1, x 2
    int radix_threads = 256;        // threads per block of a day's radix passes: 256 or 512
};

// Device pointers of a batch of simulations (one simulation is a batch of one).
// Person, household, location and bucket ids are global: an instance's ids are its
// local ids plus its bases.
struct DevArrays {
    uint32_t *state;          // P: status_p | status_s<<8 | day_p<<16 | day_s<<24
    uint8_t *gen_p, *gen_s;   // P
    uint8_t *age;             // P
    int32_t *household;       // P
    int32_t *hh_offset;       // household slots + 1
    int32_t *workplace;       // P
    int32_t *wp_people;       // P (padding persons last, in the spare bucket)
    int32_t *wp_offset;       // locations + 2
    uint4 *prec;              // P packed per-person records for the contact draws (see PersonRec)
    int32_t *keys;            // 3P schedule keys (global bucket indices)
    int32_t *bkt_offset;      // buckets (each instance's buckets and its end slot)
    int32_t *bkt_count;       // buckets histogram, zero between uses
    int32_t *bkt_people;      // 3P person ids bucket by bucket, ascending in each
    uint32_t *rk0, *rv0, *rk1, *rv1;  // 3P each: radix ping-pong keys/values
    unsigned long long *radix_status;  // ceil(3P/4096) x 256 epoch-tagged look-back words
    int *radix_ctl;           // ticket, finished
    int *digit_hist;          // K x kDigitStripes x 4 x 256 (the first 4 x 256 also serve the setup sorts)
    int *digit_base;          // K x 4 x 256
    int32_t *tile_prefix;     // K + 1: radix tiles of the instances' segments
    int32_t *tile_prefix0;    // K + 1: the same for the first pass (a dense segment's input is all its keys)
    uint32_t *mark;           // bitmap over today's buckets: 1 = materialise
    int32_t *infected;        // P ascending infected ids
    int32_t *infected_inst;   // P: instance of each infected list position
    uint16_t *sweep_flags;    // P / 16: the sweep's per-thread infected masks
    int32_t *sweep_tiles;     // P / kPersonTile + 1: infected per person tile, then their prefix
    unsigned long long *claim;// 2P (victim, strain) -> min attempt key
    int32_t *new_list;        // 2P first claims of the day
    unsigned long long *tiles;// look-back tile status words
    int tiles_cap;
    const InstConst *ic;      // K
    InstState *is;            // K
    const int32_t *tile_inst; // P / kPersonTile: instance of each person tile
    int K;
    int P;                    // persons including padding, a multiple of kPersonTile
    int buckets[2];           // weekday / weekend bucket slots over all instances
    int bucket_max[2];        // largest weekday / weekend bucket count of one instance
    int locations;            // locations over all instances
    Scalars *sc;
    Tuning tune;
};

// The static part of a person that the contact draws read, packed in 16 bytes so an
// infector's own data is one 128-bit load (built once at setup, after the workplace
// table):
//   x  first person of the person's household (household victims are x + r % size)
//   y  start of the person's workplace / school in the workplace table
//   z  persons in that workplace / school
//   w  bits 0-3 household size, 4-7 age code, 8-9 workplace contacts (the type's
//      maximum, PandemicSim.cu:3492-3511), bit 10 the location is a school (types 3-7)
// Padding persons have an all-zero record (they are never infected).
__host__ __device__ inline int prec_household_size(uint32_t w) { return (int)(w & 15u); }
__host__ __device__ inline int prec_age(uint32_t w) { return (int)((w >> 4) & 15u); }
__host__ __device__ inline int prec_desired(uint32_t w) { return (int)((w >> 8) & 3u); }
__host__ __device__ inline bool prec_school(uint32_t w) { return ((w >> 10) & 1u) != 0; }

// Launch configuration helpers
int sm_count();

// ---- setup
cudaError_t launch_household_types(const SimConst &c, uint8_t *types, int32_t *sizes, int *adults,
                                   int *persons, cudaStream_t s);
cudaError_t launch_scan_exclusive(const int32_t *in, int32_t *out, int n, int clear_in,
                                  unsigned long long *tiles, int *ctl, int *error,
                                  const int *skip, int passes, int *digit_hist, cudaStream_t s,
                                  const uint32_t *mark = nullptr, int *total_out = nullptr,
                                  unsigned long long *total_accum = nullptr);
cudaError_t launch_generate_households(const uint8_t *types, const int32_t *hh_offset, int slots,
                                       int32_t *household, uint8_t *age, cudaStream_t s);
cudaError_t launch_assign_workplaces(const SimConst &c, uint8_t *age, int32_t *workplace, int loc_base,
                                     cudaStream_t s);
// household slots of the padding persons, and the padding persons themselves
cudaError_t launch_batch_padding(const DevArrays &d, uint8_t *types, int32_t *sizes, int spare_location,
                                 bool persons, cudaStream_t s);
cudaError_t launch_count_keys(const int32_t *keys, int n, int32_t *count, cudaStream_t s);

// Segments of a day's sort: segment k (instance k) holds its entries at
// [ic[k].kbase, ic[k].kbase + is[k].marked), keys local to the instance, sorted within
// the segment; its tiles are [tile_prefix[k], tile_prefix[k + 1]).  tile_prefix ==
// nullptr: one segment [0, E).
struct RadixSegments {
    const int *tile_prefix = nullptr;   // segments + 1, on the device
    const InstConst *ic = nullptr;
    const InstState *is = nullptr;
    int segments = 0;
    // The day's sort: in its first pass a segment whose instance is dense today reads
    // its entries straight from the schedule keys (global bucket ids at
    // day_keys[kbase ...], 2N weekday hour-major / 3N weekend person-major, persons
    // implicit), keeping those of marked buckets; the other segments read the
    // entries the schedule appended.  tile_prefix0 numbers the first pass's tiles.
    const int32_t *day_keys = nullptr;
    const int *tile_prefix0 = nullptr;
    const uint32_t *mark = nullptr;
    int weekend = 0;
};

// Stable LSD radix sort of E keys in [0, buckets) with implicit person values
// (person_mode 0: entry i is person i; 1: weekday hour-major; 2: weekend 3 per person).
struct RadixArgs {
    const uint32_t *keys;
    int E, buckets, N, person_mode;
    const uint32_t *vals = nullptr;   // explicit input values (nullptr: implicit)
    const uint32_t *mark = nullptr;   // optional bucket filter of the first pass
    const int *count_dev = nullptr;   // entry count after the filter (device)
    uint32_t *k0, *v0, *k1, *v1, *out;
    bool keep_keys = false;       // the last pass also writes the sorted keys (to k0 / k1 by pass parity)
    const int *digit_base;        // [segment][pass][256]
    RadixSegments seg;
    unsigned long long *status;   // look-back words, ceil(E/4096) x 256, epoch-tagged
    int *ctl;                     // ticket, finished, epoch
    int *error;
    const int *skip;
    int blocks_per_sm = 3;        // persistent blocks per SM (1..4; 4 only for 256 threads)
    int threads = 256;            // threads per block of the explicit-value passes: 256 (16 entries
                                  // each, up to 4 blocks per SM) or 512 (8 each, up to 2 blocks)
};
int radix_passes(int buckets);
cudaError_t launch_radix_sort(const RadixArgs &r, cudaStream_t s);
// count (optional) + scan + digit bases + radix passes: a complete bucket table
cudaError_t launch_bucket_table(const RadixArgs &r, int32_t *counts, bool count_keys, int32_t *offset,
                                unsigned long long *tiles, int *lb_ctl, int *digit_hist, cudaStream_t s);
cudaError_t launch_init_status(int N, uint32_t *state, uint8_t *gen_p, uint8_t *gen_s,
                               unsigned long long *claim, cudaStream_t s);
// every instance's device state back to "set up, day 0": rand_offset after setup is
// H/4 (household types) + N/4 (workplaces)
cudaError_t launch_reset_instances(const DevArrays &d, cudaStream_t s);
// vaccinated persons start recovered from both strains (only when some instance
// has a vaccination coverage)
cudaError_t launch_vaccinate(const DevArrays &d, cudaStream_t s);
cudaError_t launch_seed_infected(const int32_t *seeds, int P, int S, uint32_t *state, uint8_t *gen_p,
                                 uint8_t *gen_s, cudaStream_t s);
// the packed per-person records (after households, workplaces and the workplace table)
cudaError_t launch_person_records(const DevArrays &d, cudaStream_t s);

// ---- day (every instance of the batch in each launch)
cudaError_t launch_sweep(const DevArrays &d, int day, cudaStream_t s);          // recover, count, scan, bookkeeping
cudaError_t launch_infected_list(const DevArrays &d, cudaStream_t s);           // the ordered infected list
cudaError_t launch_schedule(const DevArrays &d, bool weekend, int day, bool full_tables, cudaStream_t s);
cudaError_t launch_bucket_scan(const DevArrays &d, bool weekend, cudaStream_t s);
cudaError_t launch_bucket_sort(const DevArrays &d, bool weekend, cudaStream_t s);
cudaError_t launch_bucket_offsets(const DevArrays &d, bool weekend, bool full_tables, cudaStream_t s);
cudaError_t launch_infect(const DevArrays &d, bool weekend, int day, cudaStream_t s);
cudaError_t launch_apply(const DevArrays &d, int day, cudaStream_t s);
// weekday / weekend buckets of one instance (compact keys hour * R + dest - lo)
int day_buckets(const SimConst &c, bool weekend);

// ---- final: per-instance generation histograms, K x 512 (pandemic 0..255, seasonal 256..511)
cudaError_t launch_gen_hist(const DevArrays &d, int *hist, cudaStream_t s);

// ---- the bounded look-back wait in isolation (tiles: 2 zeroed words; error: zeroed)
cudaError_t launch_wait_probe(unsigned long long *tiles, int *error, int publish_first, long long spin_limit,
                              unsigned *prefix_out, cudaStream_t s);
// The errand-lookup self-test: counts[4] (zeroed by the caller) receive mismatch counts.
cudaError_t launch_errand_selftest(unsigned long long *counts, cudaStream_t s);
long long max_spin_limit();   // the polls every wait of the simulation allows

uint64_t launches();
void add_launches(int64_t n);  // kernels run by a replayed graph

}  // namespace ptk
