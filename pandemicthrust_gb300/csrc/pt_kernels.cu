// pt_kernels.cu - sm_103a kernels of the PandemicThrust daily simulation step.
//
// Stage map (reference = PandemicThrust/PandemicThrust/PandemicSim.cu):
//   setup   household types/sizes, household scan+scatter, workplace/school draw,
//           workplace buckets                         (setupSim, :146-208)
//   sweep   recover + 16 status bins + ordered infected list, one pass
//           (kernel_countInfectedStatusAndRecover :2097-2192 + copy_if :2207-2224)
//   sched   schedule keys + bucket histogram          (:2972-3022 / :2082-2094)
//   bucket  scan of the histogram (bucket offsets) and a stable LSD radix sort of
//           the (key, person) entries (CUB sort + lower_bound, :1212-1248, :1313-1354)
//   infect  contacts and infection draws; the first attempt in (position, slot)
//           order claims each (victim, strain)        (:3236-3379)
//   apply   winners write status, day, generation     (:3048-3067)
//
// Waits between thread blocks (decoupled look-back) are bounded: after kSpinLimit
// polls the block records an error in Scalars::error and carries on, so a fault in
// the ordering logic surfaces as PT_ERR_TIMEOUT on the host instead of a hang.
#include <cstdio>
#include <climits>
#include <atomic>
#include "pt_kernels.h"
#include "pt_device.cuh"
#include "pt_lookback.cuh"

namespace ptk {

static std::atomic<uint64_t> g_launches{0};
uint64_t launches() { return g_launches.load(); }
void add_launches(int64_t n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
static inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count()
{
    // initialised once, safely when several host threads drive engines
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}

static inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// ================================================================== setup
// kernel_householdTypeAssignment + hh_peopleCount_functor (PandemicSim.cu:2329-2357,
// :3579-3605): counter g -> households 4g..4g+3.  Writes each household's size and
// counts adults and persons.
__global__ void k_household_types(SimConst c, uint8_t *types, int32_t *sizes, int *adults, int *persons)
{
    const TfKey key = make_key(c);
    int local_adults = 0, local_persons = 0;
    const int G = c.H / 4;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t w[4];
        tf2x64(key, (uint64_t)g, w);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int h = 4 * g + i;
            if (h < c.H) {
                int t = fish_household_type(w[i]);
                types[h] = (uint8_t)t;
                sizes[h] = c_hh_adults[t] + c_hh_children[t];
                local_adults += c_hh_adults[t];
                local_persons += c_hh_adults[t] + c_hh_children[t];
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        local_adults += __shfl_xor_sync(0xffffffffu, local_adults, o);
        local_persons += __shfl_xor_sync(0xffffffffu, local_persons, o);
    }
    if ((threadIdx.x & 31) == 0 && local_adults) atomicAdd(adults, local_adults);
    if ((threadIdx.x & 31) == 0 && local_persons) atomicAdd(persons, local_persons);
}

cudaError_t launch_household_types(const SimConst &c, uint8_t *types, int32_t *sizes, int *adults, int *persons,
                                   cudaStream_t s)
{
    int G = c.H / 4 + 1;
    int blocks = std::min(div_up(G, 256), sm_count() * 16);
    k_household_types<<<blocks, 256, 0, s>>>(c, types, sizes, adults, persons);
    count_launch();
    return cudaGetLastError();
}

// Generic exclusive scan (single pass, decoupled look-back): out[i] = sum in[0..i),
// out[n] = total.  With clear_in the input is zeroed after it is read.  With
// passes > 0, in[] is a histogram over keys 0..n-1 and the scan also accumulates,
// for each radix pass p, the histogram of the key's 8-bit digit p weighted by the
// count (digit_hist[p][256]), from which the radix sort takes its digit bases.
constexpr int kScanThreads = 256, kScanItems = 16, kScanTile = kScanThreads * kScanItems;
static_assert(kScanTile == kScanTileEntries, "the host sizes the scan look-back words by kScanTileEntries");
constexpr int kMaxRadixPasses = 4;

__global__ void __launch_bounds__(kScanThreads) k_scan(const int32_t *in, int32_t *out, int n, int clear_in,
                                                       LookBack lb, const int *skip, int passes, int *digit_hist,
                                                       const uint32_t *mark, int *total_out,
                                                       unsigned long long *total_accum)
{
    if (skip && *(volatile const int *)skip) return;
    __shared__ int s_dh[kMaxRadixPasses][256];
    if (passes > 0) {
        for (int i = threadIdx.x; i < kMaxRadixPasses * 256; i += blockDim.x) (&s_dh[0][0])[i] = 0;
    }
    int tile;
    unsigned epoch;
    lookback_begin(lb, tile, epoch);
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        long long i = base + k;
        v[k] = i < n ? in[i] : 0;
        // with a mark filter only marked buckets keep their entries
        if (mark && i < n && !((mark[i >> 5] >> (i & 31)) & 1u)) v[k] = 0;
        sum += v[k];
    }
    if (clear_in) {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            long long i = base + k;
            if (i < n) ((int32_t *)in)[i] = 0;
        }
    }
    if (passes > 0) {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (v[k] > 0) {
                unsigned key = (unsigned)(base + k);
                for (int p = 0; p < passes; p++) atomicAdd(&s_dh[p][(key >> (8 * p)) & 255u], v[k]);
            }
        }
    }
    int total;
    int excl = block_exclusive_scan<kScanThreads, int>(sum, total);
    __shared__ unsigned s_prefix;
    if (threadIdx.x < 32) {
        const unsigned e = lookback_publish_warp(lb, epoch, tile, (unsigned)total);
        if (threadIdx.x == 0) s_prefix = e;
    }
    __syncthreads();
    int run = (int)s_prefix + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (tile == (int)gridDim.x - 1 && threadIdx.x == 0) {
        out[n] = (int)s_prefix + total;
        if (total_out) *total_out = (int)s_prefix + total;
        if (total_accum) *total_accum += (unsigned long long)((int)s_prefix + total);
    }
    if (passes > 0) {
        for (int p = 0; p < passes; p++) {
            int c = s_dh[p][threadIdx.x];
            if (c) atomicAdd(&digit_hist[p * 256 + threadIdx.x], c);
        }
    }
    lookback_end(lb);
}

cudaError_t launch_scan_exclusive(const int32_t *in, int32_t *out, int n, int clear_in,
                                  unsigned long long *tiles, int *ctl, int *error,
                                  const int *skip, int passes, int *digit_hist, cudaStream_t s,
                                  const uint32_t *mark, int *total_out, unsigned long long *total_accum)
{
    int blocks = std::max(1, div_up(n, kScanTile));
    LookBack lb;
    lb.tiles = tiles;
    lb.ctl = ctl;
    lb.error = error;
    k_scan<<<blocks, kScanThreads, 0, s>>>(in, out, n, clear_in, lb, skip, passes, digit_hist, mark, total_out,
                                                           total_accum);
    count_launch();
    return cudaGetLastError();
}

// Exclusive scan of each pass's 256-bin digit histogram -> digit bases; clears the
// histograms for the next sort.
// With stripes > 1 the histograms are split over `stripes` copies of 4 x 256 bins
// (producers spread their updates over the copies); the copies are summed.
__global__ void k_digit_bases(int *digit_hist, int *digit_base, int passes, int stripes, const int *skip)
{
    if (skip && *(volatile const int *)skip) return;
    for (int p = 0; p < passes; p++) {
        int v = 0;
        for (int st = 0; st < stripes; st++) {
            int *h = &digit_hist[(st * kMaxRadixPasses + p) * 256 + threadIdx.x];
            v += *h;
            *h = 0;
        }
        int total;
        int excl = block_exclusive_scan<256, int>(v, total);
        digit_base[p * 256 + threadIdx.x] = excl;
    }
}

// kernel_generateHouseholds (PandemicSim.cu:2490-2531): adults first (AGE_ADULT),
// then children with the AGE_5 placeholder.  Slots of type 0xFF hold an instance's
// padding persons and are skipped.
__global__ void k_generate_households(const uint8_t *types, const int32_t *hh_offset, int slots, int32_t *household,
                                      uint8_t *age)
{
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < slots; h += gridDim.x * blockDim.x) {
        int t = types[h];
        if (t > 8) continue;
        int off = hh_offset[h];
        int na = c_hh_adults[t], nc = c_hh_children[t];
        for (int i = 0; i < na + nc; i++) {
            household[off + i] = h;
            age[off + i] = i < na ? 5 : 0;
        }
    }
}

cudaError_t launch_generate_households(const uint8_t *types, const int32_t *hh_offset, int slots, int32_t *household,
                                       uint8_t *age, cudaStream_t s)
{
    int blocks = std::max(1, std::min(div_up(slots, 256), sm_count() * 16));
    k_generate_households<<<blocks, 256, 0, s>>>(types, hh_offset, slots, household, age);
    count_launch();
    return cudaGetLastError();
}

// assignWorkplaceFunctor (PandemicSim.cu:3750-3778): counter W0 + g -> persons
// 4g..4g+3; adults draw a workplace, children an age band and school.  loc_base turns
// the instance's location number into a global one.
__global__ void k_assign_workplaces(SimConst c, uint8_t *age, int32_t *workplace, int loc_base)
{
    const TfKey key = make_key(c);
    const int G = c.N / 4;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t w[4];
        tf2x64(key, c.workplace_offset + (uint64_t)g, w);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int p = 4 * g + i;
            if (p < c.N) {
                int a = age[p];
                if (a == 5) {
                    workplace[p] = loc_base + fish_workplace(c, w[i]);
                } else {
                    workplace[p] = loc_base + fish_school_and_age(c, w[i], &a);
                    age[p] = (uint8_t)a;
                }
            }
        }
    }
}

cudaError_t launch_assign_workplaces(const SimConst &c, uint8_t *age, int32_t *workplace, int loc_base, cudaStream_t s)
{
    int blocks = std::min(div_up(c.N / 4 + 1, 256), sm_count() * 16);
    k_assign_workplaces<<<blocks, 256, 0, s>>>(c, age, workplace, loc_base);
    count_launch();
    return cudaGetLastError();
}

// Padding of a batch, one block per instance.  Without `persons`: the instance's
// last household slot gets type 0xFF and the padding count as its size, so one scan
// of all slots yields tile-aligned person bases.  With `persons`: the padding persons
// get no household, no age and the spare location, which sorts them behind every
// real workplace.
__global__ void k_batch_padding(const InstConst *ic, int K, int P, uint8_t *types, int32_t *sizes,
                                int32_t *household, uint8_t *age, int32_t *workplace, int spare, int persons)
{
    const int k = blockIdx.x;
    if (k >= K) return;
    const InstConst &c = ic[k];
    const int end = k + 1 < K ? ic[k + 1].pbase : P;
    const int first = c.pbase + c.c.N;
    if (!persons) {
        if (threadIdx.x == 0) {
            types[c.hbase + c.c.H] = 0xFF;
            sizes[c.hbase + c.c.H] = end - first;
        }
        return;
    }
    for (int p = first + threadIdx.x; p < end; p += blockDim.x) {
        household[p] = -1;
        age[p] = 0;
        workplace[p] = spare;
    }
}

cudaError_t launch_batch_padding(const DevArrays &d, uint8_t *types, int32_t *sizes, int spare_location, bool persons,
                                 cudaStream_t s)
{
    k_batch_padding<<<d.K, 256, 0, s>>>(d.ic, d.K, d.P, types, sizes, d.household, d.age, d.workplace,
                                        spare_location, persons ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}

__global__ void k_count_keys(const int32_t *keys, int n, int32_t *count)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&count[keys[i]], 1);
}

cudaError_t launch_count_keys(const int32_t *keys, int n, int32_t *count, cudaStream_t s)
{
    int blocks = std::min(div_up(n, 256), sm_count() * 16);
    k_count_keys<<<std::max(blocks, 1), 256, 0, s>>>(keys, n, count);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ radix sort
// Bucket tables: the reference sorts (key, person) pairs stably by key and takes
// lower bounds (CUB radix sort + thrust::lower_bound, PandemicSim.cu:1212-1248,
// :3835-3862), so every bucket lists its persons in ascending id order.  This stable
// LSD radix sort over 8-bit digits gives the same table.  Entries enter the first
// pass in ascending person order; each pass ranks a tile of 4096 entries by digit
// (warp-blocked, so the rank is stable), finds the tile's global position per digit
// by a decoupled look-back over earlier tiles (one thread per digit), and writes.
constexpr int kRadixThreads = 256, kRadixItems = 16;   // the default block: 256 threads x 16 entries
constexpr int kRadixTile = kRadixThreads * kRadixItems;
static_assert(kRadixTile == kRadixTileEntries, "the host sizes the radix look-back words by kRadixTileEntries");

enum RadixMode { kRadixFirst = 0, kRadixMiddle = 1, kRadixLast = 2, kRadixOnly = 3 };
constexpr uint32_t kDropped = 0xFFFFFFFFu;   // value of an entry a pass leaves out (no person id is this)

// Person id of schedule entry i: the setup table is the identity, weekday entries
// are hour-major (i < N hour 0, else hour 1), weekend entries person-major (3 per person).
__device__ __forceinline__ uint32_t entry_person(long long i, int N, int person_mode)
{
    if (person_mode == 0) return (uint32_t)i;
    if (person_mode == 1) return (uint32_t)(i < N ? i : i - N);
    return (uint32_t)(i / 3);
}

// Lanes of the warp holding the same digit as this lane (among lanes in `valid`),
// from one ballot per digit bit: constant cost, unlike a match over 256 values.
__device__ __forceinline__ unsigned digit_peers(unsigned d, int nbits, unsigned valid)
{
    unsigned peers = valid;
#pragma unroll
    for (int b = 0; b < 8; b++) {
        if (b < nbits) {
            const unsigned bit = (d >> b) & 1u;
            const unsigned bal = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? bal : ~bal;
        }
    }
    return peers;
}

// Per-item record kept between the two phases of a pass: bits 0-7 digit, 8-16 the
// entry's place among the warp's entries of that digit (earlier rounds, then lanes),
// bit 17 valid.
__device__ __forceinline__ uint32_t pack_place(unsigned d, unsigned place, bool ok)
{
    return d | (place << 8) | ((unsigned)ok << 17);
}

// The warp's entries of digit d before this round (s_hist[warp][d]) for every lane of
// the round: the lowest lane of each digit group advances the count and broadcasts the
// old value to its group.  Rounds are separated by __syncwarp, so each sees the last.
__device__ __forceinline__ unsigned warp_digit_before(int *hist_d, unsigned peers, unsigned rank, unsigned cnt,
                                                      bool ok, int lane)
{
    int before = 0;
    if (ok && rank == 0) {
        before = *hist_d;
        *hist_d = before + (int)cnt;
    }
    before = __shfl_sync(0xffffffffu, before, ok ? __ffs(peers) - 1 : lane);
    return (unsigned)before;
}

// One stable radix pass over 8 bits of the keys.  FILTER (first pass only) drops
// entries whose bucket is not set in `mark`; passes whose input count lives on the
// device read it from *count_dev.  Persistent blocks take tiles from a ticket in
// order until the entries run out, so a short input costs no idle blocks.  Look-back
// words carry the launch epoch (see lb_word), so they need no reset between passes.
//
// Segmented sorts (sg.tile_prefix set): segment k's entries lie at
// [ic[k].kbase, ic[k].kbase + is[k].marked) and are ordered within the segment only,
// with digit bases of their own (digit_base[(k * passes + pass) * 256 + d]).  The
// segments' tiles are numbered consecutively (segment k owns tiles
// [tile_prefix[k], tile_prefix[k + 1])), and the look-back of a segment's first tile
// starts from zero.  Unsegmented sorts are one segment [0, E).
template <int MODE, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_radix_pass(const uint32_t *__restrict__ keys_in,
                                                                 const uint32_t *__restrict__ vals_in,
                                                                 uint32_t *__restrict__ keys_out,
                                                                 uint32_t *__restrict__ vals_out, int E_arg,
                                                                 const int *count_dev, const uint32_t *mark,
                                                                 int pass, int passes, int nbits, int N,
                                                                 int person_mode, const int *__restrict__ digit_base,
                                                                 RadixSegments sg, unsigned long long *status,
                                                                 int *ctl, int *error, const int *skip)
{
    // a tile of kRadixTile entries: THREADS threads, ITEMS entries each
    constexpr int WARPS = THREADS / 32, ITEMS = kRadixTile / THREADS, WARP_ITEMS = ITEMS * 32;
    static_assert(THREADS >= 256 && ITEMS * THREADS == kRadixTile, "one thread per digit and whole tiles");
    static_assert(WARP_ITEMS <= 512, "an entry's place in its warp's digit run fits 9 bits (pack_place)");
    if (skip && *(volatile const int *)skip) return;
    __shared__ int s_tile;
    // segment, tile within it, entry base, entry count; for a dense segment of a day's
    // first pass: 1, the instance's persons, first person and first bucket
    __shared__ int s_seg[8];
    __shared__ unsigned s_epoch;
    __shared__ int s_hist[WARPS][256];
    __shared__ int s_base[256];   // global position of digit d's entries, less its tile-local start
    __shared__ uint32_t s_key[kRadixTile];
    __shared__ uint32_t s_val[kRadixTile];
    const int shift = 8 * pass;
    // first pass of a day's sort (explicit values: the setup sorts' implicit modes never are)
    const bool day0 = (MODE == kRadixMiddle || MODE == kRadixLast) && sg.day_keys != nullptr && pass == 0;
    const int *tprefix = day0 ? sg.tile_prefix0 : sg.tile_prefix;
    int E = 0, tiles;
    if (sg.tile_prefix) {
        tiles = *(volatile const int *)&tprefix[sg.segments];
    } else {
        E = count_dev ? *(volatile const int *)count_dev : E_arg;
        tiles = (E + kRadixTile - 1) / kRadixTile;
    }
    // only as many blocks as there are tiles take part (ticket, finish count)
    const int active = tiles < (int)gridDim.x ? tiles : (int)gridDim.x;
    if ((int)blockIdx.x >= active) return;
    if (threadIdx.x == 0) s_epoch = (unsigned)(*(volatile int *)&ctl[2]) & 0x3FFFFFFFu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (;;) {
        if (threadIdx.x == 0) {
            const int t = atomicAdd(&ctl[0], 1);
            int k = 0, j = t, sbase = 0, scount = E, dense = 0, nk = 0, pb = 0, bb = 0;
            if (sg.tile_prefix && t < tiles) {
                // the segment owning tile t: the last k with tprefix[k] <= t
                int lo = 0, hi = sg.segments - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (tprefix[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
                k = lo;
                j = t - tprefix[k];
                sbase = (int)sg.ic[k].kbase;
                scount = sg.is[k].marked;
                if (day0 && sg.is[k].dense) {
                    dense = 1;
                    nk = sg.ic[k].c.N;
                    pb = sg.ic[k].pbase;
                    bb = sg.ic[k].bbase[sg.weekend];
                    scount = (sg.weekend ? 3 : 2) * nk;   // every schedule key of the instance
                }
            }
            s_tile = t;
            s_seg[0] = k;
            s_seg[1] = j;
            s_seg[2] = sbase;
            s_seg[3] = scount;
            s_seg[4] = dense;
            s_seg[5] = nk;
            s_seg[6] = pb;
            s_seg[7] = bb;
        }
        __syncthreads();
        const int tile = s_tile;
        const unsigned epoch = s_epoch;
        if (tile >= tiles) break;
        const int seg = s_seg[0], stile = s_seg[1], sbase = s_seg[2], scount = s_seg[3];
        const bool dense = s_seg[4] != 0;
        // the peer words of phase A alias the first WARPS * 256 words of s_key, which
        // phase B only writes after the barrier that ends phase A
        unsigned *const s_peer = s_key + warp * 256;
        for (int i = threadIdx.x; i < WARPS * 256; i += THREADS) {
            (&s_hist[0][0])[i] = 0;
            s_key[i] = 0u;
        }
        __syncthreads();
        const int base = stile * kRadixTile + warp * WARP_ITEMS + lane;  // index within the segment
        const bool full = (stile + 1) * kRadixTile <= scount;
        uint32_t key[ITEMS], val[ITEMS], info[ITEMS];
        if (dense) {
            // the instance's schedule keys, persons implicit (weekday hour-major: entry
            // i < N is person i's hour-0 key, i >= N person i - N's hour-1 key; weekend
            // person-major, three per person), instance-local bucket keys; an entry of
            // an unmarked bucket gets the value kDropped and is left out
            const int nk = s_seg[5], pb = s_seg[6], bb = s_seg[7];
#pragma unroll
            for (int j = 0; j < ITEMS; j++) {
                const int i = base + 32 * j;
                const bool in = full || i < scount;
                const int kg = in ? sg.day_keys[sbase + i] : bb;
                key[j] = (uint32_t)(kg - bb);
                const bool marked = in && ((sg.mark[kg >> 5] >> (kg & 31)) & 1u);
                val[j] = marked ? (uint32_t)(pb + (sg.weekend ? i / 3 : (i < nk ? i : i - nk))) : kDropped;
            }
        } else {
#pragma unroll
            for (int j = 0; j < ITEMS; j++) {
                const int i = base + 32 * j;
                const bool in = full || i < scount;
                key[j] = in ? keys_in[sbase + i] : 0u;
                if (MODE == kRadixFirst || MODE == kRadixOnly) {
                    const uint32_t u = (uint32_t)i;
                    val[j] = person_mode == 0 ? u : (person_mode == 1 ? (u < (uint32_t)N ? u : u - (uint32_t)N) : u / 3u);
                } else {
                    val[j] = in ? vals_in[sbase + i] : 0u;
                }
            }
        }
        // phase A: rank within the warp round, per-warp digit counts.  The lanes holding
        // the same digit come from one ballot per digit bit for narrow digits, and for
        // wider ones from a shared word per digit that each lane ORs its bit into (the
        // leader clears it again); both give the same set.  The leader also advances the
        // warp's count of the digit (warp_digit_before), so each entry leaves with its
        // place among the warp's entries of its digit: earlier rounds, then lanes.
        if (nbits <= 4) {
#pragma unroll
            for (int j = 0; j < ITEMS; j++) {
                const int i = base + 32 * j;
                bool ok = (full || i < scount) && val[j] != kDropped;
                if ((MODE == kRadixFirst || MODE == kRadixOnly) && mark && ok)
                    ok = (mark[key[j] >> 5] >> (key[j] & 31u)) & 1u;
                const unsigned d = (key[j] >> shift) & 255u;
                const unsigned peers = digit_peers(d, nbits, __ballot_sync(0xffffffffu, ok));
                const unsigned rank = __popc(peers & lt), cnt = __popc(peers);
                const unsigned before = warp_digit_before(&s_hist[warp][d], peers, rank, cnt, ok, lane);
                __syncwarp();
                info[j] = pack_place(d, before + rank, ok);
            }
        } else {
#pragma unroll
            for (int j = 0; j < ITEMS; j++) {
                const int i = base + 32 * j;
                bool ok = (full || i < scount) && val[j] != kDropped;
                if ((MODE == kRadixFirst || MODE == kRadixOnly) && mark && ok)
                    ok = (mark[key[j] >> 5] >> (key[j] & 31u)) & 1u;
                const unsigned d = (key[j] >> shift) & 255u;
                if (ok) atomicOr(&s_peer[d], 1u << lane);
                __syncwarp();
                const unsigned peers = ok ? s_peer[d] : 0u;
                __syncwarp();
                const unsigned rank = __popc(peers & lt), cnt = __popc(peers);
                if (ok && rank == 0) s_peer[d] = 0u;
                const unsigned before = warp_digit_before(&s_hist[warp][d], peers, rank, cnt, ok, lane);
                __syncwarp();
                info[j] = pack_place(d, before + rank, ok);
            }
        }
        __syncthreads();
        {
            // thread d < 256: exclusive bases of the warps for digit d, then the look-back
            const int d = threadIdx.x;
            int run = 0, gbase = 0;
            if (d < 256) {
#pragma unroll
                for (int w = 0; w < WARPS; w++) {
                    int c = s_hist[w][d];
                    s_hist[w][d] = run;
                    run += c;
                }
                volatile unsigned long long *st = status;
                int excl = 0;
                if (stile == 0) {
                    st[(size_t)tile * 256 + d] = lb_word(epoch, 2, (unsigned)run);
                } else {
                    st[(size_t)tile * 256 + d] = lb_word(epoch, 1, (unsigned)run);
                    int t = tile - 1;
                    long long spins = 0;
                    while (t >= 0) {
                        const unsigned long long w = st[(size_t)t * 256 + d];
                        const unsigned flag = (unsigned)(w >> 32) & 3u;
                        if ((unsigned)(w >> 34) != epoch || flag == 0) {
                            if (++spins > kSpinLimit) {
                                atomicExch(error, 2);
                                break;
                            }
                            __nanosleep(32);
                            continue;
                        }
                        excl += (int)(unsigned)w;
                        if (flag == 2) break;
                        t--;
                    }
                    st[(size_t)tile * 256 + d] = lb_word(epoch, 2, (unsigned)(excl + run));
                }
                gbase = sbase + digit_base[((size_t)seg * passes + pass) * 256 + d] + excl;
            }
            // tile-local start of digit d (entries of the tile ordered by digit)
            int tile_total;
            const int toff = block_exclusive_scan<THREADS, int>(run, tile_total);
            if (d < 256) {
                s_base[d] = gbase - toff;
                // each warp's first place of digit d in the tile's digit order
#pragma unroll
                for (int w = 0; w < WARPS; w++) s_hist[w][d] += toff;
            }
            if (d == 0) s_tile = tile_total;  // reuse: valid entries of this tile
        }
        __syncthreads();
        // phase B: place each entry in shared memory in digit order (stable): the warp's
        // first place of its digit plus its place among the warp's entries of that digit ...
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            const uint32_t r = info[j];
            if ((r >> 17) & 1u) {
                const int lpos = s_hist[warp][r & 255u] + (int)((r >> 8) & 511u);
                s_key[lpos] = key[j];
                s_val[lpos] = val[j];
            }
        }
        __syncthreads();
        // ... then write each digit's run with consecutive threads (coalesced)
        const int valid = s_tile;
        for (int i = threadIdx.x; i < valid; i += THREADS) {
            const uint32_t k = s_key[i];
            const unsigned d = (k >> shift) & 255u;
            const int pos = s_base[d] + i;
            if (MODE == kRadixFirst || MODE == kRadixMiddle || keys_out) keys_out[pos] = k;
            vals_out[pos] = s_val[i];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const int fin = atomicAdd(&ctl[1], 1);
        if (fin == active - 1) {
            ctl[0] = 0;
            ctl[1] = 0;
            atomicAdd(&ctl[2], 1);
            __threadfence();
        }
    }
}

static int key_bits(int buckets)
{
    int bits = 0;
    while (bits < 31 && (1ll << bits) < (long long)buckets) bits++;
    return bits;
}

int radix_passes(int buckets) { return std::max(1, (key_bits(buckets) + 7) / 8); }

cudaError_t launch_radix_sort(const RadixArgs &r, cudaStream_t s)
{
    const int P = radix_passes(r.buckets);
    const int bits = key_bits(r.buckets);
    const int tiles = std::max(1, div_up(r.E, kRadixTile));
    const bool wide = r.threads == 512;   // 512 threads x 8 entries per tile, at most 2 blocks per SM
    // 256 threads: 3 blocks per SM at 80 registers, or 4 at 64 (the passes with explicit
    // values only; the implicit-value first pass keeps 3)
    const int bps = std::max(1, std::min(wide ? 2 : 4, r.blocks_per_sm));
    const bool four = !wide && bps == 4;
    const int grid = std::max(1, std::min(tiles, bps * sm_count()));  // persistent blocks
    const int grid3 = std::max(1, std::min(tiles, std::min(bps, 3) * sm_count()));
    const uint32_t *kin = r.keys;
    const uint32_t *vin = r.vals;   // nullptr: implicit values (entry index -> person)
    const bool implicit = r.vals == nullptr;
    for (int p = 0; p < P; p++) {
        cudaError_t e;
        uint32_t *kout = (p & 1) ? r.k1 : r.k0;
        // the last pass writes keys only when asked to (RadixArgs::keep_keys)
        if (p == P - 1 && !r.keep_keys) kout = nullptr;
        uint32_t *vout = (p == P - 1) ? r.out : ((p & 1) ? r.v1 : r.v0);
        const int nbits = std::max(1, std::min(8, bits - 8 * p));
        // the first pass of an implicit-value sort reads all E entries (and may
        // filter); every other pass reads the count on the device, if any
        const int *cnt = (p == 0 && implicit) ? nullptr : r.count_dev;
        const uint32_t *mk = (p == 0) ? r.mark : nullptr;
#define PT_RADIX_ARGS kin, vin, kout, vout, r.E, cnt, mk, p, P, nbits, r.N, r.person_mode, r.digit_base, r.seg, r.status, \
                      r.ctl, r.error, r.skip
        if (P == 1 && implicit)
            k_radix_pass<kRadixOnly, kRadixThreads, 3><<<grid3, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
        else if (p == 0 && implicit)
            k_radix_pass<kRadixFirst, kRadixThreads, 3><<<grid3, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
        else if (p == P - 1 && wide)
            k_radix_pass<kRadixLast, 512, 2><<<grid, 512, 0, s>>>(PT_RADIX_ARGS);
        else if (p == P - 1 && four)
            k_radix_pass<kRadixLast, kRadixThreads, 4><<<grid, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
        else if (p == P - 1)
            k_radix_pass<kRadixLast, kRadixThreads, 3><<<grid, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
        else if (wide)
            k_radix_pass<kRadixMiddle, 512, 2><<<grid, 512, 0, s>>>(PT_RADIX_ARGS);
        else if (four)
            k_radix_pass<kRadixMiddle, kRadixThreads, 4><<<grid, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
        else
            k_radix_pass<kRadixMiddle, kRadixThreads, 3><<<grid, kRadixThreads, 0, s>>>(PT_RADIX_ARGS);
#undef PT_RADIX_ARGS
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        kin = kout;
        vin = vout;
    }
    return cudaSuccess;
}

// Count, scan (+digit histograms), digit bases and radix passes: the bucket table of
// `E` keys in [0, buckets).  counts must be zero on entry and is zero on exit.
cudaError_t launch_bucket_table(const RadixArgs &r, int32_t *counts, bool count_keys, int32_t *offset,
                                unsigned long long *tiles, int *lb_ctl, int *digit_hist, cudaStream_t s)
{
    const int P = radix_passes(r.buckets);
    if (count_keys) {
        cudaError_t e = launch_count_keys((const int32_t *)r.keys, r.E, counts, s);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = launch_scan_exclusive(counts, offset, r.buckets, 1, tiles, lb_ctl, r.error, r.skip, P,
                                          digit_hist, s, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    k_digit_bases<<<1, 256, 0, s>>>(digit_hist, (int *)r.digit_base, P, 1, r.skip);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_radix_sort(r, s);
}

// setup_initializeStatusArrays (PandemicSim.cu:3654-3664): S/S, day 255/255, gen 255.
__global__ void k_init_status(int N, uint32_t *state, uint8_t *gen_p, uint8_t *gen_s, unsigned long long *claim)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        state[i] = 0x01u | (0x01u << 8) | (0xFFu << 16) | (0xFFu << 24);
        gen_p[i] = 0xFF;
        gen_s[i] = 0xFF;
        claim[2 * (size_t)i] = ~0ull;
        claim[2 * (size_t)i + 1] = ~0ull;
    }
}

cudaError_t launch_init_status(int N, uint32_t *state, uint8_t *gen_p, uint8_t *gen_s,
                               unsigned long long *claim, cudaStream_t s)
{
    int blocks = std::min(div_up(N, 256), sm_count() * 16);
    k_init_status<<<std::max(1, blocks), 256, 0, s>>>(N, state, gen_p, gen_s, claim);
    count_launch();
    return cudaGetLastError();
}

// One block per instance: zero its state words, then set the counter offset.
__global__ void k_reset_instances(const InstConst *ic, InstState *is, int K)
{
    const int k = blockIdx.x;
    if (k >= K) return;
    int *w = reinterpret_cast<int *>(&is[k]);
    for (int i = threadIdx.x; i < (int)(sizeof(InstState) / 4); i += blockDim.x) w[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0)
        is[k].rand_offset = (unsigned long long)(ic[k].c.H / 4) + (unsigned long long)(ic[k].c.N / 4);
}

cudaError_t launch_reset_instances(const DevArrays &d, cudaStream_t s)
{
    k_reset_instances<<<d.K, 256, 0, s>>>(d.ic, d.is, d.K);
    count_launch();
    return cudaGetLastError();
}

// Vaccination (an intervention, no reference counterpart): one person tile per block;
// a vaccinated person starts recovered from both strains, never infected.
__global__ void k_vaccinate(const InstConst *ic, const int32_t *tile_inst, uint32_t *state)
{
    const int k = tile_inst[blockIdx.x];
    const InstConst &c = ic[k];
    if (c.vacc_thr == 0) return;
    const int first = blockIdx.x * kPersonTile - c.pbase;
    for (int i = threadIdx.x; i < kPersonTile; i += blockDim.x) {
        const int p = first + i;
        if (p >= c.c.N) break;
        if (intervention_hash(c.c.key0, c.c.key1, kTagVaccinated, 0, p) < c.vacc_thr)
            state[c.pbase + p] = (0xFFu << 16) | (0xFFu << 24);  // status R / R, day 255 / 255
    }
}

cudaError_t launch_vaccinate(const DevArrays &d, cudaStream_t s)
{
    k_vaccinate<<<d.P / kPersonTile, 256, 0, s>>>(d.ic, d.tile_inst, d.state);
    count_launch();
    return cudaGetLastError();
}

// setup_initialInfected (PandemicSim.cu:708-758): the first P seeds get the pandemic
// strain, the next S the seasonal one; status STATUS_INFECTED, day 0, generation 0.
__global__ void k_seed_infected(const int32_t *seeds, int P, int S, uint32_t *state, uint8_t *gen_p, uint8_t *gen_s)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P + S) return;
    int p = seeds[i];
    if (i < P) {
        state[p] = (state[p] & 0xFF00FF00u) | 0x02u;          // status_p = 2, day_p = 0
        gen_p[p] = 0;
    } else {
        state[p] = (state[p] & 0x00FF00FFu) | (0x02u << 8);   // status_s = 2, day_s = 0
        gen_s[p] = 0;
    }
}

cudaError_t launch_seed_infected(const int32_t *seeds, int P, int S, uint32_t *state, uint8_t *gen_p,
                                 uint8_t *gen_s, cudaStream_t s)
{
    if (P + S <= 0) return cudaSuccess;
    k_seed_infected<<<div_up(P + S, 256), 256, 0, s>>>(seeds, P, S, state, gen_p, gen_s);
    count_launch();
    return cudaGetLastError();
}

// The packed per-person records (PersonRec layout in pt_kernels.h): one thread per
// person.  Everything in a record is fixed once the workplace table exists.
__global__ void k_person_records(const InstConst *ic, const int32_t *tile_inst, int P, const int32_t *household,
                                 const int32_t *hh_offset, const int32_t *workplace, const int32_t *wp_offset,
                                 const uint8_t *age, uint4 *prec)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const int hh = household[p];
        if (hh < 0) {  // padding person
            prec[p] = make_uint4(0u, 0u, 0u, 0u);
            continue;
        }
        const InstConst &k = ic[tile_inst[p / kPersonTile]];
        const int hoff = hh_offset[hh], hcnt = hh_offset[hh + 1] - hoff;
        const int wp = workplace[p];
        const int woff = wp_offset[wp], wcnt = wp_offset[wp + 1] - woff;
        const int loc = wp - k.lbase;
        const uint32_t w = (uint32_t)hcnt | ((uint32_t)age[p] << 4) | ((uint32_t)workplace_max_contacts(k.c, loc) << 8) |
                           ((uint32_t)is_school(k.c, loc) << 10);
        prec[p] = make_uint4((uint32_t)hoff, (uint32_t)woff, (uint32_t)wcnt, w);
    }
}

cudaError_t launch_person_records(const DevArrays &d, cudaStream_t s)
{
    const int blocks = std::max(1, std::min(div_up(d.P, 256), sm_count() * 16));
    k_person_records<<<blocks, 256, 0, s>>>(d.ic, d.tile_inst, d.P, d.household, d.hh_offset, d.workplace,
                                            d.wp_offset, d.age, d.prec);
    count_launch();
    return cudaGetLastError();
}

// ================================================================== day
// Every day kernel covers all instances of a batch in one launch.  Persons are
// global ids; a person tile (kPersonTile persons) belongs to one instance
// (tile_inst), and an infected list position to the instance in infected_inst.

// An instance takes part in a day until a day counts zero infected, and for at
// most its max_days days.
__device__ __forceinline__ bool instance_running(const InstConst &c, const InstState &s, int day)
{
    return !s.done && day < c.max_days;
}

// Sweep: one tile of 4096 persons per block; each thread holds 4 rounds of 4
// persons (one 16-byte load per round).  Output order is (round, thread, item),
// which is ascending person order within the tile.
constexpr int kSweepThreads = 256, kSweepRounds = 4, kSweepTile = kSweepThreads * 4 * kSweepRounds;
static_assert(kSweepTile == kPersonTile, "a sweep tile is a person tile");

constexpr uint32_t kNeverInfected = 0x01u | (0x01u << 8) | (0xFFu << 16) | (0xFFu << 24);

__device__ __forceinline__ uint32_t recover_word(uint32_t st, int d2r, bool &changed)
{
    uint32_t sp = st & 0xFFu, ss = (st >> 8) & 0xFFu, dp = (st >> 16) & 0xFFu, ds = st >> 24;
    uint32_t out = st;
    if (d2r >= 0 && sp >= 2u && (int)dp <= d2r) out &= ~0xFFu;
    if (d2r >= 0 && ss >= 2u && (int)ds <= d2r) out &= ~0xFF00u;
    changed = out != st;
    return out;
}

// A day kernel's person tile: its look-back ticket and the instance it belongs to.
// Thread 0 takes the ticket; with a single instance the instance record is read in
// parallel with the ticket's round trip instead of after it.
struct TileInfo {
    int tile;
    unsigned epoch;
    int inst, pbase, pend, first_person_after;  // first_person_after: pbase + N, or the tile start if not running
};

__device__ __forceinline__ void tile_begin(const LookBack &lb, const InstConst *ic, const InstState *is,
                                           const int32_t *tile_inst, int K, int day, TileInfo &out)
{
    __shared__ TileInfo s_t;
    if (threadIdx.x == 0) {
        TileInfo t;
        int N = 0, running = 0;
        if (K == 1) {
            t.inst = 0;
            t.pbase = ic[0].pbase;
            t.pend = ic[0].pend;
            N = ic[0].c.N;
            running = instance_running(ic[0], is[0], day);
        }
        t.tile = atomicAdd(&lb.ctl[0], 1);
        t.epoch = (unsigned)(*(volatile int *)&lb.ctl[2]) & 0x3FFFFFFFu;
        if (K != 1) {
            const int k = tile_inst[t.tile];
            t.inst = k;
            t.pbase = ic[k].pbase;
            t.pend = ic[k].pend;
            N = ic[k].c.N;
            running = instance_running(ic[k], is[k], day);
        }
        t.first_person_after = running ? t.pbase + N : t.tile * kPersonTile;
        s_t = t;
    }
    __syncthreads();
    out = s_t;
}

// The sweep: kernel_countInfectedStatusAndRecover (PandemicSim.cu:2097-2192), the
// copy_if of the infected (:2207-2224) and runToCompletion's day bookkeeping
// (:891-937) in three launches over every instance:
//   count  four person tiles per block (one for small runs): recover, count the
//          instances' 16 status bins (reduced once per block and instance), and
//          record each thread's infected persons as a 16-bit mask and each tile's
//          infected count.  Thread t of a tile holds persons (r * 256 + t) * 4 + j,
//          rounds r = 0..3, items j = 0..3; mask bit 4r + j.
//   scan   one block: exclusive scan of the tile counts, each instance's run
//          [start, list_end) of the infected list and its day bookkeeping.
//   emit   one person tile per warp (per block for small runs): the infected ids,
//          in ascending order, at their list positions.
// Each launch depends only on the one before, so no block waits for another.
constexpr int kSweepTilesPerBlock = 4;   // at most, person tiles a count block sweeps one after another

// Adds a thread's packed status bins (and its never-infected persons, bin S of both
// strains) into instance k's row of the day: warp reductions, one shared atomic per
// bin per warp, one global atomic per bin per block.  Block-uniform; clears the bins.
__device__ __forceinline__ void sweep_flush_bins(InstState *is, int k, int day, unsigned long long &bp_lo,
                                                 unsigned long long &bp_hi, unsigned long long &bs_lo,
                                                 unsigned long long &bs_hi, int &nss, int *s_bins)
{
    bp_lo += (unsigned long long)nss << 16;  // bin 1 (S) of each strain
    bs_lo += (unsigned long long)nss << 16;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bp_lo += __shfl_xor_sync(0xffffffffu, bp_lo, o);
        bp_hi += __shfl_xor_sync(0xffffffffu, bp_hi, o);
        bs_lo += __shfl_xor_sync(0xffffffffu, bs_lo, o);
        bs_hi += __shfl_xor_sync(0xffffffffu, bs_hi, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int b = 0; b < 4; b++) {
            int a0 = (int)((bp_lo >> (16 * b)) & 0xFFFF), a1 = (int)((bp_hi >> (16 * b)) & 0xFFFF);
            int a2 = (int)((bs_lo >> (16 * b)) & 0xFFFF), a3 = (int)((bs_hi >> (16 * b)) & 0xFFFF);
            if (a0) atomicAdd(&s_bins[b], a0);
            if (a1) atomicAdd(&s_bins[4 + b], a1);
            if (a2) atomicAdd(&s_bins[8 + b], a2);
            if (a3) atomicAdd(&s_bins[12 + b], a3);
        }
    }
    __syncthreads();
    if (threadIdx.x < 16) {
        if (s_bins[threadIdx.x]) atomicAdd(&is[k].counts[day][threadIdx.x], s_bins[threadIdx.x]);
        s_bins[threadIdx.x] = 0;
    }
    __syncthreads();
    bp_lo = bp_hi = bs_lo = bs_hi = 0;
    nss = 0;
}

__global__ void __launch_bounds__(kSweepThreads, 8) k_sweep_count(const InstConst *ic, InstState *is,
                                                                  const int32_t *tile_inst, int tiles, int per_block,
                                                                  uint32_t *state, uint16_t *flags_out,
                                                                  int32_t *tile_count, const Scalars *sc, int day)
{
    if (*(volatile const int *)&sc->done) return;
    const int t0 = blockIdx.x * per_block;
    const int t1 = t0 + per_block < tiles ? t0 + per_block : tiles;
    const int d2r = day - 10;
    __shared__ int s_bins[16];
    __shared__ int s_tc[kSweepTilesPerBlock];   // infected of each of the block's tiles
    if (threadIdx.x < 16) s_bins[threadIdx.x] = 0;
    if (threadIdx.x < kSweepTilesPerBlock) s_tc[threadIdx.x] = 0;
    __syncthreads();
    // packed per-thread status bins of the current instance: 16-bit fields, bins 0-3 /
    // 4-7 per strain
    unsigned long long bp_lo = 0, bp_hi = 0, bs_lo = 0, bs_hi = 0;
    int nss = 0;         // persons in the never-infected state (S, S, day 255, day 255)
    int cur = tile_inst[t0];
    for (int tile = t0;; tile++) {
        // after the last tile, or when the tiles move on to the next instance: the bins
        const int k = tile < t1 ? tile_inst[tile] : -1;
        if (k != cur) {
            sweep_flush_bins(is, cur, day, bp_lo, bp_hi, bs_lo, bs_hi, nss, s_bins);  // (ends with a barrier)
            cur = k;
        }
        if (k < 0) break;
        const long long tile_base = (long long)tile * kSweepTile;
        // end of the tile's persons: none when the instance no longer runs
        const long long N = instance_running(ic[k], is[k], day) ? (long long)ic[k].pbase + ic[k].c.N : tile_base;
        uint32_t flags = 0;  // bit (4*round + item)
#pragma unroll
        for (int r = 0; r < kSweepRounds; r++) {
            long long p0 = tile_base + ((long long)r * kSweepThreads + threadIdx.x) * 4;
            uint32_t st[4];
            if (p0 + 3 < N) {
                uint4 v = *reinterpret_cast<const uint4 *>(state + p0);
                st[0] = v.x; st[1] = v.y; st[2] = v.z; st[3] = v.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) st[j] = (p0 + j < N) ? state[p0 + j] : 0u;
            }
            bool any_changed = false;
            uint32_t out[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                // never infected by either strain: nothing to recover, bin S twice
                if (st[j] == kNeverInfected && p0 + j < N) {
                    out[j] = st[j];
                    nss++;
                    continue;
                }
                bool ch;
                out[j] = recover_word(st[j], d2r, ch);
                if (p0 + j < N) {
                    any_changed |= ch;
                    uint32_t sp = out[j] & 0xFFu, ss = (out[j] >> 8) & 0xFFu;
                    if (sp < 4) bp_lo += 1ull << (16 * sp); else bp_hi += 1ull << (16 * (sp - 4));
                    if (ss < 4) bs_lo += 1ull << (16 * ss); else bs_hi += 1ull << (16 * (ss - 4));
                    if (sp >= 2u || ss >= 2u) flags |= 1u << (4 * r + j);
                }
            }
            if (any_changed) {
                if (p0 + 3 < N) {
                    *reinterpret_cast<uint4 *>(state + p0) = make_uint4(out[0], out[1], out[2], out[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (p0 + j < N) state[p0 + j] = out[j];
                }
            }
        }
        flags_out[(size_t)tile * kSweepThreads + threadIdx.x] = (uint16_t)flags;
        int cnt = __popc(flags);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&s_tc[tile - t0], cnt);
    }
    if (threadIdx.x < t1 - t0) tile_count[t0 + threadIdx.x] = s_tc[threadIdx.x];
}

constexpr int kSweepScanThreads = 1024;

__global__ void __launch_bounds__(kSweepScanThreads) k_sweep_scan(const InstConst *ic, InstState *is, int K,
                                                                  int32_t *tile_count, int tiles, Scalars *sc,
                                                                  int day, int dense_level)
{
    if (*(volatile const int *)&sc->done) return;
    // exclusive scan in place, a contiguous chunk per thread; entry `tiles` = total
    const int per = (tiles + kSweepScanThreads - 1) / kSweepScanThreads;
    const int lo = (int)threadIdx.x * per, hi = lo + per < tiles ? lo + per : tiles;
    int sum = 0;
    for (int i = lo; i < hi; i++) sum += tile_count[i];
    int total;
    int run = block_exclusive_scan<kSweepScanThreads, int>(sum, total);
    for (int i = lo; i < hi; i++) {
        const int v = tile_count[i];
        tile_count[i] = run;
        run += v;
    }
    if (threadIdx.x == 0) tile_count[tiles] = total;
    __syncthreads();
    // each running instance's day (runToCompletion, PandemicSim.cu:891-937: the
    // statistics row, the stop on zero infected, the counter offsets E0 / R0 of the
    // schedule and the contacts)
    const bool weekend = (day % 7) >= 5;  // PandemicSim.h:283-284
    for (int k = threadIdx.x; k < K; k += kSweepScanThreads) {
        InstState &s = is[k];
        const int start = tile_count[ic[k].pbase / kSweepTile], end = tile_count[ic[k].pend / kSweepTile];
        s.start = start;
        s.list_end = end;
        s.marked = 0;
        s.dense = 0;
        if (!instance_running(ic[k], s, day)) {
            s.infected = 0;
            continue;
        }
        const int I = end - start;
        s.infected = I;
        // When the infected (each marks one or two buckets) are many against the
        // buckets, most buckets will be read, and the sort can read the schedule keys
        // directly: dense_level 1, 2, 3 take I >= B / 4, I >= B, I >= 2 B; 0 never.
        // Either way the tables are the same.
        const long long B = ic[k].bcount[weekend ? 1 : 0];
        s.dense = dense_level > 0 && 4ll * I >= B * (dense_level == 1 ? 1 : (dense_level == 2 ? 4 : 8)) ? 1 : 0;
        s.infected_per_day[day] = I;
        s.day = day;
        s.days_run = day + 1;
        if (I == 0) {
            s.done = 1;
        } else {
            const unsigned long long N = (unsigned long long)ic[k].c.N;
            const unsigned long long E0 = s.rand_offset;
            const unsigned long long R0 = E0 + (weekend ? 2ull * N : N / 2ull);
            s.errand_offset = E0;
            s.infect_offset = R0;
            s.rand_offset = R0 + 6ull * (unsigned long long)I;
        }
    }
    if (threadIdx.x == 0) {
        sc->infected = total;
        sc->day = day;
        sc->new_count = 0;
        if (total == 0) sc->done = 1;
    }
}

// Emit for small runs: a block per person tile, a block scan of the threads' packed
// per-round counts (a warp per tile would leave most SMs idle).
__global__ void __launch_bounds__(kSweepThreads) k_sweep_emit_block(const int32_t *tile_inst, const uint16_t *flags_in,
                                                                    const int32_t *tile_prefix, int32_t *infected,
                                                                    int32_t *infected_inst, const Scalars *sc)
{
    if (*(volatile const int *)&sc->done) return;
    const int tile = blockIdx.x;
    const int prefix = tile_prefix[tile];
    if (tile_prefix[tile + 1] == prefix) return;  // no infected in this tile
    const uint32_t f = flags_in[(size_t)tile * kSweepThreads + threadIdx.x];
    unsigned long long packed = 0;
#pragma unroll
    for (int r = 0; r < kSweepRounds; r++) packed |= (unsigned long long)__popc((f >> (4 * r)) & 0xFu) << (16 * r);
    // positions in person order: scan the four per-round counts at once (16-bit fields)
    unsigned long long round_tot;
    const unsigned long long excl = block_exclusive_scan<kSweepThreads, unsigned long long>(packed, round_tot);
    const int k = tile_inst[tile];
    const long long tile_base = (long long)tile * kSweepTile;
    int round_base = prefix;
#pragma unroll
    for (int r = 0; r < kSweepRounds; r++) {
        int pos = round_base + (int)((excl >> (16 * r)) & 0xFFFF);
        const long long p0 = tile_base + ((long long)r * kSweepThreads + threadIdx.x) * 4;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (f & (1u << (4 * r + j))) {
                infected[pos] = (int32_t)(p0 + j);
                infected_inst[pos] = k;
                pos++;
            }
        }
        round_base += (int)((round_tot >> (16 * r)) & 0xFFFF);
    }
}

constexpr int kEmitWarps = 8;   // person tiles per emit block, one warp each

// Emit: a warp per person tile.  Lane l reads the masks of count-kernel threads
// 8l .. 8l+7 in one 16-byte load; per round, a warp scan of the lanes' counts places
// them, so the ids come out in (round, thread, item) order: ascending persons.
__global__ void __launch_bounds__(kEmitWarps * 32) k_sweep_emit(const int32_t *tile_inst, int tiles,
                                                                const uint16_t *flags_in,
                                                                const int32_t *tile_prefix, int32_t *infected,
                                                                int32_t *infected_inst, const Scalars *sc)
{
    if (*(volatile const int *)&sc->done) return;
    const int lane = threadIdx.x & 31;
    const int tile = blockIdx.x * kEmitWarps + (threadIdx.x >> 5);
    if (tile >= tiles) return;
    const int prefix = tile_prefix[tile];
    if (tile_prefix[tile + 1] == prefix) return;  // no infected in this tile
    const uint4 raw = *reinterpret_cast<const uint4 *>(flags_in + (size_t)tile * kSweepThreads + 8 * lane);
    const uint32_t wd[4] = {raw.x, raw.y, raw.z, raw.w};  // masks of threads 8l + 2i (low half), 8l + 2i + 1
    const int k = tile_inst[tile];
    const long long tile_base = (long long)tile * kSweepTile;
    int round_base = prefix;
#pragma unroll
    for (int r = 0; r < kSweepRounds; r++) {
        int c = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) c += __popc((wd[i] >> (4 * r)) & 0xFu) + __popc((wd[i] >> (16 + 4 * r)) & 0xFu);
        const int incl = warp_inclusive_scan(c);
        int pos = round_base + incl - c;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint32_t m = (wd[q >> 1] >> (16 * (q & 1) + 4 * r)) & 0xFu;
            if (m) {
                const long long p0 = tile_base + ((long long)r * kSweepThreads + 8 * lane + q) * 4;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if ((m >> j) & 1u) {
                        infected[pos] = (int32_t)(p0 + j);
                        infected_inst[pos] = k;
                        pos++;
                    }
                }
            }
        }
        round_base += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// The look-back control block sits right after the tile words.
static LookBack make_lb(const DevArrays &d)
{
    LookBack lb;
    lb.tiles = d.tiles;
    lb.ctl = (int *)(d.tiles + d.tiles_cap);
    lb.error = &d.sc->error;
    return lb;
}

cudaError_t launch_sweep(const DevArrays &d, int day, cudaStream_t s)
{
    const int tiles = d.P / kSweepTile;
    // several tiles per block only where the grid still fills every SM eight times over
    // (a small simulation keeps one tile per block and all its parallelism)
    const int per_block = tiles >= kSweepTilesPerBlock * 8 * sm_count() ? kSweepTilesPerBlock : 1;
    k_sweep_count<<<div_up(tiles, per_block), kSweepThreads, 0, s>>>(d.ic, d.is, d.tile_inst, tiles, per_block, d.state,
                                                                    d.sweep_flags, d.sweep_tiles, d.sc, day);
    count_launch();
    k_sweep_scan<<<1, kSweepScanThreads, 0, s>>>(d.ic, d.is, d.K, d.sweep_tiles, tiles, d.sc, day,
                                                 d.tune.dense_level);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_infected_list(const DevArrays &d, cudaStream_t s)
{
    const int tiles = d.P / kSweepTile;
    if (tiles >= kSweepTilesPerBlock * 8 * sm_count())
        k_sweep_emit<<<div_up(tiles, kEmitWarps), kEmitWarps * 32, 0, s>>>(d.tile_inst, tiles, d.sweep_flags,
                                                                           d.sweep_tiles, d.infected, d.infected_inst,
                                                                           d.sc);
    else
        k_sweep_emit_block<<<tiles, kSweepThreads, 0, s>>>(d.tile_inst, d.sweep_flags, d.sweep_tiles, d.infected,
                                                           d.infected_inst, d.sc);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ schedules
// Weekday schedule (kernel_assignWeekdayAfterschoolAndErrands, PandemicSim.cu:2972-3022):
// counter E0 + g -> the instance's persons 2g, 2g+1.  Hour-0 keys at [0,N), hour-1
// keys at [N,2N) of the instance's key slots.  Weekday destinations lie in [lo, L),
// lo = first location of type 8 (afterschool), so the instance's bucket is
// hour * R + dest - lo with R = L - lo (order-preserving); the global bucket adds the
// instance's weekday bucket base.
__device__ __forceinline__ void weekday_pair_keys(const SimConst &c, const uint32_t w[4], int k, bool adult, int lo,
                                                  int R, int &k1, int &k2)
{
    // the second errand is drawn for every lane and kept for adults (no divergence)
    const int d1 = fish_weekday_dest(c, w[2 * k], adult);
    const int e2 = fish_weekday_dest(c, w[2 * k + 1], true);
    const int d2 = adult ? e2 : d1;
    k1 = d1 - lo;
    k2 = R + d2 - lo;
}

__device__ __forceinline__ bool is_marked(const uint32_t *mark, int b) { return (mark[b >> 5] >> (b & 31)) & 1u; }

// Fire-and-forget global updates (PTX red): the thread does not wait for the result.
__device__ __forceinline__ void red_add(int *p, int v)
{
    asm volatile("red.relaxed.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_or(uint32_t *p, uint32_t v)
{
    asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void mark_bucket(uint32_t *mark, int b) { red_or(&mark[b >> 5], 1u << (b & 31)); }

// Adds this lane's key b (when `on`) to the block's digit histograms of the radix
// passes.  Called by all 32 lanes.  The lower digits are spread out and each lane
// adds its own; the top digit of a tile's keys is often the same across the warp,
// and then one lane adds the count.
__device__ __forceinline__ void digit_count(int (*s_dh)[256], int passes, bool on, uint32_t b)
{
    const unsigned act = __ballot_sync(0xffffffffu, on);
    if (!act) return;
    if (on)
        for (int p = 0; p < passes - 1; p++) atomicAdd(&s_dh[p][(b >> (8 * p)) & 255u], 1);
    const int top = passes - 1;
    const uint32_t d = (b >> (8 * top)) & 255u;
    const int leader = __ffs(act) - 1;
    const uint32_t d0 = __shfl_sync(0xffffffffu, d, leader);
    if (__all_sync(0xffffffffu, !on || d == d0)) {
        if ((int)(threadIdx.x & 31) == leader) atomicAdd(&s_dh[top][d0], __popc(act));
    } else if (on) {
        atomicAdd(&s_dh[top][d], 1);
    }
}

// Marks the errand buckets today's contact draws will read: the only buckets that
// must be materialised.  Destinations are regenerated from the schedule counter, as
// the reference's device_recalc_* functions do (PandemicSim.cu:3667-3705,
// :3742-3746), and only the hours / errands the person's contact profile uses are
// marked: weekday hours whose profile wants contacts (the adult profile comes from
// the same Threefry block, :3697-3702; children use the afterschool profile), and on
// weekends the two errand slots picked by word 3 of the infection counter's block
// (:1892, :1909, :1929).
__global__ void k_mark_buckets(const InstConst *ic, const InstState *is, const uint8_t *age, const int32_t *infected,
                               const int32_t *infected_inst, int weekend, uint32_t *mark, const Scalars *sc)
{
    if (sc->done) return;
    const int I = sc->infected;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < I; pos += gridDim.x * blockDim.x) {
        const int k = infected_inst[pos];
        const InstConst &ik = ic[k];
        const SimConst &c = ik.c;
        const InstState &s = is[k];
        const TfKey key = make_key(c);
        const int me = infected[pos] - ik.pbase;   // the instance's person number
        const int lpos = pos - s.start;            // the instance's list position
        if (weekend) {
            const int lo = c.type_offset[9], R = c.L - lo;
            int d[3];
            weekend_errands(c, key, s.errand_offset + 2ull * (unsigned long long)me, lo, R, d);
            uint32_t w[4];
            tf2x64(key, s.infect_offset + 6ull * (unsigned long long)lpos, w);
            const int prof = (int)(w[3] % 6u);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                mark_bucket(mark, ik.bbase[1] + d[c_weekend_assign[prof][j]]);
            }
        } else {
            const int lo = c.type_offset[8], R = c.L - lo;
            uint32_t w[4];
            tf2x64(key, s.errand_offset + (uint64_t)(me / 2), w);
            const bool adult = age[infected[pos]] == 5;
            const int slot = 2 * (me & 1);
            int k1, k2;
            weekday_pair_keys(c, w, me & 1, adult, lo, R, k1, k2);
            k1 += ik.bbase[0];
            k2 += ik.bbase[0];
            const int prof = adult ? (int)((w[slot] ^ w[slot + 1]) % 3u) : 3;
            if (c_weekday_assign[prof][0] > 0) mark_bucket(mark, k1);
            if (c_weekday_assign[prof][1] > 0) mark_bucket(mark, k2);
        }
    }
}

// Schedule kernel, one person tile per block.  Warps own 512 consecutive persons and
// walk them in rounds (weekday: 64 persons a round, a pair per lane, one Threefry
// block per pair; weekend: 32 persons a round, one per lane), so key writes are
// coalesced.  The kernel writes every person's keys, accumulates the radix digit
// histograms of the entries of marked buckets in shared memory, and appends those
// entries as (instance-local key, person) in ascending person order (warp scans +
// block scan + decoupled look-back) to the instance's segment: the order the radix
// sort needs for stability.  Per-round
// marked counts of a lane are packed in one register between the two phases.  The
// instance's constants are staged in shared memory.
constexpr int kSchedThreads = 256, kSchedTile = kPersonTile, kSchedWarpPersons = 512;

template <bool WEEKEND, int TF>
__global__ void __launch_bounds__(kSchedThreads, 8) k_sched(const InstConst *ic, InstState *is,
                                                         const int32_t *tile_inst, int K, const uint8_t *age,
                                                         const uint32_t *mark, int32_t *keys, int *digit_hist,
                                                         int passes, uint32_t *ckeys, uint32_t *cvals, Scalars *sc,
                                                         LookBack lb, int day, TfMul tm)
{
    if (*(volatile int *)&sc->done) return;
    __shared__ int s_dh[kMaxRadixPasses][256];   // digit histograms of the marked entries
    for (int i = threadIdx.x; i < kMaxRadixPasses * 256; i += kSchedThreads) (&s_dh[0][0])[i] = 0;
    __shared__ SimConst s_c;
    const int csz = (int)(sizeof(SimConst) / 4);
    if (K == 1)  // the only instance: copy its constants while thread 0 takes the ticket
        for (int i = threadIdx.x; i < csz; i += kSchedThreads)
            reinterpret_cast<int *>(&s_c)[i] = reinterpret_cast<const int *>(&ic[0].c)[i];
    TileInfo ti;
    tile_begin(lb, ic, is, tile_inst, K, day, ti);
    const int tile = ti.tile;
    const unsigned epoch = ti.epoch;
    const int inst = ti.inst;
    if (K != 1)
        for (int i = threadIdx.x; i < csz; i += kSchedThreads)
            reinterpret_cast<int *>(&s_c)[i] = reinterpret_cast<const int *>(&ic[inst].c)[i];
    const int pbase = ti.pbase;
    const int N = ti.first_person_after - pbase;   // persons to schedule (0 when not running)
    const int tbase = tile * kSchedTile - pbase;   // the tile's first person, instance numbering
    const int valid = N - tbase < kSchedTile ? (N - tbase > 0 ? N - tbase : 0) : kSchedTile;
    int32_t *kk = keys + ic[inst].kbase;   // the instance's key slots
    const int NK = ic[inst].c.N;           // their layout: weekday hour 0 at [0, N), hour 1 at [N, 2N)
    const uint8_t *tage = age + pbase + tbase;
    __syncthreads();
    const SimConst &c = s_c;
    const TfKey key = make_key(c);
    const int bb = ic[inst].bbase[WEEKEND ? 1 : 0];
    const unsigned long long E0 = is[inst].errand_offset;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wl = warp * kSchedWarpPersons;      // the warp's first person, tile numbering
    constexpr int kRounds = WEEKEND ? 16 : 8;
    // which of the lane's entries are marked: bit 3j + k (weekend) / 4j + k (weekday) of
    // round j, kept for the append phase
    constexpr int kPer = WEEKEND ? 3 : 4;
    unsigned long long mbits = 0;
    int mine = 0;
    if (WEEKEND) {
        // kernel_assignWeekendErrands (PandemicSim.cu:2082-2094): counters E0 + 2p, E0 + 2p + 1
        const int lo = c.type_offset[9], R = c.L - lo;
#pragma unroll 1
        for (int j = 0; j < kRounds; j++) {
            const int i = wl + 32 * j + lane;
            uint32_t kb[3] = {0u, 0u, 0u};
            bool mk[3] = {false, false, false};
            if (i < valid) {
                int d[3];
                weekend_errands<TF>(c, key, E0 + 2ull * (unsigned long long)(tbase + i), lo, R, d, &tm);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    kb[k] = (uint32_t)(bb + d[k]);
                    kk[3 * (size_t)(tbase + i) + k] = (int32_t)kb[k];
                    mk[k] = is_marked(mark, (int)kb[k]);
                }
            }
            const int cnt = (int)mk[0] + (int)mk[1] + (int)mk[2];
#pragma unroll
            for (int k = 0; k < 3; k++) digit_count(s_dh, passes, mk[k], kb[k] - (uint32_t)bb);
            mbits |= (unsigned long long)((uint32_t)mk[0] | ((uint32_t)mk[1] << 1) | ((uint32_t)mk[2] << 2)) << (kPer * j);
            mine += cnt;
        }
    } else {
        const int lo = c.type_offset[8], R = c.L - lo;
#pragma unroll 1
        for (int j = 0; j < kRounds; j++) {
            const int i = wl + 64 * j + 2 * lane;  // even: counter E0 + p/2 covers p, p+1
            uint32_t kb[4] = {0u, 0u, 0u, 0u};
            bool mk[4] = {false, false, false, false};
            if (i < valid) {
                uint32_t w[4];
                tf2x64m<TF>(key, E0 + (uint64_t)((tbase + i) / 2), w, tm);
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    if (i + k < valid) {
                        int k1, k2;
                        weekday_pair_keys(c, w, k, tage[i + k] == 5, lo, R, k1, k2);
                        kb[2 * k] = (uint32_t)(k1 + bb);
                        kb[2 * k + 1] = (uint32_t)(k2 + bb);
                        kk[tbase + i + k] = (int32_t)kb[2 * k];
                        kk[(size_t)NK + tbase + i + k] = (int32_t)kb[2 * k + 1];
                        mk[2 * k] = is_marked(mark, (int)kb[2 * k]);
                        mk[2 * k + 1] = is_marked(mark, (int)kb[2 * k + 1]);
                    }
                }
            }
            const int cnt = (int)mk[0] + (int)mk[1] + (int)mk[2] + (int)mk[3];
#pragma unroll
            for (int k = 0; k < 4; k++) digit_count(s_dh, passes, mk[k], kb[k] - (uint32_t)bb);
            mbits |= (unsigned long long)((uint32_t)mk[0] | ((uint32_t)mk[1] << 1) | ((uint32_t)mk[2] << 2) |
                                          ((uint32_t)mk[3] << 3)) << (kPer * j);
            mine += cnt;
        }
    }
    // tile position: warp totals, block scan over warps, look-back
    __shared__ int s_wtot[kSchedThreads / 32];
    __shared__ int s_wbase[kSchedThreads / 32];
    int wt = mine;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wt += __shfl_xor_sync(0xffffffffu, wt, o);
    if (lane == 0) s_wtot[warp] = wt;
    __syncthreads();
    // A dense instance (most of today's buckets are read): the sort's first pass reads
    // the keys written above, so only the marked count is needed, not the entries.
    const bool dense = is[inst].dense != 0;
    if (dense) {
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int w = 0; w < kSchedThreads / 32; w++) tot += s_wtot[w];
            if (tot) red_add(&is[inst].marked, tot);
        }
    } else if (warp == 0) {
        // the instance's entries form their own segment: its first tile starts the scan
        int tot = 0;
        for (int w = 0; w < kSchedThreads / 32; w++) tot += s_wtot[w];
        const unsigned prefix = lookback_publish_warp(lb, epoch, tile, (unsigned)tot, tbase == 0);
        if (lane == 0) {
            int run = (int)prefix;
            for (int w = 0; w < kSchedThreads / 32; w++) {
                s_wbase[w] = run;
                run += s_wtot[w];
            }
            if (pbase + tbase + kSchedTile == ti.pend) is[inst].marked = run;
        }
    }
    __syncthreads();
    {
        int *h = digit_hist + ((size_t)inst * kDigitStripes + blockIdx.x % kDigitStripes) * kMaxRadixPasses * 256;
        for (int p = 0; p < passes; p++) {
            const int v = s_dh[p][threadIdx.x];
            if (v) red_add(&h[p * 256 + threadIdx.x], v);
        }
    }
    if (dense) {
        lookback_end(lb);
        return;
    }
    ckeys += ic[inst].kbase;   // the instance's segment of the entry arrays
    cvals += ic[inst].kbase;
    // append the marked entries, rounds in order, lanes in order within a round
    int run = s_wbase[warp];
    const int gbase = pbase + tbase;   // global id of the tile's first person
#pragma unroll 1
    for (int j = 0; j < kRounds; j++) {
        const uint32_t bits = (uint32_t)(mbits >> (kPer * j)) & ((1u << kPer) - 1u);
        const int cnt = __popc(bits);
        if (__ballot_sync(0xffffffffu, cnt > 0) == 0) continue;
        const int incl = warp_inclusive_scan(cnt);
        int pos = run + incl - cnt;
        if (cnt > 0) {
            if (WEEKEND) {
                const int i = wl + 32 * j + lane;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    if ((bits >> k) & 1u) {
                        ckeys[pos] = (uint32_t)kk[3 * (size_t)(tbase + i) + k] - (uint32_t)bb;
                        cvals[pos] = (uint32_t)(gbase + i);
                        pos++;
                    }
                }
            } else {
                // entry k of the round: person i + k / 2, hour k % 2
                const int i = wl + 64 * j + 2 * lane;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if ((bits >> k) & 1u) {
                        ckeys[pos] = (uint32_t)kk[(size_t)(k & 1) * NK + tbase + i + (k >> 1)] - (uint32_t)bb;
                        cvals[pos] = (uint32_t)(gbase + i + (k >> 1));
                        pos++;
                    }
                }
            }
        }
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    lookback_end(lb);
}

// The run-time constants of tf2x64m: 1 and the powers of two of the rotations.
static TfMul tf_multipliers()
{
    TfMul m;
    m.one = 1u;
    const int r[6] = {16, 10, 12, 31, 24, 21};
    for (int i = 0; i < 6; i++) m.pow[i] = 1u << r[i];
    return m;
}

int day_buckets(const SimConst &c, bool weekend)
{
    return weekend ? 10 * (c.L - c.type_offset[9]) : 2 * (c.L - c.type_offset[8]);
}

// mark (or mark everything for complete tables), then the schedule kernel
cudaError_t launch_schedule(const DevArrays &d, bool weekend, int day, bool full_tables, cudaStream_t s)
{
    const int B = d.buckets[weekend ? 1 : 0];
    cudaError_t e = cudaMemsetAsync(d.mark, full_tables ? 0xFF : 0, ((size_t)B / 32 + 1) * 4, s);
    if (e != cudaSuccess) return e;
    if (!full_tables) {
        k_mark_buckets<<<sm_count() * 4, 128, 0, s>>>(d.ic, d.is, d.age, d.infected, d.infected_inst, weekend ? 1 : 0,
                                                      d.mark, d.sc);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int blocks = d.P / kSchedTile;
    const LookBack lb = make_lb(d);
    const int passes = radix_passes(d.bucket_max[weekend ? 1 : 0]);
    const TfMul tm = tf_multipliers();
#define PT_SCHED(W, T)                                                                                              \
    k_sched<W, T><<<blocks, kSchedThreads, 0, s>>>(d.ic, d.is, d.tile_inst, d.K, d.age, d.mark, d.keys, d.digit_hist, \
                                                    passes, d.rk1, d.rv1, d.sc, lb, day, tm)
    const int tf = d.tune.sched_tf;
    if (weekend) {
        if (tf == 2) PT_SCHED(true, 2);
        else if (tf == 1) PT_SCHED(true, 1);
        else PT_SCHED(true, 0);
    } else {
        if (tf == 2) PT_SCHED(false, 2);
        else if (tf == 1) PT_SCHED(false, 1);
        else PT_SCHED(false, 0);
    }
#undef PT_SCHED
    count_launch();
    return cudaGetLastError();
}

// The day's radix sort: one sorted segment per instance, keys local to the instance,
// so the passes cover the largest instance's buckets only.  A segment's first pass
// reads the marked entries the schedule appended to the instance's part of (rk1, rv1)
// in person order, or, for an instance dense today, every schedule key (keeping the
// marked ones).  Equal keys come from one hour, in person order, in both inputs, so
// the sorted tables are the same.
static RadixArgs day_radix_args(const DevArrays &d, bool weekend)
{
    RadixArgs r;
    r.keys = d.rk1;
    r.vals = d.rv1;
    r.E = 3 * d.P;   // at most (sizes the persistent grid)
    r.buckets = d.bucket_max[weekend ? 1 : 0];
    r.N = d.P;
    r.person_mode = weekend ? 2 : 1;
    r.k0 = d.rk0; r.v0 = d.rv0; r.k1 = d.rk1; r.v1 = d.rv1;
    r.out = (uint32_t *)d.bkt_people;
    r.digit_base = d.digit_base;
    r.seg.tile_prefix = d.tile_prefix;
    r.seg.ic = d.ic;
    r.seg.is = d.is;
    r.seg.segments = d.K;
    r.seg.day_keys = d.keys;
    r.seg.tile_prefix0 = d.tile_prefix0;
    r.seg.mark = d.mark;
    r.seg.weekend = weekend ? 1 : 0;
    r.status = d.radix_status;
    r.ctl = d.radix_ctl;
    r.error = &d.sc->error;
    r.skip = &d.sc->done;
    r.keep_keys = true;  // the bucket offsets come from the sorted keys
    r.blocks_per_sm = d.tune.radix_blocks_per_sm;
    r.threads = d.tune.radix_threads;
    return r;
}

// One block per instance: the digit bases of its segment from the digit histograms
// the schedule kernel accumulated (summing the stripes, clearing them).  Block 0
// also numbers the segments' radix tiles (tile_prefix) and adds the day's
// materialised entries to the running total.
__global__ void k_day_digit_bases(int *digit_hist, int *digit_base, int passes, const InstConst *ic,
                                  const InstState *is, int K, int weekend, int32_t *tile_prefix,
                                  int32_t *tile_prefix0, Scalars *sc)
{
    if (*(volatile const int *)&sc->done) return;
    const int k = blockIdx.x;
    for (int p = 0; p < passes; p++) {
        int v = 0;
        for (int st = 0; st < kDigitStripes; st++) {
            int *h = &digit_hist[(((size_t)k * kDigitStripes + st) * kMaxRadixPasses + p) * 256 + threadIdx.x];
            v += *h;
            *h = 0;
        }
        int total;
        const int excl = block_exclusive_scan<256, int>(v, total);
        digit_base[((size_t)k * passes + p) * 256 + threadIdx.x] = excl;
    }
    if (k != 0) return;
    int carry = 0, carry0 = 0;
    unsigned long long entries = 0;
    for (int b = 0; b < K; b += 256) {
        const int i = b + (int)threadIdx.x;
        const int m = i < K ? is[i].marked : 0;
        // the first pass reads every key of a dense instance, the appended entries otherwise
        const int m0 = (i < K && is[i].dense) ? (weekend ? 3 : 2) * ic[i].c.N : m;
        int total;
        const int excl = block_exclusive_scan<256, int>((m + kRadixTile - 1) / kRadixTile, total);
        if (i < K) tile_prefix[i] = carry + excl;
        carry += total;
        int total0;
        const int excl0 = block_exclusive_scan<256, int>((m0 + kRadixTile - 1) / kRadixTile, total0);
        if (i < K) tile_prefix0[i] = carry0 + excl0;
        carry0 += total0;
        int msum;
        block_exclusive_scan<256, int>(m, msum);
        entries += (unsigned long long)msum;
    }
    if (threadIdx.x == 0) {
        tile_prefix[K] = carry;
        tile_prefix0[K] = carry0;
        sc->materialised_sum += entries;
    }
}

cudaError_t launch_bucket_scan(const DevArrays &d, bool weekend, cudaStream_t s)
{
    const int P = radix_passes(d.bucket_max[weekend ? 1 : 0]);
    k_day_digit_bases<<<d.K, 256, 0, s>>>(d.digit_hist, d.digit_base, P, d.ic, d.is, d.K, weekend ? 1 : 0,
                                          d.tile_prefix, d.tile_prefix0, d.sc);
    count_launch();
    return cudaGetLastError();
}

// Bucket offsets from the sorted keys of each instance's segment: entry i starts
// bucket keys[i] when that differs from keys[i-1] (thrust::lower_bound in the
// reference, PandemicSim.cu:1240-1248).  Lazy tables write only the offsets the
// infection kernels read: the start of each bucket with entries and the end of the
// bucket before it.  Every bucket an infected person reads holds that person, so it
// has entries.  Complete tables write every offset, empty buckets included.  Offsets
// are positions in the batch's bucketed person array; each instance's last offset
// goes to its own end slot.
__global__ void k_bucket_offsets(const uint32_t *keys, RadixSegments sg, int weekend, int full, int32_t *offset,
                                 const int *skip)
{
    if (*(volatile const int *)skip) return;
    const int tiles = sg.tile_prefix[sg.segments];
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        int lo = 0, hi = sg.segments - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (sg.tile_prefix[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
        const InstConst &c = sg.ic[lo];
        const int m = sg.is[lo].marked;
        const int sbase = (int)c.kbase, bb = c.bbase[weekend], B = c.bcount[weekend];
        const int first = (t - sg.tile_prefix[lo]) * kRadixTile;
        int last = first + kRadixTile < m ? first + kRadixTile : m;
        if (last == m) last = m + 1;  // the segment's last tile also writes the end offset
        for (int i = first + (int)threadIdx.x; i < last; i += blockDim.x) {
            const int prev = i == 0 ? -1 : (int)keys[sbase + i - 1];
            const int cur = i == m ? B : (int)keys[sbase + i];
            if (prev == cur) continue;
            if (full) {
                for (int b = prev + 1; b <= cur; b++) offset[bb + b] = sbase + i;
            } else {
                offset[bb + prev + 1] = sbase + i;
                offset[bb + cur] = sbase + i;
            }
        }
    }
}

cudaError_t launch_bucket_sort(const DevArrays &d, bool weekend, cudaStream_t s)
{
    return launch_radix_sort(day_radix_args(d, weekend), s);
}

cudaError_t launch_bucket_offsets(const DevArrays &d, bool weekend, bool full_tables, cudaStream_t s)
{
    const RadixArgs r = day_radix_args(d, weekend);
    const int P = radix_passes(r.buckets);
    const uint32_t *sorted = ((P - 1) & 1) ? r.k1 : r.k0;  // where the last pass wrote the keys
    k_bucket_offsets<<<sm_count() * 8, 256, 0, s>>>(sorted, r.seg, weekend ? 1 : 0, full_tables ? 1 : 0,
                                                    d.bkt_offset, r.skip);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ infection
// device_selectRandomPersonFromLocation (PandemicSim.cu:2028-2071).  A location with
// at most one person gives victim = count and type NONE (kappa 0).
__device__ __forceinline__ int select_victim(int self, int off, int count, uint32_t r, bool home,
                                             const int32_t *table, int &victim)
{
    if (count <= 1) {
        victim = count;
        return 0;
    }
    int o = (int)(r % (uint32_t)count);
    int v = home ? off + o : table[off + o];
    if (v == self) {
        o = (o + 1) % count;
        v = home ? off + o : table[off + o];
    }
    victim = v;
    return 1;
}

struct Infector {
    int me, pos;   // global person id, position in the batch's infected list
    float prob[2];
    int gen[2];
};

// device_processContacts (PandemicSim.cu:3106-3233) with the claim rule: a
// successful draw on a victim whose strain status was susceptible at the start of
// the day claims (victim, strain) with key (position, slot); the smallest key wins.
// A victim is only ever drawn by infectors of its own instance, whose list positions
// keep the instance's order.
template <int NC>
__device__ __forceinline__ void process_contacts(const SimConst &c, const TfKey &key, const Infector &inf,
                                                 unsigned long long ctr, const int (&victims)[NC],
                                                 const int (&kv)[NC], const uint32_t *state,
                                                 unsigned long long *claim, int32_t *new_list, Scalars *sc)
{
    uint32_t w[16];
    tf2x64(key, ctr + 0, w + 0);
    tf2x64(key, ctr + 1, w + 4);
    tf2x64(key, ctr + 2, w + 8);
    tf2x64(key, ctr + 3, w + 12);
#pragma unroll
    for (int j = 0; j < NC; j++) {
        const float kf = __int2float_rn(kv[j]);
#pragma unroll
        for (int strain = 0; strain < 2; strain++) {
            const int u = 2 * j + strain;
            const float y = to_unit(w[u]);
            const bool hit = y < __fmul_rn(inf.prob[strain], kf);
            if (hit) {
                const int v = victims[j];
                const uint32_t st = state[v];
                const uint32_t vstatus = strain ? ((st >> 8) & 0xFFu) : (st & 0xFFu);
                if (vstatus == 1u) {
                    const int profile = infection_profile(c, w[u] ^ w[(u + 1) & 15]);
                    unsigned long long k = ((unsigned long long)((long long)inf.pos * 8 + j) << 16) |
                                           ((unsigned long long)profile << 8) | (unsigned long long)(inf.gen[strain] & 0xFF);
                    unsigned long long old = atomicMin(&claim[2 * (size_t)v + strain], k);
                    if (old == ~0ull) new_list[atomicAdd(&sc->new_count, 1)] = 2 * v + strain;
                }
            }
        }
    }
}

__device__ __forceinline__ void infector_state(const SimConst &c, Infector &inf, uint32_t st, const uint8_t *gen_p,
                                               const uint8_t *gen_s, int day, int ksum)
{
#pragma unroll
    for (int strain = 0; strain < 2; strain++) {
        uint32_t status = strain ? ((st >> 8) & 0xFFu) : (st & 0xFFu);
        uint32_t dday = strain ? (st >> 24) : ((st >> 16) & 0xFFu);
        inf.prob[strain] = -1.f;
        inf.gen[strain] = 0xFF;
        if (status >= 2u) {
            int pd = day - (int)dday;
            if (pd >= 0 && pd < 10) {
                inf.prob[strain] = infection_probability(c, (int)status - 2, pd, strain, ksum);
                inf.gen[strain] = ((strain ? gen_s[inf.me] : gen_p[inf.me]) + 1) & 0xFF;
            }
        }
    }
}

struct InfectArgs {
    const InstConst *ic;
    const InstState *is;
    const uint32_t *state;
    const uint8_t *gen_p, *gen_s, *age;
    const uint4 *prec;
    const int32_t *wp_people;
    const int32_t *keys, *bkt_offset, *bkt_people, *infected, *infected_inst;
    unsigned long long *claim;
    int32_t *new_list;
    Scalars *sc;
};

// An infector's packed record: one 128-bit read-only load.
__device__ __forceinline__ uint4 load_record(const uint4 *prec, int me) { return __ldg(&prec[me]); }

// kernel_doWeekday + device_makeContacts_weekday (PandemicSim.cu:3236-3308, :1669-1829),
// one thread per infector.
__global__ void __launch_bounds__(128) k_infect_weekday(InfectArgs a, int day)
{
    Scalars *sc = a.sc;
    if (sc->done) return;
    const int I = sc->infected;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < I; pos += gridDim.x * blockDim.x) {
        const int inst = a.infected_inst[pos];
        const InstConst &ik = a.ic[inst];
        const SimConst &c = ik.c;
        const InstState &s = a.is[inst];
        const TfKey key = make_key(c);
        Infector inf;
        inf.pos = pos;
        inf.me = a.infected[pos];
        const int me = inf.me;
        const int lme = me - ik.pbase;  // the instance's person number
        const unsigned long long ctr = s.infect_offset + 6ull * (unsigned long long)(pos - s.start);
        const uint4 rec = load_record(a.prec, me);
        uint32_t w[8];
        tf2x64(key, ctr, w);
        tf2x64(key, ctr + 1, w + 4);
        const bool adult = prec_age(rec.w) == 5;
        int victims[8], kv[8];
        int ksum = 0;
        // household: offset + r % count, the household table is the identity
        const int hoff = (int)rec.x, hcnt = prec_household_size(rec.w);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            kv[j] = select_victim(me, hoff, hcnt, w[j], true, nullptr, victims[j]);
            ksum += kv[j];
        }
        // workplace or school: max-contacts of its type
        const int woff = (int)rec.y, wcnt = (int)rec.z;
        const int desired = prec_desired(rec.w);
        // errands / afterschool: destinations from today's keys; the adult
        // profile is regenerated from the schedule counter (:3667-3705)
        const int32_t *kk = a.keys + ik.kbase;
        const int dest[2] = {kk[lme], kk[c.N + lme]};
        int prof = 3;
        if (adult) {
            uint32_t e[4];
            tf2x64(key, s.errand_offset + (uint64_t)(lme / 2), e);
            const int slot = 2 * (lme % 2);
            prof = (int)((e[slot] ^ e[slot + 1]) % 3u);
        }
        int made = 3;
        uint32_t wvoid = 0;  // contact slots voided by interventions
#pragma unroll
        for (int j = 3; j < 8; j++) {
            victims[j] = -1;
            kv[j] = 0;
        }
#pragma unroll
        for (int j = 3; j < 6; j++) {
            if (j - 3 < desired) {
                kv[j] = select_victim(me, woff, wcnt, w[j], false, a.wp_people, victims[j]);
                ksum += kv[j];
            }
        }
        made += desired;
        // interventions: a closed school or an absent adult voids the workplace / school
        // contacts; they keep their share of ksum, so the contact does not happen
        // rather than passing its weight to the others
        if (desired > 0 && (ik.absent_thr != 0 || (day >= ik.closure_start && day < ik.closure_end))) {
            const bool closed = day >= ik.closure_start && day < ik.closure_end && prec_school(rec.w);
            const bool me_absent =
                adult && intervention_hash(c.key0, c.key1, kTagAbsent, day, lme) < ik.absent_thr;
#pragma unroll
            for (int j = 3; j < 6; j++) {
                if (j - 3 < desired && kv[j] != 0) {
                    const int v = victims[j];
                    const bool v_absent = ik.absent_thr != 0 && a.age[v] == 5 &&
                                          intervention_hash(c.key0, c.key1, kTagAbsent, day, v - ik.pbase) <
                                              ik.absent_thr;
                    if (closed || me_absent || v_absent) wvoid |= 1u << j;
                }
            }
        }
#pragma unroll
        for (int hour = 0; hour < 2; hour++) {
            int want = c_weekday_assign[prof][hour];
            const int eoff = a.bkt_offset[dest[hour]], ecnt = a.bkt_offset[dest[hour] + 1] - eoff;
#pragma unroll
            for (int j = 3; j < 8; j++) {
                if (j == made && want > 0) {
                    kv[j] = select_victim(me, eoff, ecnt, w[j], false, a.bkt_people, victims[j]);
                    ksum += kv[j];
                    want--;
                    made++;
                }
            }
        }
        infector_state(c, inf, a.state[me], a.gen_p, a.gen_s, day, ksum);
#pragma unroll
        for (int j = 3; j < 6; j++)
            if ((wvoid >> j) & 1u) kv[j] = 0;
        process_contacts<8>(c, key, inf, ctr + 2, victims, kv, a.state, a.claim, a.new_list, sc);
    }
}

// kernel_doWeekend + device_makeContacts_weekend (PandemicSim.cu:3311-3379, :1833-1950)
__global__ void __launch_bounds__(128) k_infect_weekend(InfectArgs a, int day)
{
    Scalars *sc = a.sc;
    if (sc->done) return;
    const int I = sc->infected;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < I; pos += gridDim.x * blockDim.x) {
        const int inst = a.infected_inst[pos];
        const InstConst &ik = a.ic[inst];
        const SimConst &c = ik.c;
        const InstState &s = a.is[inst];
        const TfKey key = make_key(c);
        Infector inf;
        inf.pos = pos;
        inf.me = a.infected[pos];
        const int me = inf.me;
        const int lme = me - ik.pbase;
        const unsigned long long ctr = s.infect_offset + 6ull * (unsigned long long)(pos - s.start);
        const uint4 rec = load_record(a.prec, me);
        uint32_t w[4];
        tf2x64(key, ctr, w);
        int victims[5], kv[5];
        int ksum = 0;
        const int hoff = (int)rec.x, hcnt = prec_household_size(rec.w);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            kv[j] = select_victim(me, hoff, hcnt, w[j], true, nullptr, victims[j]);
            ksum += kv[j];
        }
        const int prof = (int)(w[3] % 6u);
        // Threefry-2x32 on the low seed words with counter (u32)(ctr + 1) (:1895-1901)
        uint32_t v2[2];
        tf2x32(key, (uint32_t)(ctr + 1), v2);
        const int32_t *k3 = a.keys + ik.kbase + 3 * (size_t)lme;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int loc = k3[c_weekend_assign[prof][j]];
            const int eoff = a.bkt_offset[loc], ecnt = a.bkt_offset[loc + 1] - eoff;
            kv[3 + j] = select_victim(me, eoff, ecnt, v2[j], false, a.bkt_people, victims[3 + j]);
            ksum += kv[3 + j];
        }
        infector_state(c, inf, a.state[me], a.gen_p, a.gen_s, day, ksum);
        process_contacts<5>(c, key, inf, ctr + 2, victims, kv, a.state, a.claim, a.new_list, sc);
    }
}

// ---------------------------------------------------- warp-cooperative contacts
// The same draws with eight lanes per infector (four infectors per warp round).  Lane
// j of a group first computes one Threefry block of the infector's draws, all in
// parallel:
//   weekday  j = 0, 1: contact words (counters R + 6 pos, +1); j = 2..5: infection
//            words (+2..+5); j = 6: the schedule block of the adult's errand profile
//   weekend  j = 0: contact words; j = 1: the Threefry-2x32 errand block; j = 2..5:
//            infection words
// then picks contact slot j's victim (its own gather chain) and draws slot j's two
// infections.  The words reach the lanes that use them by shuffles; the contact sum
// is a shuffle reduction over the group.  Every draw, victim and claim key equals the
// one-thread-per-infector kernels' (same counters, same words, same slots).
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t pick4(int i, uint32_t q0, uint32_t q1, uint32_t q2, uint32_t q3)
{
    return i == 0 ? q0 : (i == 1 ? q1 : (i == 2 ? q2 : q3));
}

// Slot j's infection draws: words W[2j], W[2j+1], W[(2j+2) & 15] of the four
// infection blocks, which lanes 2..5 of the group hold.
__device__ __forceinline__ void infection_words(const uint32_t blk[4], int gl, int j, uint32_t &w0, uint32_t &w1,
                                                uint32_t &w2)
{
    const int sa = gl + 2 + (j >> 1), sb = gl + 2 + (((j + 1) & 7) >> 1);
    const uint32_t a0 = __shfl_sync(kFull, blk[0], sa), a1 = __shfl_sync(kFull, blk[1], sa);
    const uint32_t a2 = __shfl_sync(kFull, blk[2], sa), a3 = __shfl_sync(kFull, blk[3], sa);
    const uint32_t b0 = __shfl_sync(kFull, blk[0], sb), b2 = __shfl_sync(kFull, blk[2], sb);
    w0 = (j & 1) ? a2 : a0;
    w1 = (j & 1) ? a3 : a1;
    w2 = ((j + 1) & 1) ? b2 : b0;
}

// Slot j's two infection draws against its victim (process_contacts for one slot).
__device__ __forceinline__ void claim_slot(const SimConst &c, const InfectArgs &a, int pos, int j, int me, int victim,
                                           int kv, const float prob[2], uint32_t w0, uint32_t w1, uint32_t w2)
{
    const float kf = __int2float_rn(kv);
#pragma unroll
    for (int strain = 0; strain < 2; strain++) {
        const float y = to_unit(strain ? w1 : w0);
        if (y < __fmul_rn(prob[strain], kf)) {
            const uint32_t st = a.state[victim];
            const uint32_t vstatus = strain ? ((st >> 8) & 0xFFu) : (st & 0xFFu);
            if (vstatus == 1u) {
                const int profile = infection_profile(c, strain ? (w1 ^ w2) : (w0 ^ w1));
                const int gen = ((strain ? a.gen_s[me] : a.gen_p[me]) + 1) & 0xFF;
                const unsigned long long k = ((unsigned long long)((long long)pos * 8 + j) << 16) |
                                             ((unsigned long long)profile << 8) | (unsigned long long)gen;
                const unsigned long long old = atomicMin(&a.claim[2 * (size_t)victim + strain], k);
                if (old == ~0ull) a.new_list[atomicAdd(&a.sc->new_count, 1)] = 2 * victim + strain;
            }
        }
    }
}

// Infection probability of each strain (device_calculateInfectionProbability); -1
// when the strain is not infectious today.
__device__ __forceinline__ void infector_probs(const SimConst &c, uint32_t st, int day, int ksum, float prob[2])
{
#pragma unroll
    for (int strain = 0; strain < 2; strain++) {
        const uint32_t status = strain ? ((st >> 8) & 0xFFu) : (st & 0xFFu);
        const uint32_t dday = strain ? (st >> 24) : ((st >> 16) & 0xFFu);
        prob[strain] = -1.f;
        if (status >= 2u) {
            const int pd = day - (int)dday;
            if (pd >= 0 && pd < 10) prob[strain] = infection_probability(c, (int)status - 2, pd, strain, ksum);
        }
    }
}

template <bool WEEKEND>
__global__ void __launch_bounds__(256) k_infect_coop(InfectArgs a, int day)
{
    Scalars *sc = a.sc;
    if (sc->done) return;
    const int I = sc->infected;
    const int lane = threadIdx.x & 31, j = lane & 7, gl = lane & ~7;
    const int gwarp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int base = gwarp * 4; base < I; base += nwarps * 4) {   // warp-uniform
        const int pos0 = base + (lane >> 3);
        const bool act = pos0 < I;       // groups past the list's end shadow its last entry
        const int pos = act ? pos0 : I - 1;
        const int inst = a.infected_inst[pos];
        const InstConst &ik = a.ic[inst];
        const SimConst &c = ik.c;
        const InstState &s = a.is[inst];
        const int me = a.infected[pos];
        const int lme = me - ik.pbase;
        const unsigned long long ctr = s.infect_offset + 6ull * (unsigned long long)(pos - s.start);
        const TfKey key = make_key(c);
        const uint4 rec = load_record(a.prec, me);
        // one Threefry block per lane
        uint32_t blk[4] = {0u, 0u, 0u, 0u};
        if (WEEKEND && j == 1) {
            tf2x32(key, (uint32_t)(ctr + 1), blk);   // :1895-1901, counter truncated to 32 bits
        } else {
            const uint64_t cc = (!WEEKEND && j >= 6) ? s.errand_offset + (uint64_t)(lme / 2) : ctr + (uint64_t)j;
            tf2x64(key, cc, blk);
        }
        // contact words: W[j] of blocks R, R + 1 (weekday), W[j] of block R (weekend)
        const int csrc = WEEKEND ? gl : gl + (j >> 2);
        const uint32_t q0 = __shfl_sync(kFull, blk[0], csrc), q1 = __shfl_sync(kFull, blk[1], csrc);
        const uint32_t q2 = __shfl_sync(kFull, blk[2], csrc), q3 = __shfl_sync(kFull, blk[3], csrc);
        const uint32_t wc = pick4(j & 3, q0, q1, q2, q3);
        int victim = -1, kv = 0;
        const int hoff = (int)rec.x, hcnt = prec_household_size(rec.w);
        if (WEEKEND) {
            const int prof = (int)(q3 % 6u);   // word 3 of block R (:1892)
            const uint32_t v0 = __shfl_sync(kFull, blk[0], gl + 1), v1 = __shfl_sync(kFull, blk[1], gl + 1);
            if (j < 3) {
                kv = select_victim(me, hoff, hcnt, wc, true, nullptr, victim);
            } else if (j < 5) {
                const int loc = a.keys[ik.kbase + 3 * (size_t)lme + c_weekend_assign[prof][j - 3]];
                const int eoff = a.bkt_offset[loc], ecnt = a.bkt_offset[loc + 1] - eoff;
                kv = select_victim(me, eoff, ecnt, j == 3 ? v0 : v1, false, a.bkt_people, victim);
            }
        } else {
            const bool adult = prec_age(rec.w) == 5;
            const int desired = prec_desired(rec.w);
            // the adult's errand profile from the schedule block on lane 6 (:3697-3702)
            const int pv = (j == 6) ? (int)(((lme & 1) ? (blk[2] ^ blk[3]) : (blk[0] ^ blk[1])) % 3u) : 0;
            const int pv6 = __shfl_sync(kFull, pv, gl + 6);   // every lane takes part in the shuffle
            const int prof = adult ? pv6 : 3;
            if (j < 3) {
                kv = select_victim(me, hoff, hcnt, wc, true, nullptr, victim);
            } else if (j < 3 + desired) {
                kv = select_victim(me, (int)rec.y, (int)rec.z, wc, false, a.wp_people, victim);
            } else {
                const int e = j - 3 - desired, want0 = c_weekday_assign[prof][0], want1 = c_weekday_assign[prof][1];
                const int hour = e < want0 ? 0 : (e < want0 + want1 ? 1 : -1);
                if (hour >= 0) {
                    const int dest = a.keys[ik.kbase + (size_t)hour * c.N + lme];
                    const int eoff = a.bkt_offset[dest], ecnt = a.bkt_offset[dest + 1] - eoff;
                    kv = select_victim(me, eoff, ecnt, wc, false, a.bkt_people, victim);
                }
            }
        }
        // the contact sum over the group's slots
        int ksum = kv;
        ksum += __shfl_xor_sync(kFull, ksum, 4);
        ksum += __shfl_xor_sync(kFull, ksum, 2);
        ksum += __shfl_xor_sync(kFull, ksum, 1);
        if (!WEEKEND && j >= 3 && j < 3 + prec_desired(rec.w) && kv != 0 &&
            (ik.absent_thr != 0 || (day >= ik.closure_start && day < ik.closure_end))) {
            // interventions void a workplace / school contact after it counted in ksum
            const bool closed = day >= ik.closure_start && day < ik.closure_end && prec_school(rec.w);
            const bool me_absent = prec_age(rec.w) == 5 &&
                                   intervention_hash(c.key0, c.key1, kTagAbsent, day, lme) < ik.absent_thr;
            const bool v_absent = ik.absent_thr != 0 && a.age[victim] == 5 &&
                                  intervention_hash(c.key0, c.key1, kTagAbsent, day, victim - ik.pbase) <
                                      ik.absent_thr;
            if (closed || me_absent || v_absent) kv = 0;
        }
        float prob[2];
        infector_probs(c, a.state[me], day, ksum, prob);
        uint32_t w0, w1, w2;
        infection_words(blk, gl, j, w0, w1, w2);
        if (act && kv != 0 && j < (WEEKEND ? 5 : 8)) claim_slot(c, a, pos, j, me, victim, kv, prob, w0, w1, w2);
    }
}

cudaError_t launch_infect(const DevArrays &d, bool weekend, int day, cudaStream_t s)
{
    InfectArgs a;
    a.ic = d.ic; a.is = d.is;
    a.state = d.state; a.gen_p = d.gen_p; a.gen_s = d.gen_s; a.age = d.age;
    a.prec = d.prec;
    a.wp_people = d.wp_people; a.keys = d.keys;
    a.bkt_offset = d.bkt_offset; a.bkt_people = d.bkt_people; a.infected = d.infected;
    a.infected_inst = d.infected_inst;
    a.claim = d.claim; a.new_list = d.new_list; a.sc = d.sc;
    const Tuning &t = d.tune;
    if (t.infect_coop) {
        const int blocks = sm_count() * t.infect_blocks_per_sm;
        if (weekend) k_infect_coop<true><<<blocks, 256, 0, s>>>(a, day);
        else k_infect_coop<false><<<blocks, 256, 0, s>>>(a, day);
    } else {
        const int blocks = sm_count() * t.infect_blocks_per_sm * 2;   // blocks of 128 threads
        if (weekend) k_infect_weekend<<<blocks, 128, 0, s>>>(a, day);
        else k_infect_weekday<<<blocks, 128, 0, s>>>(a, day);
    }
    count_launch();
    return cudaGetLastError();
}

// device_setInfectionStatus (PandemicSim.cu:3048-3067) for the winning claims:
// status = profile, day = today + 1 (8-bit), generation = infector's + 1.
__global__ void k_apply(uint32_t *state, uint8_t *gen_p, uint8_t *gen_s, unsigned long long *claim,
                        const int32_t *new_list, Scalars *sc, int day)
{
    if (sc->done) return;
    const int n = sc->new_count;
    const uint32_t dset = (uint32_t)((day + 1) & 0xFF);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = new_list[i];
        const int v = e >> 1, strain = e & 1;
        unsigned long long *cp = &claim[2 * (size_t)v + strain];
        const unsigned long long cl = *cp;
        *cp = ~0ull;
        const uint32_t profile = (uint32_t)(cl >> 8) & 0xFFu;
        const uint8_t gen = (uint8_t)(cl & 0xFFu);
        const uint32_t sshift = strain ? 8 : 0, dshift = strain ? 24 : 16;
        uint32_t old = state[v], assumed;
        do {
            assumed = old;
            uint32_t nw = (assumed & ~((0xFFu << sshift) | (0xFFu << dshift))) | (profile << sshift) | (dset << dshift);
            old = atomicCAS(&state[v], assumed, nw);
        } while (old != assumed);
        if (strain) gen_s[v] = gen;
        else gen_p[v] = gen;
    }
}

cudaError_t launch_apply(const DevArrays &d, int day, cudaStream_t s)
{
    k_apply<<<sm_count() * 8, 256, 0, s>>>(d.state, d.gen_p, d.gen_s, d.claim, d.new_list, d.sc, day);
    count_launch();
    return cudaGetLastError();
}

// ================================================================== bounded-wait probe
// The look-back wait above, in isolation: one warp plays tile 1 of a fresh look-back
// (epoch 1, words zeroed by the host) and waits for tile 0.  With publish_first the
// warp writes tile 0's inclusive prefix (1234) before waiting, and the wait returns it
// at once.  Without it nothing ever writes tile 0's word: the wait polls spin_limit
// times, records the error word and returns, and the kernel ends normally.
__global__ void k_wait_probe(LookBack lb, int publish_first, long long spin_limit, unsigned *prefix_out)
{
    constexpr unsigned kEpoch = 1;
    if (publish_first && threadIdx.x == 0) {
        *(volatile unsigned long long *)&lb.tiles[0] = lb_word(kEpoch, 2, 1234u);
        __threadfence();
    }
    __syncwarp();
    const unsigned excl = lookback_publish_warp(lb, kEpoch, 1, 5u, false, spin_limit);
    if (threadIdx.x == 0) *prefix_out = excl;
}

cudaError_t launch_wait_probe(unsigned long long *tiles, int *error, int publish_first, long long spin_limit,
                              unsigned *prefix_out, cudaStream_t s)
{
    LookBack lb;
    lb.tiles = tiles;
    lb.ctl = nullptr;   // the probe takes no ticket
    lb.error = error;
    k_wait_probe<<<1, 32, 0, s>>>(lb, publish_first, spin_limit, prefix_out);
    count_launch();
    return cudaGetLastError();
}

long long max_spin_limit() { return kSpinLimit; }

// ================================================================== errand-lookup self-test
// The schedule kernels' branch-free errand search (errand_row) against the reference's
// loop and IEEE division (errand_row_loop), on every 32-bit random word the schedule
// can draw: counts[0] weekday and counts[1] weekend words whose row or quotient bits
// differ.  counts[2]: floats x in the domain the search divides, 0 and [2^-32, 1]
// (a draw is 0 or at least 2^-32, a remainder after a subtraction at least 2^-28), and
// errand rows r in {9, 11, 12, 13} of both tables where div_rn_recip(x, pdf[r], rcp[r])
// differs from __fdiv_rn(x, pdf[r]).  (Below about 2^-100 the correction step's
// remainder underflows and the two can differ; no draw gets there.)  counts[3]:
// reciprocal table entries that differ from __frcp_rn of their probability.
__global__ void k_errand_selftest(unsigned long long *counts)
{
    unsigned long long bad_wd = 0, bad_we = 0, bad_div = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32);
         i += stride) {
        const float y = to_unit((uint32_t)i);
        float a, b;
        int ra = errand_row<false>(y, a), rb = errand_row_loop<false>(y, b);
        bad_wd += (ra != rb || __float_as_uint(a) != __float_as_uint(b)) ? 1 : 0;
        ra = errand_row<true>(y, a);
        rb = errand_row_loop<true>(y, b);
        bad_we += (ra != rb || __float_as_uint(a) != __float_as_uint(b)) ? 1 : 0;
        if (i == 0 || (i >= 0x2F800000ull && i <= 0x3F800000ull)) {   // 0 and [2^-32, 1]
            const float x = __uint_as_float((uint32_t)i);
            const int rows[4] = {9, 11, 12, 13};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int r = rows[k];
                bad_div += __float_as_uint(div_rn_recip(x, c_weekday_errand_pdf[r], c_weekday_errand_rcp[r])) !=
                                   __float_as_uint(__fdiv_rn(x, c_weekday_errand_pdf[r]))
                               ? 1
                               : 0;
                bad_div += __float_as_uint(div_rn_recip(x, c_weekend_errand_pdf[r], c_weekend_errand_rcp[r])) !=
                                   __float_as_uint(__fdiv_rn(x, c_weekend_errand_pdf[r]))
                               ? 1
                               : 0;
            }
        }
    }
    if (bad_wd) atomicAdd(&counts[0], bad_wd);
    if (bad_we) atomicAdd(&counts[1], bad_we);
    if (bad_div) atomicAdd(&counts[2], bad_div);
    if (blockIdx.x == 0 && threadIdx.x < kTypes) {
        const int t = threadIdx.x;
        unsigned long long bad = 0;
        if (c_weekday_errand_pdf[t] > 0.f && c_weekday_errand_rcp[t] != __frcp_rn(c_weekday_errand_pdf[t])) bad++;
        if (c_weekend_errand_pdf[t] > 0.f && c_weekend_errand_rcp[t] != __frcp_rn(c_weekend_errand_pdf[t])) bad++;
        if (bad) atomicAdd(&counts[3], bad);
    }
}

cudaError_t launch_errand_selftest(unsigned long long *counts, cudaStream_t s)
{
    k_errand_selftest<<<sm_count() * 8, 256, 0, s>>>(counts);
    count_launch();
    return cudaGetLastError();
}

// ================================================================== final
// final_countReproduction's generation counts (PandemicSim.cu:2227-2304) for every
// instance: one block per person tile, histogram in shared memory.
__global__ void k_gen_hist(const InstConst *ic, const int32_t *tile_inst, const uint8_t *gen_p, const uint8_t *gen_s,
                           int *hist)
{
    __shared__ int h[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int k = tile_inst[blockIdx.x];
    const long long first = (long long)blockIdx.x * kPersonTile;
    const long long end = (long long)ic[k].pbase + ic[k].c.N;
    for (long long i = first + threadIdx.x; i < first + kPersonTile && i < end; i += blockDim.x) {
        atomicAdd(&h[gen_p[i]], 1);
        atomicAdd(&h[256 + gen_s[i]], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[(size_t)k * 512 + i], h[i]);
}

cudaError_t launch_gen_hist(const DevArrays &d, int *hist, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)d.K * 512 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_gen_hist<<<d.P / kPersonTile, 256, 0, s>>>(d.ic, d.tile_inst, d.gen_p, d.gen_s, hist);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ptk
