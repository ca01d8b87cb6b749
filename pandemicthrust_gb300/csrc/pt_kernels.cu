// pt_kernels.cu - sm_103a kernels of the PandemicThrust daily simulation step.
//
// Stage map (reference = PandemicThrust/PandemicThrust/PandemicSim.cu):
//   setup   household types/sizes, household scan+scatter, workplace/school draw,
//           workplace buckets                         (setupSim, :146-208)
//   sweep   recover + 16 status bins + ordered infected list, one pass
//           (kernel_countInfectedStatusAndRecover :2097-2192 + copy_if :2207-2224)
//   sched   schedule keys + bucket histogram          (:2972-3022 / :2082-2094)
//   bucket  scan, scatter, per-bucket sort by person id (CUB sort + lower_bound,
//           :1212-1248 / :1313-1354)
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

namespace ptk {

static std::atomic<uint64_t> g_launches{0};
uint64_t launches() { return g_launches.load(); }
void add_launches(int64_t n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
static inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

static inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

constexpr long long kSpinLimit = 1ll << 22;

// ------------------------------------------------------------------ look-back
// Tile status word: bits 63..34 epoch, 33..32 flag (1 aggregate, 2 inclusive
// prefix), 31..0 value.  The epoch makes words of earlier launches stale without a
// memset: the last block to finish a launch increments it and resets the tickets.
struct LookBack {
    unsigned long long *tiles;
    int *ctl;   // ctl[0] ticket, ctl[1] finished, ctl[2] epoch
    int *error;
};

__device__ __forceinline__ unsigned long long lb_word(unsigned epoch, unsigned flag, unsigned value)
{
    return ((unsigned long long)epoch << 34) | ((unsigned long long)flag << 32) | value;
}

// Called by one thread.  Publishes the tile aggregate, walks back to the nearest
// inclusive prefix, publishes the tile's inclusive prefix and returns the exclusive one.
__device__ unsigned lookback_publish(const LookBack &lb, unsigned epoch, int tile, unsigned aggregate)
{
    volatile unsigned long long *t = lb.tiles;
    if (tile == 0) {
        t[0] = lb_word(epoch, 2, aggregate);
        return 0;
    }
    t[tile] = lb_word(epoch, 1, aggregate);
    unsigned excl = 0;
    int j = tile - 1;
    long long spins = 0;
    while (j >= 0) {
        unsigned long long w = t[j];
        unsigned ep = (unsigned)(w >> 34);
        unsigned flag = (unsigned)(w >> 32) & 3u;
        if (ep != (epoch & 0x3FFFFFFFu) || flag == 0) {
            if (++spins > kSpinLimit) {
                atomicExch(lb.error, 1);
                break;
            }
            __nanosleep(64);
            continue;
        }
        excl += (unsigned)w;
        if (flag == 2) break;
        j--;
    }
    t[tile] = lb_word(epoch, 2, excl + aggregate);
    return excl;
}

// Start of a look-back launch: returns the tile index and epoch (broadcast).
__device__ __forceinline__ void lookback_begin(const LookBack &lb, int &tile, unsigned &epoch)
{
    __shared__ int s_tile;
    __shared__ unsigned s_epoch;
    if (threadIdx.x == 0) {
        s_tile = atomicAdd(&lb.ctl[0], 1);
        s_epoch = (unsigned)(*(volatile int *)&lb.ctl[2]) & 0x3FFFFFFFu;
    }
    __syncthreads();
    tile = s_tile;
    epoch = s_epoch;
}

// End of a look-back launch: the last block resets the ticket and bumps the epoch.
__device__ __forceinline__ void lookback_end(const LookBack &lb)
{
    if (threadIdx.x == 0) {
        __threadfence();
        int fin = atomicAdd(&lb.ctl[1], 1);
        if (fin == (int)gridDim.x - 1) {
            lb.ctl[0] = 0;
            lb.ctl[1] = 0;
            atomicAdd(&lb.ctl[2], 1);
            __threadfence();
        }
    }
}

// ------------------------------------------------------------------ block scan
template <int THREADS, typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T &total)
{
    static_assert(THREADS % 32 == 0, "");
    constexpr int W = THREADS / 32;
    __shared__ T s_warp[W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < W ? s_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < W) s_warp[lane] = w;
    }
    __syncthreads();
    T warp_prefix = warp > 0 ? s_warp[warp - 1] : T(0);
    total = s_warp[W - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// ================================================================== setup
// kernel_householdTypeAssignment + hh_peopleCount_functor (PandemicSim.cu:2329-2357,
// :3579-3605): counter g -> households 4g..4g+3.  Writes each household's size and
// counts adults.
__global__ void k_household_types(SimConst c, uint8_t *types, int32_t *sizes, int *adults)
{
    const TfKey key = make_key(c);
    int local_adults = 0;
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
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local_adults += __shfl_xor_sync(0xffffffffu, local_adults, o);
    if ((threadIdx.x & 31) == 0 && local_adults) atomicAdd(adults, local_adults);
}

cudaError_t launch_household_types(const SimConst &c, uint8_t *types, int32_t *sizes, int *adults,
                                   cudaStream_t s)
{
    int G = c.H / 4 + 1;
    int blocks = std::min(div_up(G, 256), sm_count() * 16);
    k_household_types<<<blocks, 256, 0, s>>>(c, types, sizes, adults);
    count_launch();
    return cudaGetLastError();
}

// Generic exclusive scan (single pass, decoupled look-back): out[i] = sum in[0..i),
// out[n] = total.  With clear_in the input is zeroed after it is read.
constexpr int kScanThreads = 256, kScanItems = 16, kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) k_scan(const int32_t *in, int32_t *out, int n, int clear_in,
                                                       LookBack lb, const int *skip)
{
    if (skip && *(volatile const int *)skip) return;
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
        sum += v[k];
    }
    if (clear_in) {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            long long i = base + k;
            if (i < n) ((int32_t *)in)[i] = 0;
        }
    }
    int total;
    int excl = block_exclusive_scan<kScanThreads, int>(sum, total);
    __shared__ unsigned s_prefix;
    if (threadIdx.x == 0) s_prefix = lookback_publish(lb, epoch, tile, (unsigned)total);
    __syncthreads();
    int run = (int)s_prefix + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (tile == (int)gridDim.x - 1 && threadIdx.x == 0) out[n] = (int)s_prefix + total;
    lookback_end(lb);
}

// The look-back control block sits right after the tile words.
static LookBack make_lb(unsigned long long *tiles, int tiles_cap, int *error)
{
    LookBack lb;
    lb.tiles = tiles;
    lb.ctl = (int *)(tiles + tiles_cap);
    lb.error = error;
    return lb;
}

cudaError_t launch_scan_exclusive(const int32_t *in, int32_t *out, int n, int clear_in,
                                  unsigned long long *tiles, int *ticket, int *error,
                                  const int *skip, cudaStream_t s)
{
    (void)ticket;
    int blocks = std::max(1, div_up(n, kScanTile));
    LookBack lb;
    lb.tiles = tiles;
    lb.ctl = ticket;
    lb.error = error;
    k_scan<<<blocks, kScanThreads, 0, s>>>(in, out, n, clear_in, lb, skip);
    count_launch();
    return cudaGetLastError();
}

// kernel_generateHouseholds (PandemicSim.cu:2490-2531): adults first (AGE_ADULT),
// then children with the AGE_5 placeholder.
__global__ void k_generate_households(SimConst c, const uint8_t *types, const int32_t *hh_offset,
                                      int32_t *household, uint8_t *age)
{
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < c.H; h += gridDim.x * blockDim.x) {
        int t = types[h];
        int off = hh_offset[h];
        int na = c_hh_adults[t], nc = c_hh_children[t];
        for (int i = 0; i < na + nc; i++) {
            household[off + i] = h;
            age[off + i] = i < na ? 5 : 0;
        }
    }
}

cudaError_t launch_generate_households(const SimConst &c, const uint8_t *types, const int32_t *hh_offset,
                                       int32_t *household, uint8_t *age, cudaStream_t s)
{
    int blocks = std::min(div_up(c.H, 256), sm_count() * 16);
    k_generate_households<<<blocks, 256, 0, s>>>(c, types, hh_offset, household, age);
    count_launch();
    return cudaGetLastError();
}

// assignWorkplaceFunctor (PandemicSim.cu:3750-3778): counter W0 + g -> persons
// 4g..4g+3; adults draw a workplace, children an age band and school.
__global__ void k_assign_workplaces(SimConst c, uint8_t *age, int32_t *workplace)
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
                    workplace[p] = fish_workplace(c, w[i]);
                } else {
                    workplace[p] = fish_school_and_age(c, w[i], &a);
                    age[p] = (uint8_t)a;
                }
            }
        }
    }
}

cudaError_t launch_assign_workplaces(const SimConst &c, uint8_t *age, int32_t *workplace, cudaStream_t s)
{
    int blocks = std::min(div_up(c.N / 4 + 1, 256), sm_count() * 16);
    k_assign_workplaces<<<blocks, 256, 0, s>>>(c, age, workplace);
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

// Unordered scatter; the per-bucket sort that follows fixes the order.  The
// cursor (the histogram) counts down to zero, so it is clean for the next build.
__global__ void k_scatter_identity(const int32_t *keys, int n, const int32_t *offset, int32_t *cursor,
                                   int32_t *out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int k = keys[i];
        int pos = offset[k] + atomicSub(&cursor[k], 1) - 1;
        out[pos] = i;
    }
}

cudaError_t launch_scatter_identity(const int32_t *keys, int n, const int32_t *offset, int32_t *cursor,
                                    int32_t *out, cudaStream_t s)
{
    int blocks = std::min(div_up(n, 256), sm_count() * 16);
    k_scatter_identity<<<std::max(blocks, 1), 256, 0, s>>>(keys, n, offset, cursor, out);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ bucket sort
// Buckets list person ids; the reference's stable sort leaves each bucket in
// ascending id order and ids are unique within a bucket, so sorting each bucket
// reproduces it exactly.  Size classes: <=16 one thread, <=1024 one warp (bitonic
// in shared memory), larger one block (bitonic up to kBigSmem ids, then merges).
constexpr int kSmallMax = 16, kMidMax = 1024, kBigSmem = 16384;

__global__ void k_sort_classify(const int32_t *offset, int buckets, int32_t *people, int32_t *mid_list,
                                int32_t *big_list, Scalars *sc, const int *skip)
{
    if (skip && *(volatile const int *)skip) return;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < buckets; b += gridDim.x * blockDim.x) {
        int o = offset[b];
        int n = offset[b + 1] - o;
        if (n <= 1) continue;
        if (n <= kSmallMax) {
            int v[kSmallMax];
#pragma unroll
            for (int i = 0; i < kSmallMax; i++) v[i] = i < n ? people[o + i] : INT_MAX;
            // odd-even transposition network on 16 registers
#pragma unroll
            for (int r = 0; r < kSmallMax; r++) {
#pragma unroll
                for (int i = (r & 1); i + 1 < kSmallMax; i += 2) {
                    int a = v[i], bb = v[i + 1];
                    v[i] = min(a, bb);
                    v[i + 1] = max(a, bb);
                }
            }
#pragma unroll
            for (int i = 0; i < kSmallMax; i++)
                if (i < n) people[o + i] = v[i];
        } else if (n <= kMidMax) {
            mid_list[atomicAdd(&sc->mid_count, 1)] = b;
        } else {
            big_list[atomicAdd(&sc->big_count, 1)] = b;
        }
    }
}

__device__ __forceinline__ int next_pow2(int n)
{
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

constexpr int kMidWarps = 8;

__global__ void __launch_bounds__(kMidWarps * 32) k_sort_mid(const int32_t *offset, int32_t *people,
                                                             const int32_t *mid_list, const Scalars *sc,
                                                             const int *skip)
{
    if (skip && *(volatile const int *)skip) return;
    __shared__ int s_buf[kMidWarps][kMidMax];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int *buf = s_buf[warp];
    const int count = sc->mid_count;
    for (int item = blockIdx.x * kMidWarps + warp; item < count; item += gridDim.x * kMidWarps) {
        int b = mid_list[item];
        int o = offset[b];
        int n = offset[b + 1] - o;
        int P = next_pow2(n);
        for (int i = lane; i < P; i += 32) buf[i] = i < n ? people[o + i] : INT_MAX;
        __syncwarp();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < P; i += 32) {
                    int ixj = i ^ j;
                    if (ixj > i) {
                        int a = buf[i], c = buf[ixj];
                        bool up = (i & k) == 0;
                        if ((a > c) == up) {
                            buf[i] = c;
                            buf[ixj] = a;
                        }
                    }
                }
                __syncwarp();
            }
        }
        for (int i = lane; i < n; i += 32) people[o + i] = buf[i];
        __syncwarp();
    }
}

constexpr int kBigThreads = 1024;

__device__ void block_bitonic(int *buf, int P)
{
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                int ixj = i ^ j;
                if (ixj > i) {
                    int a = buf[i], c = buf[ixj];
                    bool up = (i & k) == 0;
                    if ((a > c) == up) {
                        buf[i] = c;
                        buf[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Rank of x among sorted distinct values r[0..m): number of elements < x.
__device__ __forceinline__ int lower_rank(const int32_t *r, int m, int x)
{
    int lo = 0, hi = m;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (r[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kBigThreads) k_sort_big(const int32_t *offset, int32_t *people, int32_t *tmp,
                                                          const int32_t *big_list, const Scalars *sc,
                                                          const int *skip)
{
    if (skip && *(volatile const int *)skip) return;
    extern __shared__ int s_big[];
    const int count = sc->big_count;
    for (int item = blockIdx.x; item < count; item += gridDim.x) {
        int b = big_list[item];
        int o = offset[b];
        int n = offset[b + 1] - o;
        int32_t *a = people + o;
        // sort chunks of kBigSmem in shared memory
        for (int c0 = 0; c0 < n; c0 += kBigSmem) {
            int m = min(kBigSmem, n - c0);
            int P = next_pow2(m);
            for (int i = threadIdx.x; i < P; i += blockDim.x) s_big[i] = i < m ? a[c0 + i] : INT_MAX;
            __syncthreads();
            block_bitonic(s_big, P);
            for (int i = threadIdx.x; i < m; i += blockDim.x) a[c0 + i] = s_big[i];
            __syncthreads();
        }
        // merge runs pairwise: each element's output index is its own index plus its
        // rank in the partner run (values are distinct).
        int32_t *t = tmp + o;
        for (int w = kBigSmem; w < n; w <<= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                int run = i / w;
                int start = run * w;
                int pstart, plen, base;
                if ((run & 1) == 0) {
                    pstart = start + w;
                    plen = max(0, min(w, n - pstart));
                    base = start;
                } else {
                    pstart = start - w;
                    plen = w;
                    base = pstart;
                }
                int own = i - start;
                int r = plen > 0 ? lower_rank(a + pstart, plen, a[i]) : 0;
                t[base + own + r] = a[i];
            }
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = t[i];
            __syncthreads();
        }
    }
}

cudaError_t launch_sort_buckets(const int32_t *offset, int buckets, int32_t *people, int32_t *tmp,
                                int32_t *mid_list, int32_t *big_list, Scalars *sc, const int *skip,
                                cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(&sc->mid_count, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    int blocks = std::max(1, std::min(div_up(buckets, 256), sm_count() * 32));
    k_sort_classify<<<blocks, 256, 0, s>>>(offset, buckets, people, mid_list, big_list, sc, skip);
    count_launch();
    k_sort_mid<<<sm_count() * 4, kMidWarps * 32, 0, s>>>(offset, people, mid_list, sc, skip);
    count_launch();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sort_big, cudaFuncAttributeMaxDynamicSharedMemorySize, kBigSmem * (int)sizeof(int));
        attr = true;
    }
    k_sort_big<<<sm_count(), kBigThreads, kBigSmem * sizeof(int), s>>>(offset, people, tmp, big_list, sc, skip);
    count_launch();
    return cudaGetLastError();
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

// ================================================================== day
// Sweep: one tile of 4096 persons per block; each thread holds 4 rounds of 4
// persons (one 16-byte load per round).  Output order is (round, thread, item),
// which is ascending person order within the tile.
constexpr int kSweepThreads = 256, kSweepRounds = 4, kSweepTile = kSweepThreads * 4 * kSweepRounds;

__device__ __forceinline__ uint32_t recover_word(uint32_t st, int d2r, bool &changed)
{
    uint32_t sp = st & 0xFFu, ss = (st >> 8) & 0xFFu, dp = (st >> 16) & 0xFFu, ds = st >> 24;
    uint32_t out = st;
    if (d2r >= 0 && sp >= 2u && (int)dp <= d2r) out &= ~0xFFu;
    if (d2r >= 0 && ss >= 2u && (int)ds <= d2r) out &= ~0xFF00u;
    changed = out != st;
    return out;
}

__global__ void __launch_bounds__(kSweepThreads) k_sweep(SimConst c, uint32_t *state, int32_t *infected,
                                                         Scalars *sc, LookBack lb, int day)
{
    if (*(volatile int *)&sc->done) return;
    int tile;
    unsigned epoch;
    lookback_begin(lb, tile, epoch);
    const int N = c.N;
    const int d2r = day - 10;
    const long long tile_base = (long long)tile * kSweepTile;
    // packed per-thread status bins: 16-bit fields, bins 0-3 / 4-7 per strain
    unsigned long long bp_lo = 0, bp_hi = 0, bs_lo = 0, bs_hi = 0;
    uint32_t flags = 0;  // bit (4*round + item)
    unsigned long long packed_counts = 0;
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
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            bool ch;
            out[j] = recover_word(st[j], d2r, ch);
            if (p0 + j < N) {
                any_changed |= ch;
                uint32_t sp = out[j] & 0xFFu, ss = (out[j] >> 8) & 0xFFu;
                if (sp < 4) bp_lo += 1ull << (16 * sp); else bp_hi += 1ull << (16 * (sp - 4));
                if (ss < 4) bs_lo += 1ull << (16 * ss); else bs_hi += 1ull << (16 * (ss - 4));
                if (sp >= 2u || ss >= 2u) {
                    flags |= 1u << (4 * r + j);
                    cnt++;
                }
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
        packed_counts |= (unsigned long long)cnt << (16 * r);
    }
    // status bins: warp reduction then one atomic per bin per warp
    __shared__ int s_bins[16];
    if (threadIdx.x < 16) s_bins[threadIdx.x] = 0;
    __syncthreads();
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
    // ordered compaction: scan the four per-round counts at once (16-bit fields)
    unsigned long long round_tot;
    unsigned long long excl = block_exclusive_scan<kSweepThreads, unsigned long long>(packed_counts, round_tot);
    unsigned tile_total = 0;
    unsigned round_base[kSweepRounds];
#pragma unroll
    for (int r = 0; r < kSweepRounds; r++) {
        round_base[r] = tile_total;
        tile_total += (unsigned)((round_tot >> (16 * r)) & 0xFFFF);
    }
    __shared__ unsigned s_prefix;
    if (threadIdx.x == 0) s_prefix = lookback_publish(lb, epoch, tile, tile_total);
    __syncthreads();
    const unsigned prefix = s_prefix;
#pragma unroll
    for (int r = 0; r < kSweepRounds; r++) {
        unsigned pos = prefix + round_base[r] + (unsigned)((excl >> (16 * r)) & 0xFFFF);
        long long p0 = tile_base + ((long long)r * kSweepThreads + threadIdx.x) * 4;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (flags & (1u << (4 * r + j))) infected[pos++] = (int32_t)(p0 + j);
        }
    }
    if (threadIdx.x < 16 && s_bins[threadIdx.x]) atomicAdd(&sc->counts[day][threadIdx.x], s_bins[threadIdx.x]);
    // the last tile closes the day's bookkeeping (runToCompletion, PandemicSim.cu:891-937)
    if (tile == (int)gridDim.x - 1 && threadIdx.x == 0) {
        const int I = (int)(prefix + tile_total);
        sc->infected = I;
        sc->infected_per_day[day] = I;
        sc->day = day;
        sc->days_run = day + 1;
        sc->new_count = 0;
        if (I == 0) {
            sc->done = 1;
        } else {
            const bool weekend = (day % 7) >= 5;
            unsigned long long E0 = sc->rand_offset;
            unsigned long long R0 = E0 + (weekend ? 2ull * (unsigned long long)N : (unsigned long long)(N / 2));
            sc->errand_offset = E0;
            sc->infect_offset = R0;
            sc->rand_offset = R0 + 6ull * (unsigned long long)I;
        }
    }
    lookback_end(lb);
}

cudaError_t launch_sweep(const SimConst &c, const DevArrays &d, int day, cudaStream_t s)
{
    int blocks = std::max(1, div_up(c.N, kSweepTile));
    LookBack lb = make_lb(d.tiles, d.tiles_cap, &d.sc->error);
    k_sweep<<<blocks, kSweepThreads, 0, s>>>(c, d.state, d.infected, d.sc, lb, day);
    count_launch();
    return cudaGetLastError();
}

// Weekday schedule (kernel_assignWeekdayAfterschoolAndErrands, PandemicSim.cu:2972-3022):
// counter E0 + g -> persons 2g, 2g+1.  Hour-0 keys at [0,N), hour-1 keys at [N,2N).
__global__ void k_sched_weekday(SimConst c, const uint8_t *age, int32_t *keys, int32_t *count, const Scalars *sc)
{
    if (sc->done) return;
    const TfKey key = make_key(c);
    const unsigned long long E0 = sc->errand_offset;
    const int N = c.N, G = N / 2;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x) {
        uint32_t w[4];
        tf2x64(key, E0 + (uint64_t)g, w);
#pragma unroll
        for (int k = 0; k < 2; k++) {
            int p = 2 * g + k;
            if (p < N) {
                bool adult = age[p] == 5;
                int d1 = fish_weekday_dest(c, w[2 * k], adult);
                int d2 = adult ? fish_weekday_dest(c, w[2 * k + 1], true) : d1;
                d2 += c.L;
                keys[p] = d1;
                keys[N + p] = d2;
                atomicAdd(&count[d1], 1);
                atomicAdd(&count[d2], 1);
            }
        }
    }
}

// Weekend schedule (kernel_assignWeekendErrands, PandemicSim.cu:2082-2094): person p
// uses counters E0 + 2p and E0 + 2p + 1; keys at [3p, 3p+3).
__global__ void k_sched_weekend(SimConst c, int32_t *keys, int32_t *count, const Scalars *sc)
{
    if (sc->done) return;
    const TfKey key = make_key(c);
    const unsigned long long E0 = sc->errand_offset;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < c.N; p += gridDim.x * blockDim.x) {
        int d[3];
        weekend_errands(c, key, E0 + 2ull * (unsigned long long)p, d);
        keys[3 * (size_t)p + 0] = d[0];
        keys[3 * (size_t)p + 1] = d[1];
        keys[3 * (size_t)p + 2] = d[2];
        atomicAdd(&count[d[0]], 1);
        atomicAdd(&count[d[1]], 1);
        atomicAdd(&count[d[2]], 1);
    }
}

cudaError_t launch_schedule(const SimConst &c, const DevArrays &d, bool weekend, cudaStream_t s)
{
    if (weekend) {
        int blocks = std::min(div_up(c.N, 256), sm_count() * 32);
        k_sched_weekend<<<std::max(1, blocks), 256, 0, s>>>(c, d.keys, d.bkt_count, d.sc);
    } else {
        int blocks = std::min(div_up(c.N / 2 + 1, 256), sm_count() * 32);
        k_sched_weekday<<<std::max(1, blocks), 256, 0, s>>>(c, d.age, d.keys, d.bkt_count, d.sc);
    }
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_bucket_scan(const SimConst &c, const DevArrays &d, bool weekend, cudaStream_t s)
{
    const int B = (weekend ? 10 : 2) * c.L;
    LookBack lb = make_lb(d.tiles, d.tiles_cap, &d.sc->error);
    int blocks = std::max(1, div_up(B, kScanTile));
    k_scan<<<blocks, kScanThreads, 0, s>>>(d.bkt_count, d.bkt_offset, B, 0, lb, &d.sc->done);
    count_launch();
    return cudaGetLastError();
}

__global__ void k_scatter_sched(const int32_t *keys, int N, int weekend, const int32_t *offset, int32_t *cursor,
                                int32_t *people, const Scalars *sc)
{
    if (sc->done) return;
    const long long E = (long long)(weekend ? 3 : 2) * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < E; e += (long long)gridDim.x * blockDim.x) {
        int k = keys[e];
        int person = weekend ? (int)(e / 3) : (int)(e < N ? e : e - N);
        int pos = offset[k] + atomicSub(&cursor[k], 1) - 1;
        people[pos] = person;
    }
}

cudaError_t launch_scatter_schedule(const SimConst &c, const DevArrays &d, bool weekend, cudaStream_t s)
{
    const long long E = (long long)(weekend ? 3 : 2) * c.N;
    int blocks = (int)std::min<long long>((E + 255) / 256, (long long)sm_count() * 32);
    k_scatter_sched<<<std::max(1, blocks), 256, 0, s>>>(d.keys, c.N, weekend ? 1 : 0, d.bkt_offset, d.bkt_count,
                                                        d.bkt_people, d.sc);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_sort_schedule(const SimConst &c, const DevArrays &d, bool weekend, cudaStream_t s)
{
    const int B = (weekend ? 10 : 2) * c.L;
    return launch_sort_buckets(d.bkt_offset, B, d.bkt_people, d.sort_tmp, d.mid_list, d.big_list, d.sc,
                               &d.sc->done, s);
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
    int me, pos;
    float prob[2];
    int gen[2];
};

// device_processContacts (PandemicSim.cu:3106-3233) with the claim rule: a
// successful draw on a victim whose strain status was susceptible at the start of
// the day claims (victim, strain) with key (position, slot); the smallest key wins.
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
    const uint32_t *state;
    const uint8_t *gen_p, *gen_s, *age;
    const int32_t *household, *hh_offset, *workplace, *wp_people, *wp_offset;
    const int32_t *keys, *bkt_offset, *bkt_people, *infected;
    unsigned long long *claim;
    int32_t *new_list;
    Scalars *sc;
};

// kernel_doWeekday + device_makeContacts_weekday (PandemicSim.cu:3236-3308, :1669-1829)
__global__ void __launch_bounds__(128) k_infect_weekday(SimConst c, InfectArgs a, int day)
{
    Scalars *sc = a.sc;
    if (sc->done) return;
    const TfKey key = make_key(c);
    const int I = sc->infected;
    const unsigned long long R0 = sc->infect_offset, E0 = sc->errand_offset;
    const int N = c.N;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < I; pos += gridDim.x * blockDim.x) {
        Infector inf;
        inf.pos = pos;
        inf.me = a.infected[pos];
        const int me = inf.me;
        const unsigned long long ctr = R0 + 6ull * (unsigned long long)pos;
        uint32_t w[8];
        tf2x64(key, ctr, w);
        tf2x64(key, ctr + 1, w + 4);
        const int age = a.age[me];
        const bool adult = age == 5;
        int victims[8], kv[8];
        int ksum = 0;
        // household: offset + r % count, the household table is the identity
        const int hh = a.household[me];
        const int hoff = a.hh_offset[hh], hcnt = a.hh_offset[hh + 1] - hoff;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            kv[j] = select_victim(me, hoff, hcnt, w[j], true, nullptr, victims[j]);
            ksum += kv[j];
        }
        // workplace or school: max-contacts of its type
        const int wp = a.workplace[me];
        const int woff = a.wp_offset[wp], wcnt = a.wp_offset[wp + 1] - woff;
        const int desired = workplace_max_contacts(c, wp);
        // errands / afterschool: destinations from today's keys; the adult
        // profile is regenerated from the schedule counter (:3667-3705)
        const int dest[2] = {a.keys[me], a.keys[N + me]};
        int prof = 3;
        if (adult) {
            uint32_t e[4];
            tf2x64(key, E0 + (uint64_t)(me / 2), e);
            const int slot = 2 * (me % 2);
            prof = (int)((e[slot] ^ e[slot + 1]) % 3u);
        }
        int made = 3;
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
        process_contacts<8>(c, key, inf, ctr + 2, victims, kv, a.state, a.claim, a.new_list, sc);
    }
}

// kernel_doWeekend + device_makeContacts_weekend (PandemicSim.cu:3311-3379, :1833-1950)
__global__ void __launch_bounds__(128) k_infect_weekend(SimConst c, InfectArgs a, int day)
{
    Scalars *sc = a.sc;
    if (sc->done) return;
    const TfKey key = make_key(c);
    const int I = sc->infected;
    const unsigned long long R0 = sc->infect_offset;
    for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < I; pos += gridDim.x * blockDim.x) {
        Infector inf;
        inf.pos = pos;
        inf.me = a.infected[pos];
        const int me = inf.me;
        const unsigned long long ctr = R0 + 6ull * (unsigned long long)pos;
        uint32_t w[4];
        tf2x64(key, ctr, w);
        int victims[5], kv[5];
        int ksum = 0;
        const int hh = a.household[me];
        const int hoff = a.hh_offset[hh], hcnt = a.hh_offset[hh + 1] - hoff;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            kv[j] = select_victim(me, hoff, hcnt, w[j], true, nullptr, victims[j]);
            ksum += kv[j];
        }
        const int prof = (int)(w[3] % 6u);
        // Threefry-2x32 on the low seed words with counter (u32)(ctr + 1) (:1895-1901)
        uint32_t v2[2];
        tf2x32(key, (uint32_t)(ctr + 1), v2);
        const int32_t *k3 = a.keys + 3 * (size_t)me;
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

cudaError_t launch_infect(const SimConst &c, const DevArrays &d, bool weekend, int day, cudaStream_t s)
{
    InfectArgs a;
    a.state = d.state; a.gen_p = d.gen_p; a.gen_s = d.gen_s; a.age = d.age;
    a.household = d.household; a.hh_offset = d.hh_offset; a.workplace = d.workplace;
    a.wp_people = d.wp_people; a.wp_offset = d.wp_offset; a.keys = d.keys;
    a.bkt_offset = d.bkt_offset; a.bkt_people = d.bkt_people; a.infected = d.infected;
    a.claim = d.claim; a.new_list = d.new_list; a.sc = d.sc;
    int blocks = sm_count() * 16;
    if (weekend) k_infect_weekend<<<blocks, 128, 0, s>>>(c, a, day);
    else k_infect_weekday<<<blocks, 128, 0, s>>>(c, a, day);
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

// ================================================================== final
__global__ void k_gen_hist(const uint8_t *gen_p, const uint8_t *gen_s, int N, int *hist)
{
    __shared__ int h[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        atomicAdd(&h[gen_p[i]], 1);
        atomicAdd(&h[256 + gen_s[i]], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

cudaError_t launch_gen_hist(const uint8_t *gen_p, const uint8_t *gen_s, int N, int *hist512, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(hist512, 0, 512 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    int blocks = std::max(1, std::min(div_up(N, 256), sm_count() * 4));
    k_gen_hist<<<blocks, 256, 0, s>>>(gen_p, gen_s, N, hist512);
    count_launch();
    return cudaGetLastError();
}

}  // namespace ptk
