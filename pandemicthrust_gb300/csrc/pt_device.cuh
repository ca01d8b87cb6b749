// pt_device.cuh - device-side building blocks of the daily simulation step:
// Threefry counters, the float "fishing" lookups and the model tables.
//
// Every float operation that decides a result uses an explicit round-to-nearest
// intrinsic (__fmul_rn, __fdiv_rn, __fsub_rn, __uint2float_rn), so the arithmetic
// matches the reference's IEEE single-precision code whatever the compiler flags
// (no contraction, no approximate division).
#pragma once
#include <cstdint>
#include "pt_kernels.h"

namespace ptk {

// ---------------------------------------------------------------- tables
// PandemicSim.cu:328-481 (model constants; identical in every simulation).
static __constant__ float c_child_age_cdf[5] = {0.24f, 0.47f, 0.72f, 0.85f, 1.0f};
static __constant__ float c_workplace_pdf[kTypes] = {
    0.06586f, 0.05802f, 0.30227f, 0.0048f, 0.00997f, 0.203f, 0.09736f,
    0.10598f, 0.00681f, 0.02599f, 0.f, 0.08749f, 0.03181f, 0.00064f};
static __constant__ int c_type_max_contacts[kTypes] = {3, 3, 3, 2, 2, 3, 3, 2, 2, 2, 0, 2, 2, 2};
static __constant__ float c_weekday_errand_pdf[kTypes] = {0, 0, 0, 0, 0, 0, 0, 0, 0,
                                                   0.61919f, 0, 0.27812f, 0.06601f, 0.03668f};
static __constant__ float c_weekend_errand_pdf[kTypes] = {0, 0, 0, 0, 0, 0, 0, 0, 0,
                                                   0.51493f, 0, 0.25586f, 0.1162f, 0.113f};
// The reciprocals of the errand probabilities, rounded to nearest (each quotient
// folded by the compiler in IEEE single precision; 0 where the probability is 0,
// a row the search below never ends on).
static __constant__ float c_weekday_errand_rcp[kTypes] = {0, 0, 0, 0, 0, 0, 0, 0, 0,
                                                   1.0f / 0.61919f, 0, 1.0f / 0.27812f, 1.0f / 0.06601f,
                                                   1.0f / 0.03668f};
static __constant__ float c_weekend_errand_rcp[kTypes] = {0, 0, 0, 0, 0, 0, 0, 0, 0,
                                                   1.0f / 0.51493f, 0, 1.0f / 0.25586f, 1.0f / 0.1162f,
                                                   1.0f / 0.113f};
static __constant__ int c_hh_adults[9] = {1, 1, 2, 1, 2, 1, 2, 1, 2};
static __constant__ int c_hh_children[9] = {0, 1, 0, 2, 1, 3, 2, 4, 3};
static __constant__ float c_hh_cdf[9] = {0.279f, 0.319f, 0.628f, 0.671f, 0.8f, 0.812f, 0.939f, 0.944f, 1.0f};
// Contacts per errand hour for weekday profiles 0..3 (3 = afterschool) and the
// errand slot of each of the two weekend errand contacts (PandemicSim.cu:445-481).
static __constant__ int c_weekday_assign[4][2] = {{2, 0}, {0, 2}, {1, 1}, {2, 0}};
static __constant__ int c_weekend_assign[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};

// ---------------------------------------------------------------- Threefry
// Threefry-2x64-20 and 2x32-20 (Salmon et al., SC'11; the Random123 rotation
// tables).  64-bit words are handled as 32-bit halves so each rotation is two
// funnel shifts and each add an add/add-with-carry pair.
struct u64h { uint32_t lo, hi; };

__device__ __forceinline__ u64h mk(uint64_t v) { return {(uint32_t)v, (uint32_t)(v >> 32)}; }

__device__ __forceinline__ u64h add64(u64h a, u64h b)
{
    u64h r;
    asm("add.cc.u32 %0, %2, %4;\n\taddc.u32 %1, %3, %5;"
        : "=r"(r.lo), "=r"(r.hi) : "r"(a.lo), "r"(a.hi), "r"(b.lo), "r"(b.hi));
    return r;
}

template <int R>
__device__ __forceinline__ u64h rotl64(u64h x)
{
    if constexpr (R == 32) {
        return {x.hi, x.lo};
    } else if constexpr (R < 32) {
        return {__funnelshift_l(x.hi, x.lo, R), __funnelshift_l(x.lo, x.hi, R)};
    } else {
        return {__funnelshift_l(x.lo, x.hi, R - 32), __funnelshift_l(x.hi, x.lo, R - 32)};
    }
}

template <int R>
__device__ __forceinline__ void mix64(u64h &x0, u64h &x1)
{
    x0 = add64(x0, x1);
    x1 = rotl64<R>(x1);
    x1.lo ^= x0.lo;
    x1.hi ^= x0.hi;
}

struct TfKey {
    u64h k0, k1, k2;       // key schedule: k2 = parity ^ k0 ^ k1
    uint32_t k32_0, k32_1, k32_2;
};

__device__ __forceinline__ TfKey make_key(const SimConst &c)
{
    TfKey k;
    k.k0 = mk(c.key0);
    k.k1 = mk(c.key1);
    k.k2 = mk(0x1BD11BDAA9FC1A22ULL ^ c.key0 ^ c.key1);
    k.k32_0 = (uint32_t)c.key0;
    k.k32_1 = (uint32_t)c.key1;
    k.k32_2 = 0x1BD11BDAu ^ k.k32_0 ^ k.k32_1;
    return k;
}

// Counter {ctr, ctr}; returns the block as the reference's union reads it:
// w[0] = lo(x0), w[1] = hi(x0), w[2] = lo(x1), w[3] = hi(x1).
__device__ __forceinline__ void tf2x64(const TfKey &k, uint64_t ctr, uint32_t w[4])
{
    u64h c = mk(ctr);
    u64h x0 = add64(c, k.k0);
    u64h x1 = add64(c, k.k1);
    const u64h ks[3] = {k.k0, k.k1, k.k2};
#pragma unroll
    for (int blk = 0; blk < 5; blk++) {
        if ((blk & 1) == 0) {
            mix64<16>(x0, x1); mix64<42>(x0, x1); mix64<12>(x0, x1); mix64<31>(x0, x1);
        } else {
            mix64<16>(x0, x1); mix64<32>(x0, x1); mix64<24>(x0, x1); mix64<21>(x0, x1);
        }
        const int s = blk + 1;
        x0 = add64(x0, ks[s % 3]);
        x1 = add64(x1, add64(ks[(s + 1) % 3], u64h{(uint32_t)s, 0u}));
    }
    w[0] = x0.lo; w[1] = x0.hi; w[2] = x1.lo; w[3] = x1.hi;
}

// The same Threefry-2x64-20 with part of its integer work moved from the ALU pipe
// (IADD3 / SHF / LOP3) to the multiply-add pipe.  `m` holds run-time constants (kernel
// parameters, so the compiler cannot fold the multiplies back into adds and shifts):
// m.one = 1 and m.pow[i] = 2^r for the rotation amounts r below 32.
//   MODE 1: every 64-bit add is a multiply-add with carry, x * 1 + y.
//   MODE 2: also every rotation: x * 2^r as a 32 x 32 -> 64 multiply gives both
//           halves of x shifted by r; two of them and an OR rotate a 64-bit word, and
//           the OR folds into the round's XOR.
// Bit-identical to tf2x64 (integer arithmetic, exact in every form).
struct TfMul {
    uint32_t one;
    uint32_t pow[6];   // 2^16, 2^10 (rotation 42 = swap + 10), 2^12, 2^31, 2^24, 2^21
};

__device__ __forceinline__ u64h add64m(u64h a, u64h b, uint32_t one)
{
    u64h r;
    asm("mad.lo.cc.u32 %0, %2, %6, %4;\n\tmadc.lo.u32 %1, %3, %6, %5;"
        : "=r"(r.lo), "=r"(r.hi) : "r"(a.lo), "r"(a.hi), "r"(b.lo), "r"(b.hi), "r"(one));
    return r;
}

// rotate left by r in (0, 32) with p = 2^r: the 64-bit products hold (x << r) in the
// low word and (x >> (32 - r)) in the high word
__device__ __forceinline__ u64h rotl64m(u64h x, uint32_t p)
{
    const unsigned long long t = (unsigned long long)x.lo * p, u = (unsigned long long)x.hi * p;
    return {(uint32_t)t | (uint32_t)(u >> 32), (uint32_t)u | (uint32_t)(t >> 32)};
}

template <int MODE, int R, int PI>
__device__ __forceinline__ void mix64m(u64h &x0, u64h &x1, const TfMul &m)
{
    x0 = MODE >= 1 ? add64m(x0, x1, m.one) : add64(x0, x1);
    if constexpr (MODE >= 2 && R != 32) {
        const u64h s = R > 32 ? u64h{x1.hi, x1.lo} : x1;
        x1 = rotl64m(s, m.pow[PI]);
    } else {
        x1 = rotl64<R>(x1);
    }
    x1.lo ^= x0.lo;
    x1.hi ^= x0.hi;
}

template <int MODE>
__device__ __forceinline__ void tf2x64m(const TfKey &k, uint64_t ctr, uint32_t w[4], const TfMul &m)
{
    if constexpr (MODE == 0) {
        tf2x64(k, ctr, w);
    } else {
        const u64h c = mk(ctr);
        u64h x0 = add64m(c, k.k0, m.one);
        u64h x1 = add64m(c, k.k1, m.one);
        const u64h ks[3] = {k.k0, k.k1, k.k2};
#pragma unroll
        for (int blk = 0; blk < 5; blk++) {
            if ((blk & 1) == 0) {
                mix64m<MODE, 16, 0>(x0, x1, m); mix64m<MODE, 42, 1>(x0, x1, m);
                mix64m<MODE, 12, 2>(x0, x1, m); mix64m<MODE, 31, 3>(x0, x1, m);
            } else {
                mix64m<MODE, 16, 0>(x0, x1, m); mix64m<MODE, 32, 0>(x0, x1, m);
                mix64m<MODE, 24, 4>(x0, x1, m); mix64m<MODE, 21, 5>(x0, x1, m);
            }
            const int s = blk + 1;
            x0 = add64m(x0, ks[s % 3], m.one);
            x1 = add64m(x1, add64(ks[(s + 1) % 3], u64h{(uint32_t)s, 0u}), m.one);
        }
        w[0] = x0.lo; w[1] = x0.hi; w[2] = x1.lo; w[3] = x1.hi;
    }
}

template <int R>
__device__ __forceinline__ void mix32(uint32_t &x0, uint32_t &x1)
{
    x0 += x1;
    x1 = __funnelshift_l(x1, x1, R);
    x1 ^= x0;
}

__device__ __forceinline__ void tf2x32(const TfKey &k, uint32_t ctr, uint32_t w[2])
{
    uint32_t x0 = ctr + k.k32_0, x1 = ctr + k.k32_1;
    const uint32_t ks[3] = {k.k32_0, k.k32_1, k.k32_2};
#pragma unroll
    for (int blk = 0; blk < 5; blk++) {
        if ((blk & 1) == 0) {
            mix32<13>(x0, x1); mix32<15>(x0, x1); mix32<26>(x0, x1); mix32<6>(x0, x1);
        } else {
            mix32<17>(x0, x1); mix32<29>(x0, x1); mix32<16>(x0, x1); mix32<24>(x0, x1);
        }
        const uint32_t s = blk + 1;
        x0 += ks[s % 3];
        x1 += ks[(s + 1) % 3] + s;
    }
    w[0] = x0; w[1] = x1;
}

// ---------------------------------------------------------------- fishing
// (float)r / UNSIGNED_MAX: the divisor converts to 2^32, so this is exact scaling.
__device__ __forceinline__ float to_unit(uint32_t r) { return __fmul_rn(__uint2float_rn(r), 0x1p-32f); }

// device_setup_fishHouseholdType, PandemicSim.cu:2360-2371
__device__ __forceinline__ int fish_household_type(uint32_t r)
{
    float y = to_unit(r);
    int row = 0;
    while (y > c_hh_cdf[row] && row < 8) row++;
    return row;
}

__device__ __forceinline__ int business_in_type(const SimConst &c, float frac, int type)
{
    int count = c.type_count[type];
    int b = __float2int_rz(__fmul_rn(frac, __int2float_rn(count)));
    if (b >= count) b = count - 1;
    return b + c.type_offset[type];
}

// device_setup_fishWorkplace, PandemicSim.cu:2374-2399
__device__ __forceinline__ int fish_workplace(const SimConst &c, uint32_t r)
{
    float y = to_unit(r);
    int row = 0;
    while (c_workplace_pdf[row] < y && row < kTypes - 1) {
        y = __fsub_rn(y, c_workplace_pdf[row]);
        row++;
    }
    return business_in_type(c, __fdiv_rn(y, c_workplace_pdf[row]), row);
}

// device_setup_fishSchoolAndAge, PandemicSim.cu:2402-2442
__device__ __forceinline__ int fish_school_and_age(const SimConst &c, uint32_t r, int *age)
{
    float y = to_unit(r);
    int row = 0;
    while (row < 4 && y > c_child_age_cdf[row]) row++;
    float frac;
    if (row == 0) {
        frac = __fdiv_rn(y, c_child_age_cdf[0]);
    } else {
        float pdf_here = __fsub_rn(c_child_age_cdf[row], c_child_age_cdf[row - 1]);
        float y_here = __fsub_rn(y, c_child_age_cdf[row - 1]);
        frac = __fdiv_rn(y_here, pdf_here);
    }
    *age = row;
    return business_in_type(c, frac, row + 3);
}

// x / d rounded to nearest, for the errand probabilities d with r = RN(1/d): one
// multiply and Markstein's correction (P. Markstein, IBM J. Res. Dev. 34(1), 1990):
// q = RN(x r), e = x - q d exactly (a fused multiply-add), RN(q + e r).  It equals
// __fdiv_rn(x, d) for x = 0 and every float x in [2^-32, 1] (the values the errand
// search divides) and every row the search can end on; pt_selftest_errand_lookup
// checks all of them, and the whole search on every 32-bit draw.
__device__ __forceinline__ float div_rn_recip(float x, float d, float r)
{
    const float q = __fmul_rn(x, r);
    const float e = __fmaf_rn(-q, d, x);
    return __fmaf_rn(e, r, q);
}

// The errand-type search of device_fishAfterschoolOrErrandDestination_weekday (its
// adult branch, PandemicSim.cu:2909-2947) and device_fishWeekendErrandDestination
// (PandemicSim.cu:1017-1044):
//     row = 9; while (y > pdf[row] && row < 13) { y = y - pdf[row]; row++; }
//     frac = y / pdf[row];
// without branches.  The chain of subtractions runs to the end and the stop is
// selected: once y <= pdf[t], every later remainder is <= 0 (the probabilities are
// >= 0), so every later test fails too, as the loop would have stopped.  Returns the
// row; frac receives the quotient.
template <bool WEEKEND>
__device__ __forceinline__ int errand_row(float y, float &frac)
{
    const float *pdf = WEEKEND ? c_weekend_errand_pdf : c_weekday_errand_pdf;
    const float *rcp = WEEKEND ? c_weekend_errand_rcp : c_weekday_errand_rcp;
    float x = y, d = pdf[9], rd = rcp[9], f = y;
    int row = 9;
#pragma unroll
    for (int t = 9; t < kTypes - 1; t++) {
        const bool go = f > pdf[t];
        f = __fsub_rn(f, pdf[t]);
        row = go ? t + 1 : row;
        x = go ? f : x;
        d = go ? pdf[t + 1] : d;
        rd = go ? rcp[t + 1] : rd;
    }
    frac = div_rn_recip(x, d, rd);
    return row;
}

// The same search as the reference writes it: the loop and the IEEE division.  Kept
// as the self-test's reference for errand_row.
template <bool WEEKEND>
__device__ __forceinline__ int errand_row_loop(float y, float &frac)
{
    const float *pdf = WEEKEND ? c_weekend_errand_pdf : c_weekday_errand_pdf;
    int row = 9;
    while (y > pdf[row] && row < kTypes - 1) {
        y = __fsub_rn(y, pdf[row]);
        row++;
    }
    frac = __fdiv_rn(y, pdf[row]);
    return row;
}

// device_fishAfterschoolOrErrandDestination_weekday, PandemicSim.cu:2909-2947
// (unsigned business number, as the reference).  Children go to an afterschool
// location (type 8); adults to an errand type drawn by errand_row.  Both are computed
// and one is selected, so a warp of adults and children does not diverge.
__device__ __forceinline__ int fish_weekday_dest(const SimConst &c, uint32_t r, bool adult)
{
    const float y = to_unit(r);
    float fa;
    const int ta = errand_row<false>(y, fa);
    const int type = adult ? ta : 8;   // 8: BUSINESS_TYPE_AFTERSCHOOL
    const float frac = adult ? fa : y;
    int count = c.type_count[type];
    unsigned int b = __float2uint_rz(__fmul_rn(frac, __int2float_rn(count)));
    if (b >= (unsigned int)count) b = (unsigned int)(count - 1);
    b += (unsigned int)c.type_offset[type];
    return (int)b;
}

// device_fishWeekendErrandDestination, PandemicSim.cu:1017-1044
__device__ __forceinline__ int fish_weekend_dest(const SimConst &c, uint32_t r)
{
    float frac;
    const int row = errand_row<true>(to_unit(r), frac);
    return business_in_type(c, frac, row);
}

// device_generateWeekendErrands, PandemicSim.cu:980-1014: three distinct hours of
// ten, each with a destination.  The reference's key is destination + hour * L;
// weekend destinations all lie in [lo, L) (lo = first location of type 9), so the
// bucket index used here is the order-preserving compact form hour * R + dest - lo,
// R = L - lo.
template <int MODE = 0>
__device__ __forceinline__ void weekend_errands(const SimConst &c, const TfKey &k, uint64_t ctr, int lo, int R,
                                                int out[3], const TfMul *m = nullptr)
{
    uint32_t w[8];
    if constexpr (MODE == 0) {
        tf2x64(k, ctr, w);
        tf2x64(k, ctr + 1, w + 4);
    } else {
        tf2x64m<MODE>(k, ctr, w, *m);
        tf2x64m<MODE>(k, ctr + 1, w + 4, *m);
    }
    int h1 = (int)(w[0] % 10u);
    int h2 = (int)(w[1] % 10u);
    if (h2 == h1) h2 = (h2 + 1) % 10;
    int h3 = (int)(w[2] % 10u);
    while (h3 == h1 || h3 == h2) h3 = (h3 + 1) % 10;
    out[0] = fish_weekend_dest(c, w[3]) - lo + h1 * R;
    out[1] = fish_weekend_dest(c, w[4]) - lo + h2 * R;
    out[2] = fish_weekend_dest(c, w[5]) - lo + h3 * R;
}

// ---------------------------------------------------------------- interventions
// The interventions have no counterpart in the reference.  Their random choices come
// from this hash, not from the reference's Threefry counter stream, so a run whose
// interventions are all zero draws exactly the reference's numbers.  The mix is the
// splitmix64 finaliser (Steele, Lea and Flood, OOPSLA 2014); the high 32 bits of
// mix(mix(key0 ^ (key1 << 1) ^ tag) ^ (day << 32 | person)) decide.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t intervention_hash(uint64_t key0, uint64_t key1, uint64_t tag, int day,
                                                               int person)
{
    const uint64_t k = splitmix64(key0 ^ (key1 << 1) ^ tag);
    return splitmix64(k ^ (((uint64_t)(uint32_t)day << 32) | (uint32_t)person)) >> 32;
}

// School-type locations: types 3-7 (the children's schools by age band,
// PandemicSim.cu:2402-2442), contiguous in location order.
__device__ __forceinline__ bool is_school(const SimConst &c, int loc)
{
    return loc >= c.type_offset[3] && loc < c.type_offset[7] + c.type_count[7];
}

// device_getWorkplaceMaxContacts, PandemicSim.cu:3492-3511
__device__ __forceinline__ int workplace_max_contacts(const SimConst &c, int loc)
{
    int lid = loc % c.L;
    int t = 0, off, cnt, mx;
    do {
        off = c.type_offset[t];
        cnt = c.type_count[t];
        mx = c_type_max_contacts[t];
        t++;
    } while (lid >= off + cnt);
    return mx;
}

// device_getInfectionProfile, PandemicSim.cu:3974-3988
__device__ __forceinline__ int infection_profile(const SimConst &c, uint32_t r)
{
    int p = (int)(r % 3u) + 2;
    if (to_unit(r) > c.pct_sympt) p += 3;
    return p;
}

// device_calculateInfectionProbability, PandemicSim.cu:2307-2326
__device__ __forceinline__ float infection_probability(const SimConst &c, int profile, int pday, int strain, int ksum)
{
    if (ksum == 0) ksum = 1;
    float avg = __fmul_rn(c.shedding[profile][pday], c.infectiousness[strain]);
    return __fdiv_rn(avg, __int2float_rn(ksum));
}

}  // namespace ptk
