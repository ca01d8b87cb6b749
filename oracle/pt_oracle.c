/*
 * pt_oracle.c - CPU oracle for the PandemicThrust daily simulation step.
 *
 * TEST INFRASTRUCTURE ONLY: see pt_oracle.h.  Every function below names the
 * reference lines it restates.  Paths are relative to the reference project:
 * "PandemicSim.cu" = PandemicThrust/PandemicThrust/PandemicSim.cu,
 * "host_functions.cpp" = PandemicThrust/PandemicThrust/host_functions.cpp,
 * "threefry.h" = PandemicThrust/Random123/Random123/threefry.h.
 *
 * Build with -O2 -ffp-contract=off and without -ffast-math: the float "fishing"
 * lookups must round exactly like the reference's IEEE single-precision code.
 */
#include "pt_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Model constants (simParameters.h:27-100, PandemicSim.h:283-302)     */
/* ------------------------------------------------------------------ */
#define NUM_BUSINESS_TYPES 14
#define HH_TABLE_ROWS 9
#define CHILD_DATA_ROWS 5
#define CULMINATION_PERIOD 10
#define STATUS_RECOVERED 0
#define STATUS_SUSCEPTIBLE 1
#define STATUS_INFECTED 2
#define AGE_5 0
#define AGE_ADULT 5
#define DAY_NOT_INFECTED 255
#define GEN_NOT_INFECTED 255
#define CONTACT_NONE 0
#define CONTACT_WORKPLACE 1
#define CONTACT_SCHOOL 2
#define CONTACT_ERRAND 3
#define CONTACT_AFTERSCHOOL 4
#define CONTACT_HOME 5
#define MAX_CONTACTS_WEEKDAY 8
#define MAX_CONTACTS_WEEKEND 5
#define WEEKDAY_ERRAND_HOURS 2
#define WEEKEND_ERRAND_HOURS 10
#define FIRST_ERRAND_ROW 9
#define BUSINESS_TYPE_PRESCHOOL 3
#define BUSINESS_TYPE_AFTERSCHOOL 8
#define WEEKDAY_PROFILE_AFTERSCHOOL 3

/* PandemicSim.cu:328-340 */
static const float CHILD_AGE_CDF[CHILD_DATA_ROWS] = {0.24f, 0.47f, 0.72f, 0.85f, 1.0f};
/* PandemicSim.cu:343-356 */
static const float WORKPLACE_PDF[NUM_BUSINESS_TYPES] = {
    0.06586f, 0.05802f, 0.30227f, 0.0048f, 0.00997f, 0.203f, 0.09736f,
    0.10598f, 0.00681f, 0.02599f, 0.f, 0.08749f, 0.03181f, 0.00064f};
/* PandemicSim.cu:359-372 (base counts, scaled in setup) */
static const int BASE_TYPE_COUNT[NUM_BUSINESS_TYPES] = {
    1000, 7000, 2400, 300, 100, 200, 100, 100, 300, 500, 0, 300, 400, 100};
/* PandemicSim.cu:375-388 */
static const int TYPE_MAX_CONTACTS[NUM_BUSINESS_TYPES] = {3, 3, 3, 2, 2, 3, 3, 2, 2, 2, 0, 2, 2, 2};
/* PandemicSim.cu:392-406 */
static const float WEEKDAY_ERRAND_PDF[NUM_BUSINESS_TYPES] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0.61919f, 0, 0.27812f, 0.06601f, 0.03668f};
static const float WEEKEND_ERRAND_PDF[NUM_BUSINESS_TYPES] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0.51493f, 0, 0.25586f, 0.1162f, 0.113f};
/* PandemicSim.cu:410-440 */
static const int HH_ADULTS[HH_TABLE_ROWS] = {1, 1, 2, 1, 2, 1, 2, 1, 2};
static const int HH_CHILDREN[HH_TABLE_ROWS] = {0, 1, 0, 2, 1, 3, 2, 4, 3};
static const float HH_CDF[HH_TABLE_ROWS] = {0.279f, 0.319f, 0.628f, 0.671f, 0.8f,
                                            0.812f, 0.939f, 0.944f, 1.0f};
/* PandemicSim.cu:445-456: contacts per hour for weekday errand profiles 0..3
 * (profile 3 = afterschool, WORKPLACE_TYPE_MAX_CONTACTS[8] contacts in hour 0). */
static const int WEEKDAY_ASSIGN[4][2] = {{2, 0}, {0, 2}, {1, 1}, {2, 0}};
/* PandemicSim.cu:460-481: errand slot of each of the two weekend errand contacts. */
static const int WEEKEND_ASSIGN[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
/* PandemicSim.cu:486-555 */
static const float SHEDDING_BASE[6][CULMINATION_PERIOD] = {
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
/* PandemicSim.cu:560-562: kappa 0 for "no contact", 1 for every other type. */
static const int KVAL[6] = {0, 1, 1, 1, 1, 1};

/* ------------------------------------------------------------------ */
/* Threefry (threefry.h:190-290, default 20 rounds threefry.h:174-180)  */
/* Published algorithm: Salmon, Moraes, Dror, Shaw, "Parallel random   */
/* numbers: as easy as 1, 2, 3", SC'11.  Rotation constants are the    */
/* Threefry-2x64 / 2x32 tables (threefry.h:86-93, :135-142).           */
/* ------------------------------------------------------------------ */
static const unsigned ROT64[8] = {16, 42, 12, 31, 16, 32, 24, 21};
static const unsigned ROT32[8] = {13, 15, 26, 6, 17, 29, 16, 24};

void ptor_threefry2x64(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2])
{
    uint64_t ks[3];
    ks[0] = key[0];
    ks[1] = key[1];
    ks[2] = 0x1BD11BDAA9FC1A22ULL ^ key[0] ^ key[1];
    uint64_t x0 = ctr[0] + ks[0];
    uint64_t x1 = ctr[1] + ks[1];
    for (int r = 0; r < 20; r++) {
        unsigned rot = ROT64[r & 7];
        x0 += x1;
        x1 = (x1 << rot) | (x1 >> (64 - rot));
        x1 ^= x0;
        if ((r & 3) == 3) {
            unsigned s = (unsigned)(r >> 2) + 1u; /* injection number 1..5 */
            x0 += ks[s % 3];
            x1 += ks[(s + 1) % 3] + s;
        }
    }
    out[0] = x0;
    out[1] = x1;
}

void ptor_threefry2x32(const uint32_t ctr[2], const uint32_t key[2], uint32_t out[2])
{
    uint32_t ks[3];
    ks[0] = key[0];
    ks[1] = key[1];
    ks[2] = 0x1BD11BDAu ^ key[0] ^ key[1];
    uint32_t x0 = ctr[0] + ks[0];
    uint32_t x1 = ctr[1] + ks[1];
    for (int r = 0; r < 20; r++) {
        unsigned rot = ROT32[r & 7];
        x0 += x1;
        x1 = (x1 << rot) | (x1 >> (32 - rot));
        x1 ^= x0;
        if ((r & 3) == 3) {
            uint32_t s = (uint32_t)(r >> 2) + 1u;
            x0 += ks[s % 3];
            x1 += ks[(s + 1) % 3] + s;
        }
    }
    out[0] = x0;
    out[1] = x1;
}

/* The reference reads a Threefry2x64 block as four 32-bit words through a union
 * (e.g. PandemicSim.cu:985-994): little-endian, so word 0 = low half of x0,
 * word 1 = high half of x0, word 2 = low half of x1, word 3 = high half of x1.
 * Key = {(long)SEED[0], (long)SEED[1]}, counter = {c, c}. */
static void tf_words(const ptor_sim *s, uint64_t c, uint32_t w[4]);

/* ------------------------------------------------------------------ */
/* glibc srand()/rand() (TYPE_3 additive feedback, degree 31, sep 3).  */
/* Published description: glibc random_r.c; P. Selinger, "The GLIBC    */
/* pseudo-random number generator".  The reference calls srand/rand at */
/* PandemicSim.cu:2856-2861 (seeds) and :1648 (initial infected).       */
/* ------------------------------------------------------------------ */
void ptor_glibc_srand(ptor_glibc_rand *g, unsigned int seed)
{
    if (seed == 0) seed = 1;
    int32_t word = (int32_t)seed;
    g->r[0] = word;
    for (int i = 1; i < 31; i++) {
        long hi = word / 127773;
        long lo = word % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        word = (int32_t)w;
        g->r[i] = word;
    }
    g->f = 3;   /* front index (fptr) */
    g->b = 0;   /* rear index  (rptr) */
    for (int i = 0; i < 310; i++) (void)ptor_glibc_rand_next(g);
}

int ptor_glibc_rand_next(ptor_glibc_rand *g)
{
    uint32_t val = (uint32_t)g->r[g->f] + (uint32_t)g->r[g->b];
    g->r[g->f] = (int32_t)val;
    g->f = (g->f + 1) % 31;
    g->b = (g->b + 1) % 31;
    return (int)(val >> 1);
}

/* ------------------------------------------------------------------ */
/* Simulation state                                                    */
/* ------------------------------------------------------------------ */
struct ptor_sim {
    ptor_params p;
    int core_seed;
    int seeds[4];
    ptor_glibc_rand rng;      /* continues after the four seed draws */
    uint64_t key[2];
    uint32_t key32[2];
    int N, H, L, adults, children;
    int type_count[NUM_BUSINESS_TYPES];
    int type_offset[NUM_BUSINESS_TYPES];
    float shedding[6][CULMINATION_PERIOD];
    float infectiousness[2];
    float pct_sympt;
    uint64_t rand_offset, wp_rand_offset, errand_rand_offset;
    int day;                  /* current_day */
    int infected_count;
    uint8_t *status_p, *status_s, *day_p, *day_s, *gen_p, *gen_s, *age;
    int32_t *household, *hh_offset, *workplace, *wp_people, *wp_off;
    int32_t *infected;
    int32_t *ekeys, *epeople, *eoffset;
    int32_t *ecursor;
    int e_entries, e_buckets;
    int setup_done;
    /* interventions (the build's extensions; all zero reproduces the reference) */
    int closure_start, closure_end;
    uint64_t absent_thr, vacc_thr;
};

/* Interventions have no counterpart in the reference.  Their random choices use the
 * splitmix64 finaliser (Steele, Lea and Flood, OOPSLA 2014) over (key, tag, day,
 * person), apart from the reference's Threefry stream: high 32 bits of
 * mix(mix(key0 ^ (key1 << 1) ^ tag) ^ (day << 32 | person)). */
enum { TAG_ABSENT = 1, TAG_VACCINATED = 2 };

static uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t intervention_hash(const ptor_sim *s, uint64_t tag, int day, int person)
{
    uint64_t k = splitmix64(s->key[0] ^ (s->key[1] << 1) ^ tag);
    return splitmix64(k ^ (((uint64_t)(uint32_t)day << 32) | (uint32_t)person)) >> 32;
}

static uint64_t fraction_threshold(float f)
{
    double t = (double)f * 4294967296.0;
    return t <= 0.0 ? 0ull : (t >= 4294967296.0 ? 4294967296ull : (uint64_t)(t + 0.5));
}

void ptor_set_interventions(ptor_sim *s, int closure_start, int closure_days, float absenteeism, float coverage)
{
    s->closure_start = closure_start;
    s->closure_end = closure_days > 0 ? closure_start + closure_days : 0;
    s->absent_thr = fraction_threshold(absenteeism);
    s->vacc_thr = fraction_threshold(coverage);
}

static int g_threads = 0;
void ptor_set_threads(int n) { g_threads = n; }

static void tf_words(const ptor_sim *s, uint64_t c, uint32_t w[4])
{
    uint64_t ctr[2] = {c, c}, out[2];
    ptor_threefry2x64(ctr, s->key, out);
    w[0] = (uint32_t)out[0];
    w[1] = (uint32_t)(out[0] >> 32);
    w[2] = (uint32_t)out[1];
    w[3] = (uint32_t)(out[1] >> 32);
}

/* y = (float)r / UNSIGNED_MAX; the divisor converts to 4294967296.0f, so this is
 * an exact power-of-two scaling (PandemicSim.cu:2363 and siblings). */
static inline float to_unit(uint32_t r) { return (float)r / 4294967296.0f; }

/* roundHalfUp_toInt, PandemicSim.cu:1662-1665 */
static int round_half_up(double d) { return (int)floor(d + 0.5); }

/* ------------------------------------------------------------------ */
/* Fishing lookups                                                     */
/* ------------------------------------------------------------------ */
/* device_setup_fishHouseholdType, PandemicSim.cu:2360-2371 */
static int fish_household_type(uint32_t r)
{
    float y = to_unit(r);
    int row = 0;
    while (y > HH_CDF[row] && row < HH_TABLE_ROWS - 1) row++;
    return row;
}

/* device_setup_fishWorkplace, PandemicSim.cu:2374-2399 (= host_functions.cpp:80-104) */
static int fish_workplace(const ptor_sim *s, uint32_t r)
{
    float y = to_unit(r);
    int row = 0;
    while (WORKPLACE_PDF[row] < y && row < NUM_BUSINESS_TYPES - 1) {
        y -= WORKPLACE_PDF[row];
        row++;
    }
    float frac = y / WORKPLACE_PDF[row];
    int type_count = s->type_count[row];
    int business = (int)(frac * (float)type_count);
    if (business >= type_count) business = type_count - 1;
    return business + s->type_offset[row];
}

/* device_setup_fishSchoolAndAge, PandemicSim.cu:2402-2442 (= host_functions.cpp:41-78) */
static int fish_school_and_age(const ptor_sim *s, uint32_t r, int *age_out)
{
    float y = to_unit(r);
    int row = 0;
    while (row < CHILD_DATA_ROWS - 1 && y > CHILD_AGE_CDF[row]) row++;
    int wp_type = row + BUSINESS_TYPE_PRESCHOOL;
    float frac;
    if (row == 0) {
        frac = y / CHILD_AGE_CDF[row];
    } else {
        float pdf_here = CHILD_AGE_CDF[row] - CHILD_AGE_CDF[row - 1];
        float y_here = y - CHILD_AGE_CDF[row - 1];
        frac = y_here / pdf_here;
    }
    int type_count = s->type_count[wp_type];
    int business = (int)(frac * (float)type_count);
    if (business >= type_count) business = type_count - 1;
    *age_out = row;
    return business + s->type_offset[wp_type];
}

/* device_setup_assignWorkplaceOrSchool, PandemicSim.cu:2445-2457 */
static int assign_workplace_or_school(const ptor_sim *s, uint32_t r, int *age)
{
    if (*age == AGE_ADULT) return fish_workplace(s, r);
    return fish_school_and_age(s, r, age);
}

/* device_fishAfterschoolOrErrandDestination_weekday, PandemicSim.cu:2909-2947
 * (= host_functions.cpp:167-204).  Note the unsigned business number. */
static int fish_weekday_dest(const ptor_sim *s, uint32_t r, int age)
{
    int type = BUSINESS_TYPE_AFTERSCHOOL;
    float frac = to_unit(r);
    if (age == AGE_ADULT) {
        type = FIRST_ERRAND_ROW;
        float row_pdf = WEEKDAY_ERRAND_PDF[type];
        while (frac > row_pdf && type < NUM_BUSINESS_TYPES - 1) {
            frac -= row_pdf;
            type++;
            row_pdf = WEEKDAY_ERRAND_PDF[type];
        }
        frac = frac / row_pdf;
    }
    int type_count = s->type_count[type];
    int type_offset = s->type_offset[type];
    unsigned int business = (unsigned int)(frac * (float)type_count);
    if (business >= (unsigned int)type_count) business = (unsigned int)(type_count - 1);
    business += (unsigned int)type_offset;
    return (int)business;
}

/* device_fishWeekendErrandDestination, PandemicSim.cu:1017-1044
 * (= host_functions.cpp:248-268) */
static int fish_weekend_dest(const ptor_sim *s, uint32_t r)
{
    float y = to_unit(r);
    int row = FIRST_ERRAND_ROW;
    while (y > WEEKEND_ERRAND_PDF[row] && row < NUM_BUSINESS_TYPES - 1) {
        y -= WEEKEND_ERRAND_PDF[row];
        row++;
    }
    float frac = y / WEEKEND_ERRAND_PDF[row];
    int type_count = s->type_count[row];
    int business = (int)(frac * (float)type_count);
    if (business >= type_count) business = type_count - 1;
    return business + s->type_offset[row];
}

/* device_assignAfterschoolOrErrandDests_weekday, PandemicSim.cu:2950-2969 */
static void weekday_dests(const ptor_sim *s, uint32_t r1, uint32_t r2, int age, int *d1, int *d2)
{
    int dest1 = fish_weekday_dest(s, r1, age);
    int dest2 = dest1;
    if (age == AGE_ADULT) dest2 = fish_weekday_dest(s, r2, age);
    dest2 += s->L;
    *d1 = dest1;
    *d2 = dest2;
}

/* device_generateWeekendErrands, PandemicSim.cu:980-1014 */
static void weekend_errands(const ptor_sim *s, uint64_t c, int out[3])
{
    uint32_t w[8];
    tf_words(s, c, w);
    tf_words(s, c + 1, w + 4);
    int h1 = (int)(w[0] % WEEKEND_ERRAND_HOURS);
    int h2 = (int)(w[1] % WEEKEND_ERRAND_HOURS);
    if (h2 == h1) h2 = (h2 + 1) % WEEKEND_ERRAND_HOURS;
    int h3 = (int)(w[2] % WEEKEND_ERRAND_HOURS);
    while (h3 == h1 || h3 == h2) h3 = (h3 + 1) % WEEKEND_ERRAND_HOURS;
    out[0] = fish_weekend_dest(s, w[3]) + h1 * s->L;
    out[1] = fish_weekend_dest(s, w[4]) + h2 * s->L;
    out[2] = fish_weekend_dest(s, w[5]) + h3 * s->L;
}

/* ------------------------------------------------------------------ */
/* Regeneration (device_recalc*, PandemicSim.cu:3667-3705, 3742-3746,  */
/* 3872-3890; host twins host_functions.cpp:6-25, 106-144, 207-211)    */
/* ------------------------------------------------------------------ */
int ptor_recalc_workplace(const ptor_sim *s, int idx, int age)
{
    uint32_t w[4];
    tf_words(s, s->wp_rand_offset + (uint64_t)(idx / 4), w);
    return assign_workplace_or_school(s, w[idx % 4], &age);
}

int ptor_recalc_weekday_errands(const ptor_sim *s, uint64_t errand_offset, int idx, int age,
                                int *dest1, int *dest2)
{
    uint32_t w[4];
    tf_words(s, errand_offset + (uint64_t)(idx / 2), w);
    int slot = 2 * (idx % 2);
    weekday_dests(s, w[slot], w[slot + 1], age, dest1, dest2);
    if (age != AGE_ADULT) return WEEKDAY_PROFILE_AFTERSCHOOL;
    uint32_t x = w[slot] ^ w[slot + 1];
    return (int)(x % WEEKDAY_PROFILE_AFTERSCHOOL);
}

void ptor_recalc_weekend_errands(const ptor_sim *s, uint64_t errand_offset, int idx, int dests[3])
{
    weekend_errands(s, errand_offset + 2 * (uint64_t)idx, dests);
}

/* ------------------------------------------------------------------ */
/* Construction: seed, parameters, scaling, infection data            */
/* ------------------------------------------------------------------ */
ptor_sim *ptor_create(const ptor_params *p, int core_seed)
{
    if (p->max_days < 0 || p->max_days > 255) return NULL;
    if (p->initial_pandemic < 0 || p->initial_seasonal < 0) return NULL;
    ptor_sim *s = (ptor_sim *)calloc(1, sizeof(ptor_sim));
    if (!s) return NULL;
    s->p = *p;
    s->core_seed = core_seed;
    /* setup_loadSeed, PandemicSim.cu:2843-2862 */
    ptor_glibc_srand(&s->rng, (unsigned int)core_seed);
    for (int i = 0; i < 4; i++) s->seeds[i] = ptor_glibc_rand_next(&s->rng);
    s->key[0] = (uint64_t)(int64_t)s->seeds[0];
    s->key[1] = (uint64_t)(int64_t)s->seeds[1];
    s->key32[0] = (uint32_t)s->seeds[0];
    s->key32[1] = (uint32_t)s->seeds[1];

    /* setup_scaleSimulation, PandemicSim.cu:1127-1162 */
    s->H = round_half_up(p->people_scaling * (double)1000000);
    int sum = 0;
    for (int t = 0; t < NUM_BUSINESS_TYPES; t++) {
        int original = round_half_up(BASE_TYPE_COUNT[t]);
        float scaled = p->location_scaling * (float)original; /* float product */
        int n = round_half_up((double)scaled);
        if (n == 0 && original > 0) n = 1;
        s->type_count[t] = n;
        sum += n;
    }
    s->L = sum;
    int acc = 0;
    for (int t = 0; t < NUM_BUSINESS_TYPES; t++) {
        s->type_offset[t] = acc;
        acc += s->type_count[t];
    }

    /* setup_calculateInfectionData, PandemicSim.cu:2828-2840 */
    memcpy(s->shedding, SHEDDING_BASE, sizeof(SHEDDING_BASE));
    for (int i = 3; i < 6; i++)
        for (int j = 0; j < CULMINATION_PERIOD; j++) s->shedding[i][j] *= p->asymp_factor;
    float denom = (1.0f - p->asymp_factor) * p->percent_symptomatic;
    s->infectiousness[0] = p->r_pandemic / denom;
    s->infectiousness[1] = p->r_seasonal / denom;
    s->pct_sympt = p->percent_symptomatic;
    if (s->H <= 0 || s->L <= 0) {
        free(s);
        return NULL;
    }
    return s;
}

void ptor_destroy(ptor_sim *s)
{
    if (!s) return;
    free(s->status_p); free(s->status_s); free(s->day_p); free(s->day_s);
    free(s->gen_p); free(s->gen_s); free(s->age); free(s->household);
    free(s->hh_offset); free(s->workplace); free(s->wp_people); free(s->wp_off);
    free(s->infected); free(s->ekeys); free(s->epeople); free(s->eoffset); free(s->ecursor);
    free(s);
}

/* Stable counting sort of person ids by key: the same result as the reference's
 * stable radix sort of (key, person) pairs followed by lower_bound offsets with
 * offsets[B] = E (PandemicSim.cu:1212-1248, :1313-1354, :3835-3862). */
static void stable_bucket(int E, const int32_t *keys, int B, int32_t *offset, int32_t *cursor,
                          int32_t *people, int weekday_N, int per_person)
{
    memset(offset, 0, sizeof(int32_t) * (size_t)(B + 1));
    for (int e = 0; e < E; e++) offset[keys[e] + 1]++;
    for (int b = 0; b < B; b++) offset[b + 1] += offset[b];
    memcpy(cursor, offset, sizeof(int32_t) * (size_t)B);
    for (int e = 0; e < E; e++) {
        int person;
        if (weekday_N > 0) person = e < weekday_N ? e : e - weekday_N;
        else person = e / per_person;
        people[cursor[keys[e]]++] = person;
    }
}

/* setupSim, PandemicSim.cu:146-208 */
int ptor_setup(ptor_sim *s)
{
    s->rand_offset = 0;
    s->day = 0;
    const int H = s->H;
    /* setup_calcPopulationSize_thrust + kernel_householdTypeAssignment: both use
     * counters 0..H/4, four households per counter (PandemicSim.cu:3579-3605,
     * :2329-2357), then rand_offset += H/4 (:2570-2571). */
    uint8_t *types = (uint8_t *)malloc((size_t)H + 1);
    int32_t *adult_scan = (int32_t *)malloc(sizeof(int32_t) * ((size_t)H + 1));
    int32_t *child_scan = (int32_t *)malloc(sizeof(int32_t) * ((size_t)H + 1));
    if (!types || !adult_scan || !child_scan) return -1;
    for (int g = 0; g <= H / 4; g++) {
        uint32_t w[4];
        tf_words(s, s->rand_offset + (uint64_t)g, w);
        for (int i = 0; i < 4; i++)
            if (4 * g + i < H) types[4 * g + i] = (uint8_t)fish_household_type(w[i]);
    }
    s->rand_offset += (uint64_t)(H / 4);
    /* exclusive scans over H+1 entries (PandemicSim.cu:2579-2593) */
    int a = 0, c = 0;
    for (int h = 0; h < H; h++) {
        adult_scan[h] = a;
        child_scan[h] = c;
        a += HH_ADULTS[types[h]];
        c += HH_CHILDREN[types[h]];
    }
    adult_scan[H] = a;
    child_scan[H] = c;
    s->adults = a;
    s->children = c;
    const int N = a + c;
    s->N = N;
    if (N <= 0) return -1;

    size_t n = (size_t)N;
    s->status_p = (uint8_t *)malloc(n); s->status_s = (uint8_t *)malloc(n);
    s->day_p = (uint8_t *)malloc(n); s->day_s = (uint8_t *)malloc(n);
    s->gen_p = (uint8_t *)malloc(n); s->gen_s = (uint8_t *)malloc(n);
    s->age = (uint8_t *)malloc(n);
    s->household = (int32_t *)malloc(4 * n);
    s->hh_offset = (int32_t *)malloc(4 * ((size_t)H + 1));
    s->workplace = (int32_t *)malloc(4 * n);
    s->wp_people = (int32_t *)malloc(4 * n);
    s->wp_off = (int32_t *)malloc(4 * ((size_t)s->L + 1));
    s->infected = (int32_t *)malloc(4 * n);
    s->ekeys = (int32_t *)malloc(4 * 3 * n);
    s->epeople = (int32_t *)malloc(4 * 3 * n);
    s->eoffset = (int32_t *)malloc(4 * (10 * (size_t)s->L + 1));
    s->ecursor = (int32_t *)malloc(4 * (10 * (size_t)s->L + 1));
    if (!s->status_p || !s->status_s || !s->day_p || !s->day_s || !s->gen_p || !s->gen_s ||
        !s->age || !s->household || !s->hh_offset || !s->workplace || !s->wp_people ||
        !s->wp_off || !s->infected || !s->ekeys || !s->epeople || !s->eoffset || !s->ecursor)
        return -1;

    /* kernel_generateHouseholds, PandemicSim.cu:2490-2531: adults first, then
     * children with the AGE_5 placeholder; household_offsets[H] = N (:2613). */
    for (int h = 0; h < H; h++) {
        int off = adult_scan[h] + child_scan[h];
        s->hh_offset[h] = off;
        int na = HH_ADULTS[types[h]], nc = HH_CHILDREN[types[h]];
        for (int i = 0; i < na; i++) { s->household[off + i] = h; s->age[off + i] = AGE_ADULT; }
        for (int i = 0; i < nc; i++) { s->household[off + na + i] = h; s->age[off + na + i] = AGE_5; }
    }
    s->hh_offset[H] = N;
    free(types); free(adult_scan); free(child_scan);


    /* setup_assignWorkplaces + assignWorkplaceFunctor, PandemicSim.cu:3750-3778,
     * :3812-3869: counters W0..W0+N/4, four persons per counter; children get their
     * age band here.  rand_offset += N/4 (:3829-3830). */
    s->wp_rand_offset = s->rand_offset;
    for (int g = 0; g <= N / 4; g++) {
        uint32_t w[4];
        tf_words(s, s->wp_rand_offset + (uint64_t)g, w);
        for (int i = 0; i < 4 && 4 * g + i < N; i++) {
            int idx = 4 * g + i;
            int age = s->age[idx];
            s->workplace[idx] = assign_workplace_or_school(s, w[i], &age);
            s->age[idx] = (uint8_t)age;
        }
    }
    s->rand_offset += (uint64_t)(N / 4);
    /* workplace_people / workplace_offsets: stable sort by workplace + lower_bound
     * (PandemicSim.cu:3835-3862).  The reference assumes CUB leaves the result in
     * workplace_people; the intended, sorted table is what is restated here. */
    stable_bucket(N, s->workplace, s->L, s->wp_off, s->ecursor, s->wp_people, 0, 1);

    /* setup_initializeStatusArrays, PandemicSim.cu:3654-3664 */
    memset(s->status_p, STATUS_SUSCEPTIBLE, n);
    memset(s->status_s, STATUS_SUSCEPTIBLE, n);
    memset(s->day_p, DAY_NOT_INFECTED, n);
    memset(s->day_s, DAY_NOT_INFECTED, n);
    memset(s->gen_p, GEN_NOT_INFECTED, n);
    memset(s->gen_s, GEN_NOT_INFECTED, n);
    /* vaccination (intervention): recovered from both strains, never infected */
    if (s->vacc_thr)
        for (int i = 0; i < N; i++)
            if (intervention_hash(s, TAG_VACCINATED, 0, i) < s->vacc_thr) {
                s->status_p[i] = STATUS_RECOVERED;
                s->status_s[i] = STATUS_RECOVERED;
            }

    /* setup_initialInfected + n_unique_numbers, PandemicSim.cu:708-758, :1642-1659:
     * distinct rand() % N, the first P pandemic, the next S seasonal; status
     * STATUS_INFECTED (profile 0), day 0, generation 0. */
    int P = s->p.initial_pandemic, S = s->p.initial_seasonal;
    int total = P + S;
    if (total > N) return -1;
    int32_t *seeds = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    if (!seeds) return -1;
    for (int i = 0; i < total; i++) {
        int dup;
        do {
            seeds[i] = ptor_glibc_rand_next(&s->rng) % N;
            dup = 0;
            for (int j = 0; j < i; j++)
                if (seeds[j] == seeds[i]) { dup = 1; break; }
        } while (dup);
    }
    for (int i = 0; i < P; i++) {
        s->status_p[seeds[i]] = STATUS_INFECTED;
        s->day_p[seeds[i]] = 0;
        s->gen_p[seeds[i]] = 0;
    }
    for (int i = P; i < total; i++) {
        s->status_s[seeds[i]] = STATUS_INFECTED;
        s->day_s[seeds[i]] = 0;
        s->gen_s[seeds[i]] = 0;
    }
    free(seeds);
    s->e_entries = 0;
    s->e_buckets = 0;
    s->infected_count = 0;
    s->setup_done = 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Daily stages                                                        */
/* ------------------------------------------------------------------ */
/* kernel_countInfectedStatusAndRecover, PandemicSim.cu:2097-2192 */
void ptor_count_and_recover(ptor_sim *s, int counts16[16])
{
    int day_to_recover = s->day - CULMINATION_PERIOD;
    long cnt[16] = {0};
    for (int i = 0; i < s->N; i++) {
        int sp = s->status_p[i];
        if (day_to_recover >= 0 && sp >= STATUS_INFECTED && (int)s->day_p[i] <= day_to_recover) {
            sp = STATUS_RECOVERED;
            s->status_p[i] = STATUS_RECOVERED;
        }
        int ss = s->status_s[i];
        if (day_to_recover >= 0 && ss >= STATUS_INFECTED && (int)s->day_s[i] <= day_to_recover) {
            ss = STATUS_RECOVERED;
            s->status_s[i] = STATUS_RECOVERED;
        }
        cnt[sp]++;
        cnt[8 + ss]++;
    }
    for (int k = 0; k < 16; k++) counts16[k] = (int)cnt[k];
}

/* daily_buildInfectedArray_global, PandemicSim.cu:2195-2224: ascending ids with
 * either strain's status >= STATUS_INFECTED. */
int ptor_build_infected(ptor_sim *s)
{
    int I = 0;
    for (int i = 0; i < s->N; i++)
        if (s->status_p[i] >= STATUS_INFECTED || s->status_s[i] >= STATUS_INFECTED)
            s->infected[I++] = i;
    s->infected_count = I;
    return I;
}

static int is_weekend_day(int day) { return (day % 7) >= 5; } /* PandemicSim.h:283-284 */

/* Weekday: kernel_assignWeekdayAfterschoolAndErrands, PandemicSim.cu:2972-3022
 * (hour-0 keys in [0,N), hour-1 keys in [N,2N), rand_offset += N/2, :3039-3040).
 * Weekend: kernel_assignWeekendErrands, PandemicSim.cu:2082-2094 (keys 3p..3p+2,
 * rand_offset += 2N, :1414-1415).  Then the stable bucket build. */
void ptor_build_schedule(ptor_sim *s)
{
    const int N = s->N, L = s->L;
    s->errand_rand_offset = s->rand_offset;
    if (!is_weekend_day(s->day)) {
        int G = N / 2;
#pragma omp parallel for schedule(static) num_threads(g_threads > 0 ? g_threads : 1)
        for (int g = 0; g <= G; g++) {
            uint32_t w[4];
            tf_words(s, s->errand_rand_offset + (uint64_t)g, w);
            for (int k = 0; k < 2; k++) {
                int idx = 2 * g + k;
                if (idx < N) {
                    int d1, d2;
                    weekday_dests(s, w[2 * k], w[2 * k + 1], s->age[idx], &d1, &d2);
                    s->ekeys[idx] = d1;
                    s->ekeys[N + idx] = d2;
                }
            }
        }
        s->rand_offset += (uint64_t)(N / 2);
        s->e_entries = 2 * N;
        s->e_buckets = WEEKDAY_ERRAND_HOURS * L;
        stable_bucket(2 * N, s->ekeys, s->e_buckets, s->eoffset, s->ecursor, s->epeople, N, 0);
    } else {
#pragma omp parallel for schedule(static) num_threads(g_threads > 0 ? g_threads : 1)
        for (int i = 0; i < N; i++)
            weekend_errands(s, s->errand_rand_offset + 2 * (uint64_t)i, s->ekeys + 3 * (size_t)i);
        s->rand_offset += 2 * (uint64_t)N;
        s->e_entries = 3 * N;
        s->e_buckets = WEEKEND_ERRAND_HOURS * L;
        stable_bucket(3 * N, s->ekeys, s->e_buckets, s->eoffset, s->ecursor, s->epeople, 0, 3);
    }
}

/* device_selectRandomPersonFromLocation + device_getVictimAtIndex,
 * PandemicSim.cu:2016-2071.  A location with at most one person yields victim =
 * count and type NONE. */
static int select_victim(int self, int off, int count, uint32_t r, int type,
                         const int32_t *table, int *victim, int *ctype)
{
    int v = count;
    int t = CONTACT_NONE;
    if (count > 1) {
        int o = (int)(r % (uint32_t)count);
        v = (type == CONTACT_HOME) ? off + o : table[off + o];
        if (v == self) {
            o = (o + 1) % count;
            v = (type == CONTACT_HOME) ? off + o : table[off + o];
        }
        t = type;
    }
    *victim = v;
    *ctype = t;
    return KVAL[t];
}

/* device_getWorkplaceMaxContacts, PandemicSim.cu:3492-3511 */
static int workplace_max_contacts(const ptor_sim *s, int loc)
{
    int lid = loc % s->L;
    int t = 0, off, cnt, mx;
    do {
        off = s->type_offset[t];
        cnt = s->type_count[t];
        mx = TYPE_MAX_CONTACTS[t];
        t++;
    } while (lid >= off + cnt);
    return mx;
}

/* device_getInfectionProfile, PandemicSim.cu:3974-3988 */
static int infection_profile(const ptor_sim *s, uint32_t r)
{
    int profile = (int)(r % 3u) + STATUS_INFECTED;
    float y = to_unit(r);
    if (y > s->pct_sympt) profile += 3;
    return profile;
}

/* device_calculateInfectionProbability, PandemicSim.cu:2307-2326 */
static float infection_probability(const ptor_sim *s, int profile, int pday, int strain, int kval_sum)
{
    if (kval_sum == 0) kval_sum = 1;
    float alpha = s->shedding[profile][pday];
    float avg = alpha * s->infectiousness[strain];
    return avg / (float)kval_sum;
}

/* device_makeContacts_weekday, PandemicSim.cu:1669-1829 */
static int make_contacts_weekday(const ptor_sim *s, int me, uint64_t c, int victims[8], int types[8],
                                 int *work_slots, int *work_loc)
{
    uint32_t w[8];
    tf_words(s, c, w);
    tf_words(s, c + 1, w + 4);
    int age = s->age[me];
    int hh = s->household[me];
    int hoff = s->hh_offset[hh], hcnt = s->hh_offset[hh + 1] - hoff;
    int ksum = 0;
    for (int j = 0; j < 3; j++) ksum += select_victim(me, hoff, hcnt, w[j], CONTACT_HOME, NULL, &victims[j], &types[j]);
    int made = 3;
    /* workplace / school, regenerated from the workplace counter */
    int wp = ptor_recalc_workplace(s, me, age);
    int woff = s->wp_off[wp], wcnt = s->wp_off[wp + 1] - woff;
    int desired = workplace_max_contacts(s, wp);
    int ctype = (age == AGE_ADULT) ? CONTACT_WORKPLACE : CONTACT_SCHOOL;
    int local = made;
    *work_slots = desired;
    *work_loc = wp;
    made += desired;
    while (desired > 0) {
        ksum += select_victim(me, woff, wcnt, w[local], ctype, s->wp_people, &victims[local], &types[local]);
        desired--;
        local++;
    }
    /* errands / afterschool */
    int etype = (age == AGE_ADULT) ? CONTACT_ERRAND : CONTACT_AFTERSCHOOL;
    int dests[2];
    int prof = ptor_recalc_weekday_errands(s, s->errand_rand_offset, me, age, &dests[0], &dests[1]);
    for (int hour = 0; hour < WEEKDAY_ERRAND_HOURS; hour++) {
        int want = WEEKDAY_ASSIGN[prof][hour];
        int eoff = s->eoffset[dests[hour]], ecnt = s->eoffset[dests[hour] + 1] - eoff;
        while (want > 0 && made < MAX_CONTACTS_WEEKDAY) {
            ksum += select_victim(me, eoff, ecnt, w[made], etype, s->epeople, &victims[made], &types[made]);
            want--;
            made++;
        }
    }
    while (made < MAX_CONTACTS_WEEKDAY) {
        victims[made] = -1;
        types[made] = CONTACT_NONE;
        made++;
    }
    return ksum;
}

/* device_makeContacts_weekend, PandemicSim.cu:1833-1950 */
static int make_contacts_weekend(const ptor_sim *s, int me, uint64_t c, int victims[5], int types[5])
{
    uint32_t w[4];
    tf_words(s, c, w);
    int hh = s->household[me];
    int hoff = s->hh_offset[hh], hcnt = s->hh_offset[hh + 1] - hoff;
    int ksum = 0;
    for (int j = 0; j < 3; j++) ksum += select_victim(me, hoff, hcnt, w[j], CONTACT_HOME, NULL, &victims[j], &types[j]);
    int prof = (int)(w[3] % 6u);
    /* Threefry-2x32 keyed by the low words of the seeds, counter (u32)(c+1) on
     * both words (PandemicSim.cu:1895-1901). */
    uint32_t ctr32[2] = {(uint32_t)(c + 1), (uint32_t)(c + 1)}, v[2];
    ptor_threefry2x32(ctr32, s->key32, v);
    int dests[3];
    ptor_recalc_weekend_errands(s, s->errand_rand_offset, me, dests);
    for (int k = 0; k < 2; k++) {
        int loc = dests[WEEKEND_ASSIGN[prof][k]];
        int eoff = s->eoffset[loc], ecnt = s->eoffset[loc + 1] - eoff;
        ksum += select_victim(me, eoff, ecnt, v[k], CONTACT_ERRAND, s->epeople, &victims[3 + k], &types[3 + k]);
    }
    return ksum;
}

/* device_setInfectionStatus, PandemicSim.cu:3048-3067, executed in the canonical
 * sequential order (the first attempt on a susceptible victim wins). */
static void try_infect(uint8_t *status, uint8_t *dayv, uint8_t *genv, int victim,
                       int profile, int day_to_set, int gen_to_set)
{
    if (status[victim] != STATUS_SUSCEPTIBLE) return;
    status[victim] = (uint8_t)profile;
    dayv[victim] = (uint8_t)day_to_set;
    genv[victim] = (uint8_t)gen_to_set;
}

/* device_processContacts, PandemicSim.cu:3106-3233 */
static void process_contacts(ptor_sim *s, int me, int ksum, const int *victims, const int *types,
                             int ncontacts, uint64_t c)
{
    int sp = s->status_p[me], ss = s->status_s[me];
    float prob_p = -1.f, prob_s = -1.f;
    int gen_p = GEN_NOT_INFECTED, gen_s = GEN_NOT_INFECTED;
    if (sp >= STATUS_INFECTED) {
        int pd = s->day - (int)s->day_p[me];
        if (pd >= 0 && pd < CULMINATION_PERIOD) {
            prob_p = infection_probability(s, sp - STATUS_INFECTED, pd, 0, ksum);
            gen_p = (uint8_t)(s->gen_p[me] + 1);
        }
    }
    if (ss >= STATUS_INFECTED) {
        int pd = s->day - (int)s->day_s[me];
        if (pd >= 0 && pd < CULMINATION_PERIOD) {
            prob_s = infection_probability(s, ss - STATUS_INFECTED, pd, 1, ksum);
            gen_s = (uint8_t)(s->gen_s[me] + 1);
        }
    }
    uint32_t w[16];
    for (int k = 0; k < 4; k++) tf_words(s, c + (uint64_t)k, w + 4 * k);
    int day_to_set = (uint8_t)(s->day + 1);
    int used = 0;
    for (int j = 0; j < ncontacts; j++) {
        int victim = victims[j];
        int kval = KVAL[types[j]];
        float y_p = to_unit(w[used]);
        int inf_p = y_p < (float)(prob_p * (float)kval);
        int prof_p = infection_profile(s, w[used] ^ w[(used + 1) % 16]);
        used++;
        float y_s = to_unit(w[used]);
        int inf_s = y_s < (float)(prob_s * (float)kval);
        int prof_s = infection_profile(s, w[used] ^ w[(used + 1) % 16]);
        used++;
        if (inf_p) try_infect(s->status_p, s->day_p, s->gen_p, victim, prof_p, day_to_set, gen_p);
        if (inf_s) try_infect(s->status_s, s->day_s, s->gen_s, victim, prof_s, day_to_set, gen_s);
    }
}

/* kernel_doWeekday / kernel_doWeekend with one thread, PandemicSim.cu:3236-3379:
 * counter c = R0 + 6*pos, contacts use c and c+1, processing c+2..c+5; then
 * rand_offset += 6*I (:1278-1279, :1393-1394). */
void ptor_infect(ptor_sim *s)
{
    const uint64_t R0 = s->rand_offset;
    const int weekend = is_weekend_day(s->day);
    for (int pos = 0; pos < s->infected_count; pos++) {
        int me = s->infected[pos];
        uint64_t c = R0 + (uint64_t)(6 * (int64_t)pos);
        int victims[8], types[8];
        int ksum, nc;
        if (weekend) {
            ksum = make_contacts_weekend(s, me, c, victims, types);
            nc = MAX_CONTACTS_WEEKEND;
        } else {
            int wslots = 0, wloc = 0;
            ksum = make_contacts_weekday(s, me, c, victims, types, &wslots, &wloc);
            nc = MAX_CONTACTS_WEEKDAY;
            /* interventions: a closed school or an absent adult voids the workplace /
             * school contacts, which keep their share of ksum */
            int day = s->day;
            int closed_day = day >= s->closure_start && day < s->closure_end;
            if (wslots > 0 && (s->absent_thr || closed_day)) {
                int lid = wloc % s->L;
                int school = lid >= s->type_offset[3] && lid < s->type_offset[7] + s->type_count[7];
                int closed = closed_day && school;
                int me_absent = s->age[me] == AGE_ADULT && s->absent_thr &&
                                intervention_hash(s, TAG_ABSENT, day, me) < s->absent_thr;
                for (int j = 3; j < 3 + wslots; j++) {
                    if (KVAL[types[j]] == 0) continue;
                    int v = victims[j];
                    int v_absent = s->absent_thr && s->age[v] == AGE_ADULT &&
                                   intervention_hash(s, TAG_ABSENT, day, v) < s->absent_thr;
                    if (closed || me_absent || v_absent) types[j] = CONTACT_NONE;
                }
            }
        }
        process_contacts(s, me, ksum, victims, types, nc, c + 2);
    }
    s->rand_offset += 6 * (uint64_t)s->infected_count;
}

void ptor_finish_day(ptor_sim *s) { s->day++; }

int ptor_step_day(ptor_sim *s, int counts16[16], int *infected_count)
{
    if (!s->setup_done) return -1;
    if (s->day >= s->p.max_days) return 2;
    ptor_count_and_recover(s, counts16);
    int I = ptor_build_infected(s);
    if (infected_count) *infected_count = I;
    if (I == 0) return 1;
    ptor_build_schedule(s);
    ptor_infect(s);
    ptor_finish_day(s);
    return 0;
}

void ptor_gen_counts(const ptor_sim *s, int gen_p[256], int gen_s[256])
{
    memset(gen_p, 0, 256 * sizeof(int));
    memset(gen_s, 0, 256 * sizeof(int));
    for (int i = 0; i < s->N; i++) {
        gen_p[s->gen_p[i]]++;
        gen_s[s->gen_s[i]]++;
    }
}

void ptor_get_view(const ptor_sim *s, ptor_view *v)
{
    memset(v, 0, sizeof(*v));
    v->N = s->N; v->H = s->H; v->L = s->L;
    v->adults = s->adults; v->children = s->children;
    v->infected_count = s->infected_count;
    v->current_day = s->day;
    v->rand_offset = s->rand_offset;
    v->workplace_rand_offset = s->wp_rand_offset;
    v->errand_rand_offset = s->errand_rand_offset;
    for (int i = 0; i < 4; i++) v->seeds[i] = s->seeds[i];
    for (int t = 0; t < NUM_BUSINESS_TYPES; t++) {
        v->type_count[t] = s->type_count[t];
        v->type_offset[t] = s->type_offset[t];
    }
    v->infectiousness[0] = s->infectiousness[0];
    v->infectiousness[1] = s->infectiousness[1];
    memcpy(v->shedding, s->shedding, sizeof(s->shedding));
    v->status_p = s->status_p; v->status_s = s->status_s;
    v->day_p = s->day_p; v->day_s = s->day_s;
    v->gen_p = s->gen_p; v->gen_s = s->gen_s; v->age = s->age;
    v->household = s->household; v->household_offset = s->hh_offset;
    v->workplace = s->workplace; v->workplace_people = s->wp_people;
    v->workplace_offset = s->wp_off; v->infected = s->infected;
    v->errand_keys = s->ekeys; v->errand_people = s->epeople; v->errand_offset = s->eoffset;
    v->errand_entries = s->e_entries;
    v->errand_buckets = s->e_buckets;
}

/* ------------------------------------------------------------------ */
/* Whole run with the reference's output files                         */
/* ------------------------------------------------------------------ */
static FILE *open_in(const char *dir, const char *name)
{
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    return fopen(path, "w");
}

/* runToCompletion + daily_writeInfectedStats + final_countReproduction +
 * logging_closeOutputStreams, PandemicSim.cu:877-967, :2771-2825, :2227-2304,
 * :855-866. */
int ptor_run_to_files(const ptor_params *p, int core_seed, const char *dir)
{
    ptor_sim *s = ptor_create(p, core_seed);
    if (!s) return -1;
    if (ptor_setup(s) != 0) { ptor_destroy(s); return -1; }
    FILE *fs = open_in(dir, "output_infected_stats.csv");
    if (!fs) { ptor_destroy(s); return -1; }
    fprintf(fs, "day,pandemic_susceptible,pandemic_infectious,pandemic_symptomatic,pandemic_asymptomatic,pandemic_recovered,seasonal_susceptible,seasonal_infectious,seasonal_symptomatic,seasonal_asymptomatic,seasonal_recovered\n");
    float max_prop = 0.f;
    int max_day = 0;
    int days = 0;
    while (s->day < p->max_days) {
        int c[16];
        ptor_count_and_recover(s, c);
        int sym_p = c[2] + c[3] + c[4], asym_p = c[5] + c[6] + c[7];
        int sym_s = c[10] + c[11] + c[12], asym_s = c[13] + c[14] + c[15];
        fprintf(fs, "%d,%d,%d,%d,%d,%d,%d,%d,%d,%d,%d\n", s->day, c[1], sym_p + asym_p, sym_p,
                asym_p, c[0], c[9], sym_s + asym_s, sym_s, asym_s, c[8]);
        int I = ptor_build_infected(s);
        if (I == 0) break;
        float prop = (float)I / (float)s->N;
        if (prop > max_prop) { max_prop = prop; max_day = s->day; }
        ptor_build_schedule(s);
        ptor_infect(s);
        ptor_finish_day(s);
        days++;
    }
    fclose(fs);
    int gp[256], gs[256];
    ptor_gen_counts(s, gp, gs);
    FILE *fr = open_in(dir, "output_rn.csv");
    if (fr) {
        fprintf(fr, "gen,gen_size_p,rn_p,gen_size_s,rn_s\n");
        /* lower-bound offsets over the sorted u8 generations, offsets[MAX_DAYS] = N */
        int M = p->max_days;
        long *lbp = (long *)calloc((size_t)M + 1, sizeof(long));
        long *lbs = (long *)calloc((size_t)M + 1, sizeof(long));
        long ap = 0, as = 0;
        for (int g = 0; g < M; g++) {
            lbp[g] = ap; lbs[g] = as;
            if (g < 256) { ap += gp[g]; as += gs[g]; }
        }
        lbp[M] = s->N; lbs[M] = s->N;
        for (int g = 0; g < M - 1; g++) {
            int size_p = (int)(lbp[g + 1] - lbp[g]);
            int next_p = (int)(lbp[g + 2] - lbp[g + 1]);
            float rn_p = (float)next_p / (float)size_p;
            int size_s = (int)(lbs[g + 1] - lbs[g]);
            int next_s = (int)(lbs[g + 2] - lbs[g + 1]);
            float rn_s = (float)next_s / (float)size_s;
            fprintf(fr, "%d,%d,%f,%d,%f\n", g, size_p, rn_p, size_s, rn_s);
        }
        free(lbp); free(lbs);
        fclose(fr);
    }
    FILE *fm = open_in(dir, "infected_max.txt");
    if (fm) {
        fprintf(fm, "max_proportion,day\n%f,%d\n", max_prop, max_day);
        fclose(fm);
    }
    ptor_destroy(s);
    return days;
}
