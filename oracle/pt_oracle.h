/*
 * pt_oracle.h - CPU oracle for the PandemicThrust daily simulation step.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle restates in plain C the arithmetic of
 * PandemicThrust's simulation (PandemicThrust/PandemicThrust/PandemicSim.cu and
 * host_functions.cpp) so the CUDA library can be checked bit-for-bit against it.
 * Only the test suite, the smoke entry point and the benchmark's CPU-baseline leg
 * may load it.  The product library never links or calls it.
 *
 * Infection is executed sequentially in the canonical order: infected-list
 * position ascending, then contact slot, then pandemic before seasonal.  That is
 * what the reference's kernel_doWeekday / kernel_doWeekend compute when run with a
 * single thread (PandemicSim.cu:3236-3379); with many threads the reference races
 * on atomicCAS (PandemicSim.cu:3058) and is not deterministic.
 */
#ifndef PT_ORACLE_H
#define PT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The nine numeric columns of constants.csv (PandemicSim.cu:299-309). */
typedef struct ptor_params {
    int   max_days;
    float r_pandemic;
    float r_seasonal;
    int   initial_pandemic;
    int   initial_seasonal;
    float people_scaling;
    float location_scaling;
    float percent_symptomatic;
    float asymp_factor;
} ptor_params;

typedef struct ptor_sim ptor_sim;

/* Views of the oracle's arrays (read-only for callers). */
typedef struct ptor_view {
    int N, H, L;
    int adults, children;
    int infected_count;
    int current_day;          /* next day to simulate */
    uint64_t rand_offset;
    uint64_t workplace_rand_offset;
    uint64_t errand_rand_offset;
    int seeds[4];
    int type_count[14];
    int type_offset[14];
    float infectiousness[2];
    float shedding[6][10];
    uint8_t *status_p, *status_s, *day_p, *day_s, *gen_p, *gen_s, *age;
    int32_t *household;       /* person -> household, N */
    int32_t *household_offset;/* H+1 */
    int32_t *workplace;       /* person -> workplace or school, N */
    int32_t *workplace_people;/* N, sorted by workplace, ascending ids */
    int32_t *workplace_offset;/* L+1 */
    int32_t *infected;        /* ascending infected ids, infected_count */
    int32_t *errand_keys;     /* today's schedule keys (2N weekday / 3N weekend) */
    int32_t *errand_people;   /* person ids stably sorted by key */
    int32_t *errand_offset;   /* bucket offsets (2L+1 / 10L+1) */
    int errand_entries;       /* 2N or 3N for the last built day, 0 before */
    int errand_buckets;       /* 2L or 10L */
} ptor_view;

/* Published Threefry-2x64-20 and Threefry-2x32-20 block functions. */
void ptor_threefry2x64(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2]);
void ptor_threefry2x32(const uint32_t ctr[2], const uint32_t key[2], uint32_t out[2]);

/* glibc's srand()/rand() additive-feedback generator, restated (reentrant). */
typedef struct ptor_glibc_rand { int32_t r[34]; int f, b; } ptor_glibc_rand;
void ptor_glibc_srand(ptor_glibc_rand *g, unsigned int seed);
int  ptor_glibc_rand_next(ptor_glibc_rand *g);

/* Lifecycle.  Returns NULL on invalid parameters. */
ptor_sim *ptor_create(const ptor_params *p, int core_seed);
void ptor_destroy(ptor_sim *s);
int  ptor_setup(ptor_sim *s);
/* Runs one day: count/recover, build the infected list, then (if any infected)
 * schedules, buckets and infection.  counts16 receives the 8+8 status bins.
 * Returns 0 when the day ran, 1 when the infected count was zero (the reference
 * breaks out of its loop there, PandemicSim.cu:900-901), 2 when max_days is reached. */
int  ptor_step_day(ptor_sim *s, int counts16[16], int *infected_count);
/* Sub-steps, for stage-by-stage comparisons. */
void ptor_count_and_recover(ptor_sim *s, int counts16[16]);
int  ptor_build_infected(ptor_sim *s);
void ptor_build_schedule(ptor_sim *s);
void ptor_infect(ptor_sim *s);
void ptor_finish_day(ptor_sim *s);
/* Per-generation counts for the final Rn table (256 bins each). */
void ptor_gen_counts(const ptor_sim *s, int gen_p[256], int gen_s[256]);
void ptor_get_view(const ptor_sim *s, ptor_view *v);

/* Runs a whole simulation and writes output_infected_stats.csv, output_rn.csv and
 * infected_max.txt into dir.  Returns days simulated, or -1. */
int  ptor_run_to_files(const ptor_params *p, int core_seed, const char *dir);

/* Regeneration helpers with the reference's signatures' meaning
 * (host_functions.cpp:6-268), on a set-up simulation. */
int  ptor_recalc_workplace(const ptor_sim *s, int idx, int age);
int  ptor_recalc_weekday_errands(const ptor_sim *s, uint64_t errand_offset, int idx, int age,
                                 int *dest1, int *dest2);
void ptor_recalc_weekend_errands(const ptor_sim *s, uint64_t errand_offset, int idx, int dests[3]);
void ptor_set_threads(int n);
/* Interventions (the build's extensions, no reference counterpart); before setup. */
void ptor_set_interventions(ptor_sim *s, int closure_start, int closure_days, float absenteeism, float coverage);

#ifdef __cplusplus
}
#endif
#endif
