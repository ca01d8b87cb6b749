/*
 * pandemic_gb300.h - C ABI of the GB300-native PandemicThrust daily simulation step.
 *
 * The reference has no plugin or FFI layer: its boundary is class PandemicSim
 * (PandemicThrust/PandemicThrust/PandemicSim.h:68-281) driven by main.cu:19-21,
 * plus the file contract constants.csv + seed.txt -> output_infected_stats.csv,
 * output_rn.csv, infected_max.txt.  Each entry point below names the reference
 * member or routine it replaces.  All pointers are host pointers; the library
 * owns every device buffer and never keeps a caller pointer after returning.
 *
 * A pt_sim is not thread-safe.  Its work runs on one CUDA stream (the caller's, or
 * one it creates).  Results do not depend on the stream, grid shape or GPU.
 */
#ifndef PANDEMIC_GB300_H
#define PANDEMIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pt_status {
    PT_OK = 0,
    PT_DONE = 1,          /* the infected count reached zero: the reference breaks its day loop */
    PT_FINISHED = 2,      /* max_days simulated */
    PT_ERR_ARG = -1,      /* invalid argument or parameter value */
    PT_ERR_IO = -2,       /* a file could not be opened */
    PT_ERR_PARSE = -3,    /* a file could not be parsed */
    PT_ERR_OOM = -4,      /* device or host allocation failed */
    PT_ERR_CUDA = -5,     /* a CUDA call or kernel failed */
    PT_ERR_STATE = -6,    /* call out of order (e.g. step before setup) */
    PT_ERR_TIMEOUT = -7   /* a device-side wait gave up; see pt_last_error */
} pt_status;

/* The nine numeric columns of constants.csv, in file order
 * (PandemicSim.cu:299-309; PandemicSim::setup_loadParameters). */
typedef struct pt_params {
    int   max_days;              /* 0..255: the reference's day counter is 8-bit */
    float r_pandemic;
    float r_seasonal;
    int   initial_pandemic;
    int   initial_seasonal;
    float people_scaling;        /* households = round(people_scaling * 1e6) */
    float location_scaling;      /* scales the 14 business-type counts */
    float percent_symptomatic;
    float asymp_factor;
} pt_params;

/* Sizes and derived values of a created (and set-up) simulation. */
typedef struct pt_info {
    int number_people;           /* 0 until pt_setup */
    int number_households;
    int number_workplaces;
    int number_adults;
    int number_children;
    int current_day;             /* next day to simulate */
    int days_run;                /* rows written to the daily statistics */
    int infected_count;          /* infected count of the last day counted */
    uint64_t rand_offset;        /* the reference's global Random123 counter */
    int seeds[4];                /* SEED_HOST after srand(core_seed) (PandemicSim.cu:2856-2861) */
    int type_count[14];
    int type_offset[14];
    float infectiousness[2];
    int max_day_of_peak;         /* day with the largest infected proportion */
    float max_infected_proportion;
    int sm_count;
    uint64_t device_bytes;       /* device memory held by this simulation */
    uint64_t bucket_entries_scheduled;    /* errand entries scheduled over the days run */
    uint64_t bucket_entries_materialised; /* of those, entries written to bucket tables */
} pt_info;

/* Public-health interventions.  The reference has none (its thesis, section 6.1,
 * only sketches them); these are this library's extensions, and all fields zero
 * reproduce the reference exactly.  Their random choices use a hash of (seed, day,
 * person), never the reference's random stream.
 *   school closure: on days [start, start + days) workplace / school contacts made at
 *     school-type locations (types 3-7) do not happen;
 *   workplace absenteeism: on each weekday each adult is absent from work with this
 *     probability; workplace / school contacts of an absent infector, or with an
 *     absent adult, do not happen;
 *   vaccination coverage: this fraction of persons starts recovered from both
 *     strains (initial infections are placed afterwards, as in the reference).
 * A contact that does not happen keeps its weight in the infector's contact sum, so
 * it removes transmission instead of moving it to the other contacts. */
typedef struct pt_interventions {
    int   school_closure_start;   /* first closed day, >= 0 */
    int   school_closure_days;    /* 0: schools stay open */
    float workplace_absenteeism;  /* 0..1 */
    float vaccination_coverage;   /* 0..1 */
} pt_interventions;

typedef struct pt_sim pt_sim;

/* PandemicSim::setup_loadParameters (PandemicSim.cu:286-310): the reference's
 * positional fscanf parse of constants.csv. */
pt_status pt_params_from_csv(const char *path, pt_params *out);

/* PandemicSim::setup_loadSeed (PandemicSim.cu:2843-2862): one int from seed.txt. */
pt_status pt_seed_from_file(const char *path, int *core_seed);

/* PandemicSim::PandemicSim() (PandemicSim.cu:98-133): seeds, scaling
 * (setup_scaleSimulation, :1127-1162), infection data (:2828-2840) and device
 * constants.  cuda_stream is a cudaStream_t or NULL for a library-owned stream. */
pt_status pt_create(const pt_params *params, int core_seed, void *cuda_stream, pt_sim **out);

/* PandemicSim::setupSim (PandemicSim.cu:146-208): population, households,
 * workplaces and schools, workplace table, status arrays, initial infected. */
pt_status pt_setup(pt_sim *sim);

/* One iteration of PandemicSim::runToCompletion (PandemicSim.cu:882-954):
 * daily_countAndRecover, daily_buildInfectedArray_global and, when anyone is
 * infected, doWeekday_wholeDay or doWeekend_wholeDay.  counts16 (may be NULL)
 * receives the 8 pandemic then 8 seasonal status bins counted before the day's
 * contacts (status_counts_today, :2760).  Returns PT_OK, PT_DONE when the
 * infected count was zero (no contacts ran, as the reference's break at :900) or
 * PT_FINISHED when max_days days have run.  Synchronises the stream. */
pt_status pt_step_day(pt_sim *sim, int counts16[16], int *infected_count);

/* PandemicSim::runToCompletion without per-day host synchronisation: runs the
 * remaining days on the device (captured as one CUDA graph) and copies back, per
 * day, the 16 status bins (counts, max_days*16 ints, may be NULL) and the
 * infected count (infected, max_days ints, may be NULL).  days_run receives the
 * number of statistics rows, as the reference's output_infected_stats.csv. */
pt_status pt_run(pt_sim *sim, int *counts, int *infected, int *days_run);

/* final_countReproduction (PandemicSim.cu:2227-2304): the number of persons per
 * generation value 0..255, for each strain (256 ints each). */
pt_status pt_final_gen_counts(pt_sim *sim, int gen_p[256], int gen_s[256]);

/* Resets the epidemic to the state right after pt_setup (status arrays, initial
 * infected, counters) without regenerating the population.  Used to repeat a run. */
pt_status pt_reset_epidemic(pt_sim *sim);

pt_status pt_get_info(const pt_sim *sim, pt_info *out);

/* Copies per-person state to host buffers (any may be NULL; each holds N entries):
 * status and day per strain, generation per strain, age code. */
pt_status pt_get_person_state(pt_sim *sim, uint8_t *status_p, uint8_t *status_s,
                              uint8_t *day_p, uint8_t *day_s, uint8_t *gen_p, uint8_t *gen_s,
                              uint8_t *age);

/* Copies setup tables: person -> household (N), household offsets (H+1), person ->
 * workplace or school (N), workplace people (N), workplace offsets (L+1). */
pt_status pt_get_population(pt_sim *sim, int32_t *household, int32_t *household_offset,
                            int32_t *workplace, int32_t *workplace_people,
                            int32_t *workplace_offset);

/* Copies the last built day's tables: infected list (infected_count entries),
 * schedule keys and bucketed person ids (2N weekday / 3N weekend) and bucket
 * offsets (2L+1 / 10L+1), in the reference's layout (key = hour * L + location).
 * entries and buckets receive the sizes.  By default a day materialises only the
 * buckets that its infected persons visit (the only ones the contact draws read), so
 * the person table and the offsets of the other buckets are complete only after
 * pt_set_full_tables(sim, 1). */
pt_status pt_get_day_tables(pt_sim *sim, int32_t *infected, int32_t *keys, int32_t *people,
                            int32_t *offsets, int *entries, int *buckets);

/* Sets the simulation's interventions (see pt_interventions; no counterpart in the
 * reference).  Allowed before or after pt_setup; vaccination takes effect at setup or
 * at the next pt_reset_epidemic, the others from the next day run. */
pt_status pt_set_interventions(pt_sim *sim, const pt_interventions *iv);

/* With enabled != 0 every day materialises all of its buckets, not only those its
 * infected persons visit.  Results are identical either way; this exists so the
 * tables returned by pt_get_day_tables are complete. */
pt_status pt_set_full_tables(pt_sim *sim, int enabled);

/* Device time per stage, from CUDA events recorded on the simulation's stream
 * around each stage of every day run while timing is enabled (pt_set_timing).
 * ms[0..7] sum the weekday stages, ms[8..15] the weekend stages, in the order:
 * sweep (recover, count), infected list, schedule, digit bases, bucket radix sort,
 * bucket offsets, infection, apply.
 * days[0], days[1] receive the number of weekdays and weekend days timed.  The sums
 * reset after each call.  With timing enabled, a day run by pt_step_day or pt_run
 * records events but adds no host synchronisation. */
pt_status pt_set_timing(pt_sim *sim, int enabled);
pt_status pt_get_stage_ms(pt_sim *sim, float ms[16], int days[2]);

/* The eight stage times of one day of the last timed run (zeros if that day was not
 * timed).  The drop-in executable writes them as the reference's profile_log.csv. */
pt_status pt_get_day_stage_ms(pt_sim *sim, int day, float ms[8]);

/* Launch shapes of the day's kernels.  The reference fixes its grids per device at
 * compile time (device_K20.h:4-8: 32 blocks of 256 threads); here they are chosen at
 * run time, by the caller or by pt_autotune.  Every choice gives bit-identical
 * results; only the speed differs. */
typedef struct pt_tuning {
    int infect_coop;            /* 0: one thread per infector; 1: eight lanes per infector */
    int infect_blocks_per_sm;   /* infection grid, 256-thread blocks per SM: 1..32 */
    int radix_blocks_per_sm;    /* persistent blocks of a day's radix pass per SM: 1..4
                                   (3 at 80 registers a thread, 4 at 64) */
    int sched_tf;               /* the schedule kernel's Threefry arithmetic (same results):
                                   0 integer adds and funnel shifts; 1 the 64-bit adds as
                                   multiply-adds with carry; 2 also the rotations as wide
                                   multiplies (moves work from the ALU to the FMA pipe) */
    int dense_level;            /* days whose sort reads every schedule key directly instead
                                   of entries the schedule kernel appends: 0 none; 1, 2, 3
                                   when the instance's infected are at least a quarter of,
                                   as many as, twice its buckets */
    int radix_threads;          /* threads per block of a day's radix passes: 256 (16 entries
                                   each) or 512 (8 each; radix_blocks_per_sm at most 2) */
} pt_tuning;

/* Sets / reads the launch shapes of sim (allowed before or after pt_setup). */
pt_status pt_set_tuning(pt_sim *sim, const pt_tuning *t);
pt_status pt_get_tuning(const pt_sim *sim, pt_tuning *t);

/* The tuner: after pt_setup, runs the first `days` days (0: all of max_days) once
 * per candidate launch shape with per-stage CUDA events, keeps the fastest shape for
 * the infection stage and for the radix stage (each is timed on its own stage), sets
 * it, and resets the epidemic.  Results of later runs do not depend on the choice.
 * A shape found for an engine of the same size (instances, persons, bucket counts,
 * SM count) earlier in the process is reused without timing.  chosen may be NULL. */
pt_status pt_autotune(pt_sim *sim, int days, pt_tuning *chosen);

/* Checks the error path of the library's device-side waits (no counterpart in the
 * reference, whose kernel errors go unchecked, PandemicSim.cu:2754-2761).  Every wait
 * of one thread block for another (the decoupled look-backs of the scans and sorts)
 * gives up after a bounded number of polls, records an error word and returns, and
 * the host then reports PT_ERR_TIMEOUT with the device still usable.  This runs that
 * same wait code in one small kernel, waiting for a predecessor's prefix: with
 * publish_predecessor != 0 the prefix is written first and the call returns PT_OK
 * with *prefix = 1234; with 0 nothing ever writes it, the wait gives up after
 * spin_limit polls and the call returns PT_ERR_TIMEOUT (text in pt_last_error(NULL)).
 * spin_limit must lie in [0, 2^22], the limit the simulation's own waits use, else
 * PT_ERR_ARG.  Allocates and frees 64 bytes of device memory; synchronises the device. */
pt_status pt_selftest_bounded_wait(int publish_predecessor, int64_t spin_limit, uint32_t *prefix);

/* Checks the schedule kernels' errand lookup against the reference's form of it
 * (device_fishAfterschoolOrErrandDestination_weekday, PandemicSim.cu:2909-2947, and
 * device_fishWeekendErrandDestination, :1017-1044: a loop over the errand types and
 * an IEEE division).  The kernels search without branches and divide by multiplying
 * with the reciprocal and one correction step.  counts receives: [0] weekday and [1]
 * weekend random words (all 2^32) whose errand type or quotient differs; [2] pairs
 * (x, probability) with x = 0 or any float in [2^-32, 1] (the values the search
 * divides) whose quotient differs from the IEEE division; [3] reciprocal table
 * entries that are not the rounded reciprocal.  All
 * zero is a pass.  Runs one kernel of about 2^32 iterations; synchronises the device. */
pt_status pt_selftest_errand_lookup(uint64_t counts[4]);

/* Kernel launches issued by this library in the calling process so far. */
uint64_t pt_launch_count(void);

/* Bytes this simulation has copied host-to-device and device-to-host so far. */
pt_status pt_transfer_bytes(const pt_sim *sim, uint64_t *h2d, uint64_t *d2h);

/* Largest input pt_bucket_table_static accepts: its scratch space is compiled into
 * the library, about 21 MiB of device memory, committed on a device when the
 * library's device code first loads there (its first call, or the first kernel any
 * entry point launches) and held until the process exits. */
#define PT_STATIC_TABLE_MAX_ENTRIES (1 << 20)
#define PT_STATIC_TABLE_MAX_BUCKETS (1 << 20)

/* Builds a bucket table without allocating any device memory.  No counterpart in
 * the reference: it is for callers that cannot call cudaMalloc on their path, such
 * as a host that passes in device buffers carved from its own pool and forbids any
 * other allocation, or a loop that keeps other streams busy, where cudaMalloc and
 * cudaFree would synchronise the whole device and stall that work.
 *
 * keys (device, n entries, each in [0, buckets)) -> table (device, n entries): the
 * indices 0..n-1 grouped by key, ascending within each key; offsets (device,
 * buckets+1 entries): offsets[k] = number of entries with a key below k, and
 * offsets[buckets] = n.  The same table pt_setup builds for workplaces.
 * n <= PT_STATIC_TABLE_MAX_ENTRIES and buckets <= PT_STATIC_TABLE_MAX_BUCKETS, else
 * PT_ERR_ARG; a key outside [0, buckets) also gives PT_ERR_ARG.  Work runs on
 * cuda_stream (NULL: the default stream); the call synchronises that stream and
 * returns once the table is complete, so it cannot be captured into a CUDA graph.
 * The first call on a device (or any kernel of this library) commits the scratch
 * and looks up its device address; make one call at initialisation when a memory
 * pool will later claim the device's budget.  The address is kept: do not use the
 * library across a cudaDeviceReset.
 * All calls share one scratch area, so calls that overlap on the GPU race with each
 * other: do not overlap them. */
pt_status pt_bucket_table_static(const int32_t *keys, int n, int buckets, int32_t *offsets,
                                 int32_t *table, void *cuda_stream);

/* ------------------------------------------------------------------ surrogate MLP
 * The multilayer perceptron behind the learned surrogate (no counterpart in the
 * reference): BF16 weights and activations, FP32 accumulation, FP32 master weights
 * and Adam, trained and evaluated by this library's own kernels.  layers linear
 * maps widths[0] -> widths[1] -> ... -> widths[layers]; GELU after every hidden layer
 * (its tanh form, 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))), with the hardware
 * tanh), none after the last.  Parameters are one float array, layer by layer: W (out x in,
 * row-major) then b (out).  The loss is the mean squared error over a batch. */
typedef struct pt_mlp pt_mlp;

pt_status pt_mlp_create(int layers, const int *widths, int max_batch, uint64_t seed, void *cuda_stream,
                        pt_mlp **out);
pt_status pt_mlp_param_count(const pt_mlp *mlp, int64_t *count);
pt_status pt_mlp_set_params(pt_mlp *mlp, const float *params);   /* also clears the Adam state */
pt_status pt_mlp_get_params(pt_mlp *mlp, float *params);
/* n rows of inputs (n x widths[0]) and targets (n x widths[layers]) kept on the device */
pt_status pt_mlp_set_data(pt_mlp *mlp, const float *x, const float *y, int n);
/* epochs of Adam over the data in shuffled batches; epoch_loss receives the last
 * epoch's mean loss */
pt_status pt_mlp_train(pt_mlp *mlp, int epochs, int batch, float lr, uint64_t shuffle_seed, float *epoch_loss);
/* loss and the gradient of every parameter on n <= max_batch rows (no update) */
pt_status pt_mlp_gradients(pt_mlp *mlp, const float *x, const float *y, int n, float *grads, float *loss);
pt_status pt_mlp_predict(pt_mlp *mlp, const float *x, int n, float *y);
/* the mean output of `count` networks of one shape on n rows (an ensemble): all run
 * on the first network's stream, the mean is formed on the device and copied once */
pt_status pt_mlp_predict_ensemble(pt_mlp *const *members, int count, const float *x, int n, float *y);
/* The same with x (n x widths[0]) and y (n x widths[layers]) in device memory: no
 * copies and no synchronisation; the work is queued on the first network's stream. */
pt_status pt_mlp_predict_ensemble_device(pt_mlp *const *members, int count, const float *x, int n, float *y);
/* Inference (pt_mlp_predict*) runs on the tcgen05 tensor-core kernel by default (TMA
 * operand loads into shared memory, FP32 accumulators in tensor memory) when every
 * layer is at most 256 wide and hidden widths are multiples of 32; enabled = 0
 * selects the warp-level mma.sync kernel that training uses.  Both accumulate in FP32
 * and round activations to BF16, and both evaluate the same activation step by step,
 * so they agree to FP32 summation order. */
pt_status pt_mlp_set_tcgen05(pt_mlp *mlp, int enabled);
void pt_mlp_destroy(pt_mlp *mlp);
const char *pt_mlp_last_error(const pt_mlp *mlp);

/* Returns the simulation's device memory to the library's pool.  Simulations and
 * batches take their device memory from one stream-ordered pool per GPU that keeps
 * what they free, so creating and destroying simulations of similar sizes (replicate
 * loops, scenario sweeps) reuses it instead of mapping and unmapping it each time. */
void pt_destroy(pt_sim *sim);

/* Hands the memory the pool of the current GPU keeps, and no simulation uses, back to
 * the device (cudaMemPoolTrimTo).  Call it before allocating elsewhere what the
 * library no longer needs. */
pt_status pt_trim_device_memory(void);

/* Text of the last error on sim (or of the last failed pt_create when sim is NULL). */
const char *pt_last_error(const pt_sim *sim);

/* ------------------------------------------------------------------ batches
 * A batch runs many independent simulations (replicates, scenarios, uneven sizes)
 * together: every day is one set of kernel launches over all of them, and the whole
 * day loop is one CUDA graph.  The reference runs one simulation per process; its
 * PythonBatcher scripts (write_gpu_constants.py) start one process per scenario and
 * seed.  Instance k of a batch gives exactly the results of pt_create(&params[k],
 * core_seeds[k]) run alone: statistics rows, generation counts and per-person state.
 * A pt_batch is not thread-safe and runs on one CUDA stream. */
typedef struct pt_batch pt_batch;

#define PT_BATCH_MAX_INSTANCES 4096

/* instances simulations, params[k] and core_seeds[k] each as pt_create takes them. */
pt_status pt_batch_create(const pt_params *params, const int *core_seeds, int instances, void *cuda_stream,
                          pt_batch **out);

/* setupSim of every instance, each in its own region of the batch's arrays. */
pt_status pt_batch_setup(pt_batch *batch);

/* Runs every instance to completion (its zero-infected day or max_days) and copies
 * the per-day results back; read them with pt_batch_counts. */
pt_status pt_batch_run(pt_batch *batch);

/* One day of every instance still running.  running (may be NULL) receives the
 * number of instances still running after the day.  Returns PT_DONE once no instance
 * has infected left, PT_FINISHED once the longest max_days has run. */
pt_status pt_batch_step_day(pt_batch *batch, int *running);

pt_status pt_batch_reset_epidemic(pt_batch *batch);

/* pt_set_interventions for every instance: iv holds one entry per instance. */
pt_status pt_batch_set_interventions(pt_batch *batch, const pt_interventions *iv);

/* Instance count, real persons over all instances and persons including the padding
 * that starts each instance on a 4096-person boundary. */
pt_status pt_batch_size(const pt_batch *batch, int *instances, int64_t *persons, int64_t *padded_persons);

/* Results of one instance as pt_run returns them (any pointer may be NULL). */
pt_status pt_batch_counts(const pt_batch *batch, int instance, int *counts, int *infected, int *days_run);

/* final_countReproduction of every instance: instances x 256 ints per strain. */
pt_status pt_batch_final_gen_counts(pt_batch *batch, int *gen_p, int *gen_s);

pt_status pt_batch_get_info(const pt_batch *batch, int instance, pt_info *out);

/* pt_get_person_state and pt_get_population of one instance, in its own numbering
 * (person, household and location ids as the instance run alone has them). */
pt_status pt_batch_get_person_state(pt_batch *batch, int instance, uint8_t *status_p, uint8_t *status_s,
                                    uint8_t *day_p, uint8_t *day_s, uint8_t *gen_p, uint8_t *gen_s,
                                    uint8_t *age);
pt_status pt_batch_get_population(pt_batch *batch, int instance, int32_t *household, int32_t *household_offset,
                                  int32_t *workplace, int32_t *workplace_people, int32_t *workplace_offset);

/* As pt_set_timing / pt_get_stage_ms, for the batch's days. */
pt_status pt_batch_set_timing(pt_batch *batch, int enabled);
pt_status pt_batch_get_stage_ms(pt_batch *batch, float ms[16], int days[2]);

pt_status pt_batch_transfer_bytes(const pt_batch *batch, uint64_t *h2d, uint64_t *d2h);

/* As pt_set_tuning / pt_get_tuning / pt_autotune, for the batch. */
pt_status pt_batch_set_tuning(pt_batch *batch, const pt_tuning *t);
pt_status pt_batch_get_tuning(const pt_batch *batch, pt_tuning *t);
pt_status pt_batch_autotune(pt_batch *batch, int days, pt_tuning *chosen);

void pt_batch_destroy(pt_batch *batch);

/* Text of the last error on batch (or of the last failed pt_batch_create when NULL). */
const char *pt_batch_last_error(const pt_batch *batch);

#ifdef __cplusplus
}
#endif
#endif
