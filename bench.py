#!/usr/bin/env python3
"""Benchmark: simulated person-days per second of the GB300-native daily step.

Workload (one GPU): 50,000,000 persons x 100 days, the reference's generator at
people_scaling 21.24044 (21.24M households) and location_scaling 212.4044 (2.72M
locations), R 1.5 / 1.2, 100 + 100 seed infections, seed 777.  Synthetic: the
population is generated by the simulation itself from its seed, as in the reference.

A step is one whole epidemic on the resident population: reset of the status arrays
and initial infected, then the 100-day loop on the device.  value =
persons x days simulated x steps / device time of the timed steps (CUDA events on
the simulation's stream).  The per-person state (~4 GB) is far larger than the
129 MB L2, so no flush is needed between steps.

e2e: the same metric through the C ABI from host buffers: pt_create -> pt_setup
(population generation) -> pt_run -> pt_final_gen_counts -> pt_destroy per step.

--impl reference times the reference's algorithm on the host cores: the CPU
restatement in oracle/ (the reference's own host code covers only schedule
regeneration, so it cannot run a day), on every host thread for the per-person
stages.  Its timed region is one whole 100-day run of the same 50M workload, cut into
the requested number of steps of consecutive days.

Parity evidence in the line (`parity`): the last timed 100-day run against the
committed run of the reference's own kernels (tests/golden/headline_50M_100d.json),
the first days against the oracle run by the CPU baseline, and every batched instance
against the same instance run alone.

Multi-GPU: replicas only (one independent simulation per rank, seed 777 + rank).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "plain_50M_persons_100_days"
PARAMS = dict(max_days=100, r_pandemic=1.5, r_seasonal=1.2, initial_pandemic=100, initial_seasonal=100,
              people_scaling=21.24044, location_scaling=212.4044, percent_symptomatic=1.0, asymp_factor=0.0)
SEED = 777
METRIC = "person-days/s on 1 GB300 (plain vs batched); surrogate scenarios/s at ≤5% error"
UNIT = "person-days/s"
FALLBACK_HBM_GBS = 6800.0

# Algorithmic bytes per launch of each stage (layout-neutral compulsory traffic,
# fields at their information size: status/day/gen/age 1 B, ids and offsets 4 B).
# E = entries of the day's schedule (2N weekday, 3N weekend); Bc = buckets a day can
# use (2 hours x locations of types 8-13 weekday, 10 hours x types 9-13 weekend).
#   sweep          4N read (status + day, both strains)
#   infected_list  4I written (the ascending infected ids)
#   schedule       weekday 1N age read + 4E keys written; weekend 4E keys written
#   digit_bases    (no compulsory traffic: the radix bookkeeping of the sort)
#   bucket_sort    4E schedule read + 4E' bucket entries written, E' = entries of the
#                  buckets that the day's infected visit (the only ones materialised)
#   bucket_offsets 4(Bc+1) offsets written (the reference's lower_bound output)
#   infect         79 B per infected weekday, 52 B weekend
#   apply          claim 8 B read + 8 B reset + state 4 B + generation 1 B per new infection
def stage_bytes(stage, weekend, N, Bc, I_mean, new_mean=0.0, mat_frac=1.0):
    E = (3 if weekend else 2) * N
    return {
        "sweep": 4 * N,
        "infected_list": 4 * I_mean,
        "schedule": (4 * E) if weekend else (N + 4 * E),
        "digit_bases": 0,
        "bucket_sort": 4 * E + 4 * E * mat_frac,
        "bucket_offsets": 4 * (Bc + 1),
        "infect": (52 if weekend else 79) * I_mean,
        "apply": 21 * new_mean,
    }[stage]


def day_bytes(weekend, N, L, I):
    """Whole-day algorithmic bytes: 13N + 8L + 83I weekday, 16N + 40L + 56I weekend."""
    return (16 * N + 40 * L + 56 * I) if weekend else (13 * N + 8 * L + 83 * I)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_records(kind):
    """`kind` lines of the committed ncu summary (profiles/ncu_traffic.txt), by stage."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    out = {}
    try:
        for line in open(path):
            if line.startswith(kind + " "):
                kv = dict(x.split("=", 1) for x in line.split()[1:])
                out[kv.pop("stage")] = kv
    except Exception:
        pass
    return out


def ncu_traffic():
    """DRAM bytes per launch of the profiled kernel, from the committed ncu summary."""
    return {k: float(v["bytes_per_launch"]) for k, v in ncu_records("traffic").items()}


def int_roof(stage, n_weekday, n_weekend):
    """The integer-pipe roof of a Threefry-bound kernel: ALU-pipe utilisation
    (IADD3/LOP3/SHF) from the committed ncu capture, weighted by this run's weekday
    and weekend launches."""
    r = ncu_records("pipe").get(stage)
    if not r:
        return None
    wd, we = float(r["alu_weekday"]), float(r["alu_weekend"])
    n = max(n_weekday + n_weekend, 1)
    return {"kernel": stage, "pipe": "alu (int32)", "frac": (wd * n_weekday + we * n_weekend) / n,
            "weekday": wd, "weekend": we, "source": "profiles/" + r["source"]}


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def apply_tuning(engine, spec):
    """Launch shapes of an engine: its tuner's choice ("auto"), the library's defaults
    ("default"), or the defaults with name=value overrides ("sched_tf=1,infect_coop=1").
    Every choice gives identical results.  Returns the shapes in use."""
    if spec == "auto":
        return engine.autotune()
    if spec != "default":
        t = engine.tuning()
        for item in spec.split(","):
            name, _, value = item.partition("=")
            if name.strip() not in t:
                raise SystemExit("--tuning: unknown launch shape %r (known: %s)" % (name, ", ".join(t)))
            t[name.strip()] = int(value)
        engine.set_tuning(t)
    return engine.tuning()


def reduce_replicas(ms, person_days, device):
    """Whole-job figures over replica ranks: total person-days and the slowest rank's
    time (max over ranks).  One independent simulation per rank, no data exchange."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    pd = torch.tensor([float(person_days)], device=device, dtype=torch.float64)
    dist.all_reduce(pd)
    return float(t.item()), float(pd.item())


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


STATE_FIELDS = ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s")
HEADLINE_GOLDEN = os.path.join(ROOT, "tests", "golden", "headline_50M_100d.json")


def state_digests(state):
    """SHA-256 of each per-person state array (equal digests: equal arrays)."""
    import hashlib
    import numpy as np
    return {k: hashlib.sha256(np.ascontiguousarray(state[k]).tobytes()).hexdigest() for k in STATE_FIELDS}


def cpu_sample(days, threads, params=PARAMS, seed=SEED):
    """The oracle on the same 50M workload: setup (untimed), then `days` simulated days
    (timed).  Also returns what the GPU's first days are checked against: each day's
    16 bins, infected count and counter offset, and the digests of the per-person
    state after the last day (recorded outside the timed region)."""
    from oracle import build_oracle
    from oracle.oracle import Oracle
    build_oracle.build()
    o = Oracle(params, seed, threads=threads)
    o.setup()
    N = o.view()["N"]
    dt = 0.0
    ran = 0
    rows = []
    for _ in range(days):
        t0 = time.perf_counter()
        rc, c, i = o.step_day()
        dt += time.perf_counter() - t0
        rows.append({"rc": rc, "counts": list(c), "infected": i, "rand_offset": o.view()["rand_offset"]})
        if rc != 0:
            break
        ran += 1
    record = {"rows": rows, "digests": state_digests(o.view())}
    o.close()
    return N, ran, dt, record


def gpu_days(sim, days):
    """The same days on the GPU through pt_step_day, from a reset of the resident
    population: the record cpu_sample returns."""
    sim.reset_epidemic()
    rows = []
    for _ in range(days):
        rc, c, i = sim.step_day()
        rows.append({"rc": rc, "counts": list(c), "infected": i, "rand_offset": sim.info()["rand_offset"]})
        if rc != 0:
            break
    return {"rows": rows, "digests": state_digests(sim.person_state())}


def parity_vs_oracle(gpu, cpu):
    """Day-by-day comparison of the GPU's first days with the oracle's, exact."""
    bad = []
    if len(gpu["rows"]) != len(cpu["rows"]):
        bad.append("days %d vs %d" % (len(gpu["rows"]), len(cpu["rows"])))
    for d, (g, c) in enumerate(zip(gpu["rows"], cpu["rows"])):
        for k in ("rc", "counts", "infected", "rand_offset"):
            if g[k] != c[k]:
                bad.append("day %d %s" % (d, k))
    for k in STATE_FIELDS:
        if gpu["digests"][k] != cpu["digests"][k]:
            bad.append("final %s" % k)
    return {"workload": WORKLOAD, "against": "oracle (C restatement), run in this bench", "days": len(cpu["rows"]),
            "compared": "per-day 16 status bins, infected count, counter offset; SHA-256 of the six per-person "
                        "state arrays after the last day",
            "equal": not bad, "mismatches": bad[:8],
            "final_state_sha256_prefix": {k: gpu["digests"][k][:16] for k in STATE_FIELDS}}


def parity_vs_golden(counts, infected, digests, gen_p, gen_s, rand_offset):
    """The timed 100-day runs against the committed run of the reference's own kernels
    (compiled for the host, one thread: the canonical order) on the same workload."""
    if not os.path.exists(HEADLINE_GOLDEN):
        return None
    try:
        with open(HEADLINE_GOLDEN) as fh:
            g = json.load(fh)
    except ValueError as e:
        return {"workload": WORKLOAD, "equal": False, "mismatches": ["unreadable golden fixture: %s" % e]}
    bad = []
    if len(g["days"]) != len(infected):
        bad.append("days %d vs %d" % (len(infected), len(g["days"])))
    for d, ref in enumerate(g["days"][:len(infected)]):
        if [int(x) for x in counts[d]] != ref["counts"]:
            bad.append("day %d counts" % d)
        if int(infected[d]) != ref["infected"]:
            bad.append("day %d infected" % d)
    if g["days"] and int(rand_offset) != g["days"][-1]["rand_offset"]:
        bad.append("final rand_offset")
    for k in STATE_FIELDS:
        if digests[k] != g["final"][k]:
            bad.append("final %s" % k)
    if [int(x) for x in gen_p] != g["gen_p"] or [int(x) for x in gen_s] != g["gen_s"]:
        bad.append("generation counts")
    return {"workload": WORKLOAD, "against": "the reference's kernels compiled for the host "
                                             "(tests/golden/headline_50M_100d.json, tests/golden/make_golden.py)",
            "days": len(g["days"]),
            "compared": "every day's 16 status bins and infected count of each timed run's last step; final "
                        "counter offset, SHA-256 of the six per-person state arrays, generation counts",
            "equal": not bad, "mismatches": bad[:8]}


def cpu_model():
    """Host CPU model and core count, for the CPU baseline's record."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                name = line.split(":", 1)[1].strip()
                if not name.isdigit():
                    break
    except Exception:
        pass
    return {"model": name, "nproc": os.cpu_count()}


# Single-thread oracle figures (the reference's CPU path has no engine of its own that
# runs a day): the 100,000-person x 30-day workload and a 1M-person run shaped like
# the 50M one (same location ratio, R, seeds).
SINGLE_THREAD_WORKLOADS = {
    "c1_100k_persons_30_days": (dict(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10,
                                     initial_seasonal=10, people_scaling=0.04248, location_scaling=0.04248,
                                     percent_symptomatic=1.0, asymp_factor=0.0), 12345),
    "c2_shape_1M_persons_30_days": (dict(max_days=30, r_pandemic=1.5, r_seasonal=1.2, initial_pandemic=100,
                                         initial_seasonal=100, people_scaling=0.42481, location_scaling=4.2481,
                                         percent_symptomatic=1.0, asymp_factor=0.0), 777),
}


def single_thread_baselines():
    from oracle.oracle import Oracle
    out = {}
    for name, (p, seed) in SINGLE_THREAD_WORKLOADS.items():
        o = Oracle(p, seed, threads=1)
        o.setup()
        N = o.view()["N"]
        t0 = time.perf_counter()
        days = 0
        for _ in range(p["max_days"]):
            rc, _, _ = o.step_day()
            if rc == 2:
                break
            days += 1
            if rc == 1:
                break
        dt = time.perf_counter() - t0
        o.close()
        out[name] = {"value": N * days / dt, "unit": UNIT, "persons": N, "days": days, "seconds": dt, "cores": 1}
    return out


def workload_config(N, H, L, max_days):
    """The `config` object both arms print: the workload, not the hardware."""
    return {"workload": WORKLOAD, "persons": N, "households": H, "locations": L, "days": max_days,
            "l2": "inputs larger than L2 (about 4 GB of per-person state)"}


def run_reference(args, world, rank):
    """The reference's algorithm on the host cores (the oracle restatement, every host
    thread on the per-person stages).  The timed region is one whole 100-day run of
    the workload, cut into `steps` steps of ceil(100 / steps) consecutive days; the
    warm-up steps run the same days on a separate copy of the population first."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import build_oracle
    from oracle.oracle import Oracle
    build_oracle.build()
    params = dict(PARAMS)
    params["people_scaling"] = PARAMS["people_scaling"] * args.scale
    params["location_scaling"] = PARAMS["location_scaling"] * args.scale
    max_days = params["max_days"]
    per = max(1, -(-max_days // max(args.steps, 1)))

    def steps_of(o, nsteps):
        dt, days = 0.0, 0
        for _ in range(nsteps):
            t0 = time.perf_counter()
            for _ in range(per):
                rc, _, _ = o.step_day()
                if rc == 2:
                    break
                days += 1
                if rc == 1:
                    break
            dt += time.perf_counter() - t0
        return dt, days

    o = Oracle(params, SEED, threads=threads)
    o.setup()
    steps_of(o, min(args.warmup, -(-max_days // per)))
    o.close()
    o = Oracle(params, SEED, threads=threads)
    o.setup()
    v = o.view()
    N, H, L = v["N"], v["H"], v["L"]
    dt, days = steps_of(o, args.steps)
    o.close()
    value = N * days / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/i32/f32",
        "data": "synthetic (the reference's generator, seed 777)",
        "config": workload_config(N, H, L, max_days),
        "parallelism": "%d host threads" % threads,
        "days_per_step": per, "days_simulated": days,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "host": cpu_model(),
                         "sample": "%d persons, days 0-%d of one run (%d per step), setup excluded; %d warm-up "
                                   "steps on a separate copy" % (N, days - 1, per, args.warmup)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_plain_l_eq_p(pt, torch, stream, tuning, steps=2):
    """The same 50M-person population with one location per household unit
    (location_scaling = people_scaling: 271,872 locations instead of 2.72M), the
    thesis-style shape: fewer, larger buckets.  Same launch shapes as the main run;
    device time of `steps` 100-day runs after one warm-up run."""
    params = dict(PARAMS, location_scaling=PARAMS["people_scaling"])
    sim = pt.PandemicSim(params, SEED, stream=ctypes.c_void_p(stream.cuda_stream))
    sim.setupSim()
    sim.set_tuning(tuning)
    info = sim.info()
    sim.reset_epidemic()
    sim.runToCompletion()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    days = 0
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        sim.reset_epidemic()
        _, inf = sim.runToCompletion()
        days += len(inf)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    sim.close()
    N = info["number_people"]
    return {"workload": "plain_50M_persons_l_eq_p_100_days", "persons": N, "locations": info["number_workplaces"],
            "value": N * days / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
            "note": "location_scaling = people_scaling; the headline uses 10x as many locations"}


def run_batched(args, pt, torch, stream, local):
    """The batched workload (256 uneven instances x 100 days, one batch) and the same
    instances run one after another through the plain path, both timed with CUDA
    events on the same stream after warm-up."""
    from pandemicthrust_gb300 import scenarios
    params, seeds = scenarios.batched_workload(count=args.batch_instances)
    sp = ctypes.c_void_p(stream.cuda_stream)
    b = pt.PandemicBatch(params, seeds, stream=sp)
    b.setup()
    # launch shapes for this batch (part of the warm-up)
    tuning = apply_tuning(b, args.tuning)
    K, persons, padded = b.size()
    sizes = [b.info(k)["number_people"] for k in range(K)]
    for _ in range(args.batch_warmup):
        b.reset_epidemic()
        b.run()
    sampler = ClockSampler(local)
    torch.cuda.synchronize()
    sampler.start()
    launches0 = pt.launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    person_days = 0
    for _ in range(args.batch_steps):
        b.reset_epidemic()
        b.run()
        person_days += sum(n * int(d) for n, d in zip(sizes, b.days_run()))
    t1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = pt.launch_count() - launches0
    ms = t0.elapsed_time(t1)
    value = person_days / (ms / 1000.0)
    days = b.days_run()
    # each instance's results of the last timed step (read after the timed region),
    # for the comparison with the same instance run alone below
    bgp, bgs = b.final_gen_counts()
    batch_results = []
    for k in range(K):
        c, i = b.counts(k)
        batch_results.append((c, i, bgp[k], bgs[k], state_digests(b.person_state(k))))
    # stage breakdown: one more run with per-stage CUDA events (outside the timed region)
    b.set_timing(True)
    b.reset_epidemic()
    b.run()
    stages, _ = b.stage_ms()
    b.set_timing(False)
    tot = {n: stages["weekday"][n] + stages["weekend"][n] for n in pt.PandemicSim.STAGES}
    run_ms = sum(tot.values())
    breakdown = {n: {"ms": round(v, 2), "share": round(v / run_ms, 4) if run_ms else None} for n, v in tot.items()}
    infected_days = 0
    for k in range(K):
        infected_days += int(b.counts(k)[1].sum())
    b.close()
    # e2e: create + setup + run + generation counts + destroy through the C ABI
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b2 = pt.PandemicBatch(params, seeds, stream=sp)
    b2.setup()
    apply_tuning(b2, args.tuning)   # auto: the shapes chosen above for this size (cached: no timing runs)
    b2.run()
    b2.final_gen_counts()
    e2e_pd = sum(n * int(d) for n, d in zip(sizes, b2.days_run()))
    h2d, d2h = b2.transfer_bytes()
    b2.close()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    # the same instances run one after another through the plain path (each after one
    # warm-up run, so its day loop is already a captured graph)
    plain_ms = 0.0
    plain_pd = 0
    identical = 0
    differing = []
    import numpy as np
    for k, (p, sd) in enumerate(zip(params, seeds)):
        sim = pt.PandemicSim(p, sd, stream=sp)
        sim.setupSim()
        sim.runToCompletion()
        sim.reset_epidemic()
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        cnt, inf = sim.runToCompletion()
        a1.record(stream)
        torch.cuda.synchronize()
        plain_ms += a0.elapsed_time(a1)
        plain_pd += sim.info()["number_people"] * len(inf)
        # bit-identity of instance k with its run alone
        gp, gs = sim.final_gen_counts()
        c, i, bgp_k, bgs_k, dig = batch_results[k]
        same = (np.array_equal(c, cnt) and np.array_equal(i, inf) and np.array_equal(bgp_k, gp) and
                np.array_equal(bgs_k, gs) and dig == state_digests(sim.person_state()))
        if same:
            identical += 1
        else:
            differing.append(k)
        sim.close()
    plain_value = plain_pd / (plain_ms / 1000.0)
    return {
        "workload": "batched_%d_instances_100_days" % K, "instances": K, "persons": persons,
        "padded_persons": padded, "value": value, "unit": UNIT, "steps": args.batch_steps,
        "warmup": args.batch_warmup, "ms_per_step": ms / args.batch_steps,
        "days_run": {"min": int(min(days)), "max": int(max(days)), "mean": float(sum(days)) / K},
        "gpu_launches": launches,
        "tuning": tuning,
        "stages": breakdown,
        "infected_fraction_mean": infected_days / max(float(sum(n * int(d) for n, d in zip(sizes, days))), 1.0),
        "e2e": {"value": e2e_pd / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "plain_sequential": {"value": plain_value, "unit": UNIT, "ms": plain_ms,
                             "note": "each instance alone through the plain path, device time of its run"},
        "speedup_vs_plain_sequential": value / plain_value,
        "parity": {"instances": K, "bit_identical_instances": identical, "equal": identical == K,
                   "differing_instances": differing[:16],
                   "compared": "each instance of the batch against the same parameters and seed run alone "
                               "through the plain path: every statistics row, generation counts, SHA-256 of "
                               "the six per-person state arrays"},
        "config": "persons log-uniform in [2e5, 4e6], R per strain uniform in [1.1, 2.0], 10 + 10 seeds, "
                  "seed 1000 + k, inputs larger than L2",
        "clocks": clocks,
    }


def run_surrogate(args):
    """The learned surrogate at 1,000,000 persons per scenario.

    The headline model is the ensemble shipped with the package
    (`surrogate.SHIPPED_MODEL`, made on a GB300 by `python -m
    pandemicthrust_gb300.surrogate build`; the file records how).  It is scored on
    scenarios it has never seen (new parameter draws, new core seeds): the error of
    peak height and attack rate against the mean of `reps` simulator replicates, and
    its scenarios/s against the batched simulator's.  A single network is also
    trained here from scratch (`--surrogate-train` scenarios, one run each) to time
    the trainer, with nearest neighbour in its training set as the baseline."""
    import numpy as np
    from pandemicthrust_gb300 import surrogate as sg
    persons, ntest, reps = 1_000_000, 256, 32
    rng = np.random.default_rng(2025)
    train = sg.sample_scenarios(args.surrogate_train, rng)
    test = sg.sample_scenarios(ntest, rng)
    t0 = time.time()
    te = sg.simulate(test, reps, persons, seed_base=50_000_000)
    t_test_sim = time.time() - t0
    truth = sg.truth_summary(te)
    abm_rate = ntest * reps / t_test_sim

    def errors(pred):
        pk, at = sg.relative_errors(sg.predicted_summary(pred), truth)
        pd = sg.peak_day_errors(pred, truth)
        return {"peak_height_median": float(np.median(pk)), "peak_height_mean": float(np.mean(pk)),
                "attack_rate_median": float(np.median(at)), "attack_rate_mean": float(np.mean(at)),
                "peak_day_abs_days_median": float(np.median(pd)), "peak_day_abs_days_mean": float(np.mean(pd)),
                "pairs": int(len(pk)), "min_attack": 0.01}

    X = sg.features(sg.sample_scenarios(262144, np.random.default_rng(5)))
    out = {"workload": "surrogate_1M_persons", "test_scenarios": ntest, "test_replicates": reps,
           "network": "11 -> 4 x 256 GELU -> %d, BF16 weights, FP32 accumulate and Adam" % sg.OUTPUTS,
           "abm_scenarios_per_s": abm_rate,
           "target": "<=5% relative error on peak height and attack rate; >=1000x scenarios/s"}
    seconds = {"test_data": t_test_sim}
    if os.path.exists(sg.SHIPPED_MODEL):
        import torch
        s = sg.Surrogate.load(sg.SHIPPED_MODEL, max_batch=262144)   # one chunk: 13.5 row tiles per SM
        pred, _ = s.predict(test)
        # device time of the ensemble's kernels alone (inputs and outputs resident),
        # CUDA events on the networks' stream (the legacy default stream)
        xd = torch.from_numpy(X).cuda()
        yd = torch.empty((len(X), sg.OUTPUTS), dtype=torch.float32, device="cuda")
        s.raw_device(xd.data_ptr(), 4096, yd.data_ptr())
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(torch.cuda.default_stream())
        s.raw_device(xd.data_ptr(), len(X), yd.data_ptr())
        ev1.record(torch.cuda.default_stream())
        torch.cuda.synchronize()
        t_dev = ev0.elapsed_time(ev1) / 1000.0
        flops = 2.0 * len(X) * len(s.nets) * sum(a * b for a, b in zip(s.nets[0].widths[:-1], s.nets[0].widths[1:]))
        out["inference_device"] = {"scenarios_per_s": len(X) / t_dev, "seconds": t_dev, "flop": flops,
                                   "tflops": flops / t_dev / 1e12, "rows": len(X), "members": len(s.nets)}
        del xd, yd
        # end to end from pinned host memory: features in, ensemble-mean outputs back
        Xp = torch.from_numpy(X).pin_memory().numpy()
        Yp = torch.empty((len(X), sg.OUTPUTS), dtype=torch.float32).pin_memory().numpy()
        members = (ctypes.c_void_p * len(s.nets))(*[net.h.value for net in s.nets])
        fp = ctypes.POINTER(ctypes.c_float)
        lib = s.nets[0].lib
        lib.pt_mlp_predict_ensemble(members, len(s.nets), Xp.ctypes.data_as(fp), 4096, Yp.ctypes.data_as(fp))
        t0 = time.time()
        rc = lib.pt_mlp_predict_ensemble(members, len(s.nets), Xp.ctypes.data_as(fp), len(X), Yp.ctypes.data_as(fp))
        t_inf = time.time() - t0
        assert rc == 0
        out["model"] = dict(s.info, file=os.path.relpath(sg.SHIPPED_MODEL, ROOT), members=len(s.nets))
        out["error"] = errors(pred)
        out["scenarios_per_s"] = len(X) / t_inf
        out["scenarios_per_s_measures"] = ("end to end through pt_mlp_predict_ensemble: features from pinned host "
                                           "memory, every member, the mean copied back to pinned host memory")
        out["speedup"] = out["scenarios_per_s"] / abm_rate
        seconds["inference"] = t_inf
        if args.search_judge > 0:
            # the surrogate-screened intervention search at 50M persons: 100,000 candidates
            # scored by the surrogate, the best `search_judge` of the top 1% judged by 32
            # simulator replicates each
            t0 = time.time()
            out["search_50M"] = sg.search(s, persons=50_000_000, candidates=100_000, budget_days=28,
                                          top_fraction=0.01, judge_top=args.search_judge, replicates=32)
            seconds["search_50M"] = time.time() - t0
        s.close()
    if args.surrogate_train:
        t0 = time.time()
        tr = sg.simulate(train, 1, persons, seed_base=10_000)
        t_train_sim = time.time() - t0
        Y = sg.targets(tr)[:, 0, :]
        s = sg.Surrogate(persons, seed=1)
        t0 = time.time()
        val_loss = s.fit(train, Y, epochs=400, batch=512)
        t_fit = time.time() - t0
        pred, _ = s.predict(test)
        nn = sg.decode(sg.nearest_neighbour(sg.features(train), Y, sg.features(test)), persons)
        s.nets[0].predict(X[:4096])
        t0 = time.time()
        s.nets[0].predict(X)
        t_inf1 = time.time() - t0
        s.close()
        fit = {"train_scenarios": len(train), "members": 1, "error": errors(pred),
               "nearest_neighbour_error": errors(nn), "validation_mse": val_loss,
               "scenarios_per_s": len(X) / t_inf1,
               "seconds": {"train_data": t_train_sim, "fit": t_fit, "inference": t_inf1}}
        out["in_bench_fit"] = fit
        if "error" not in out:   # no shipped model: the network trained here is the result
            out["error"] = fit["error"]
            out["scenarios_per_s"] = fit["scenarios_per_s"]
            out["speedup"] = fit["scenarios_per_s"] / abm_rate
    out["seconds"] = seconds
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-days", type=int, default=7)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=256,
                    help="instances of the batched workload (0: skip it)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--batch-warmup", type=int, default=3)
    ap.add_argument("--only-batched", action="store_true", help="run the batched workload alone")
    ap.add_argument("--surrogate-train", type=int, default=16384,
                    help="training scenarios of the network the surrogate section trains (0: none)")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate section")
    ap.add_argument("--search-judge", type=int, default=4,
                    help="intervention search at 50M: top-1%% scenarios re-simulated (32 replicates each; 0: skip)")
    ap.add_argument("--only-surrogate", action="store_true", help="run the surrogate section alone")
    ap.add_argument("--tuning", default="auto",
                    help="launch shapes: auto (pt_autotune), default (the library's), or name=value pairs, e.g. "
                         "sched_tf=1,infect_coop=1 (profiling captures of tuned shapes without the tuner's runs)")
    ap.add_argument("--no-lp", action="store_true", help="skip the location_scaling = people_scaling run")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="population scale (profiling captures only; the bench line is for 1.0)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import pandemicthrust_gb300 as pt
    pt.build()
    stream = torch.cuda.Stream()
    if args.only_batched:
        if rank == 0:
            print(json.dumps(run_batched(args, pt, torch, stream, local)))
        return 0
    if args.only_surrogate:
        if rank == 0:
            print(json.dumps(run_surrogate(args)))
        return 0
    seed = SEED + rank
    params = dict(PARAMS)
    params["people_scaling"] = PARAMS["people_scaling"] * args.scale
    params["location_scaling"] = PARAMS["location_scaling"] * args.scale
    sim = pt.PandemicSim(params, seed, stream=ctypes.c_void_p(stream.cuda_stream))
    sim.setupSim()
    info = sim.info()
    N, L = info["number_people"], info["number_workplaces"]
    Bc_wd = 2 * (L - info["type_offset"][8])
    Bc_we = 10 * (L - info["type_offset"][9])
    # launch shapes (untimed, before the warm-up)
    tuning = apply_tuning(sim, args.tuning)

    # warm-up steps (untimed)
    for _ in range(args.warmup):
        sim.reset_epidemic()
        sim.runToCompletion()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = pt.launch_count()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    days_total = 0
    for _ in range(args.steps):
        sim.reset_epidemic()
        counts, infected = sim.runToCompletion()
        days_total += len(infected)
    end.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    launches = pt.launch_count() - launches0
    ms = start.elapsed_time(end)
    if world > 1:
        ms, person_days = reduce_replicas(ms, float(N) * days_total, "cuda")
    else:
        person_days = float(N) * days_total
    value = person_days / (ms / 1000.0)
    # parity of the last timed step (read after the timed region) against the
    # committed run of the reference's own kernels on the same workload
    golden = None
    if rank == 0 and args.scale == 1.0 and seed == SEED:
        gp, gs = sim.final_gen_counts()
        golden = parity_vs_golden(counts, infected, state_digests(sim.person_state()), gp, gs,
                                  sim.info()["rand_offset"])

    # stage breakdown: one more step with per-stage CUDA events (outside the timed region)
    sim.set_timing(True)
    sim.reset_epidemic()
    counts, infected = sim.runToCompletion()
    stages, (nwd, nwe) = sim.stage_ms()
    sim.set_timing(False)
    tinfo = sim.info()
    mat_frac = tinfo["bucket_entries_materialised"] / max(tinfo["bucket_entries_scheduled"], 1)
    days = len(infected)
    I_wd = [int(infected[d]) for d in range(days) if d % 7 < 5]
    I_we = [int(infected[d]) for d in range(days) if d % 7 >= 5]
    Imean_wd = sum(I_wd) / max(len(I_wd), 1)
    Imean_we = sum(I_we) / max(len(I_we), 1)
    # new infections of day d: drop of the susceptible bins (index 1 and 9) to day d+1
    new = [int(counts[d][1] - counts[d + 1][1] + counts[d][9] - counts[d + 1][9]) for d in range(days - 1)] + [0]
    new_wd = sum(new[d] for d in range(days) if d % 7 < 5) / max(len(I_wd), 1)
    new_we = sum(new[d] for d in range(days) if d % 7 >= 5) / max(len(I_we), 1)
    run_ms = sum(stages["weekday"].values()) + sum(stages["weekend"].values())
    breakdown = {}
    for name in pt.PandemicSim.STAGES:
        tot = stages["weekday"][name] + stages["weekend"][name]
        byt = (stage_bytes(name, False, N, Bc_wd, Imean_wd, new_wd, mat_frac) * nwd +
               stage_bytes(name, True, N, Bc_we, Imean_we, new_we, mat_frac) * nwe)
        breakdown[name] = {"ms": round(tot, 3), "share": round(tot / run_ms, 4) if run_ms else None,
                           "GBps": round(byt / (tot / 1000.0) / 1e9, 1) if tot > 0 and byt > 0 else None}
    dominant = max(pt.PandemicSim.STAGES, key=lambda n: stages["weekday"][n] + stages["weekend"][n])
    dom_ms = stages["weekday"][dominant] + stages["weekend"][dominant]
    dom_launches = nwd + nwe
    dom_bytes = (stage_bytes(dominant, False, N, Bc_wd, Imean_wd, new_wd, mat_frac) * nwd +
                 stage_bytes(dominant, True, N, Bc_we, Imean_we, new_we, mat_frac) * nwe) / max(dom_launches, 1)
    achieved = dom_bytes / (dom_ms / dom_launches / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic().get(dominant)
    all_bytes = sum(day_bytes(d % 7 >= 5, N, L, int(infected[d])) for d in range(days))
    day_achieved = all_bytes / (run_ms / 1000.0) / 1e9

    # the first days again through pt_step_day, for the comparison with the oracle
    gpu_first_days = gpu_days(sim, args.cpu_days) if (rank == 0 and world == 1 and not args.no_cpu) else None

    # e2e: whole pipeline through the C ABI from host buffers
    e2e_value = None
    h2d = d2h = 0
    if args.e2e_steps > 0:
        sim.close()
        e2e_days = 0
        e2e_start = torch.cuda.Event(enable_timing=True)
        e2e_end = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e2e_start.record(stream)
        for _ in range(args.e2e_steps):
            s2 = pt.PandemicSim(params, seed, stream=ctypes.c_void_p(stream.cuda_stream))
            s2.setupSim()
            apply_tuning(s2, args.tuning)   # auto: the shapes chosen above for this size (cached: no timing runs)
            c2, i2 = s2.runToCompletion()
            s2.final_gen_counts()
            e2e_days += len(i2)
            a, b = s2.transfer_bytes()
            h2d += a
            d2h += b
            s2.close()
        e2e_end.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e2e_start.elapsed_time(e2e_end)
        e2e_value = N * e2e_days / (e2e_ms / 1000.0) * (world if world > 1 else 1)
        h2d //= args.e2e_steps
        d2h //= args.e2e_steps
    else:
        sim.close()

    plain_lp = None
    if world == 1 and args.scale == 1.0 and not args.no_lp:
        plain_lp = run_plain_l_eq_p(pt, torch, stream, tuning)

    batched = None
    if args.batch_instances > 0 and world == 1:
        batched = run_batched(args, pt, torch, stream, local)
    surrogate = None
    if not args.no_surrogate and world == 1:
        surrogate = run_surrogate(args)

    cpu = None
    oracle_parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cN, cdays, cdt, record = cpu_sample(args.cpu_days, threads, params, seed)
        oracle_parity = parity_vs_oracle(gpu_first_days, record)
        cpu = {"value": cN * cdays / cdt, "unit": UNIT, "cores": threads, "kind": "port", "host": cpu_model(),
               "sample": "oracle (C restatement) on the same %d-person workload, days 0-%d (setup excluded), "
                         "%d host threads" % (cN, cdays - 1, threads),
               "single_thread": single_thread_baselines()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/i32/f32",
            "data": "synthetic (the reference's population generator, seed 777 + rank)",
            "config": workload_config(N, info["number_households"], L, params["max_days"]),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "days_per_step": days_total / args.steps,
            "parity": {"plain_50M_vs_reference_kernels_100_days": golden,
                       "plain_50M_vs_oracle_first_days": oracle_parity,
                       "batched_instances_vs_alone": batched.get("parity") if batched else None},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "tuning": tuning,
            "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": ("mean DRAM bytes per launch over one 100-day run of this workload, "
                                            "one-pass ncu capture (profiles/ncu_schedule_traffic_50M.md, "
                                            "profiles/ncu_traffic.txt)") if traffic else None},
            "int_roofline": int_roof(dominant, nwd, nwe),
            "day_roofline": {"achieved": day_achieved, "peak": peak, "unit": "GB/s", "frac": day_achieved / peak,
                             "bytes_per_run": all_bytes},
            "stages": breakdown,
            "buckets_materialised_fraction": round(mat_frac, 4),
            "cpu_baseline": cpu,
            "clocks": clocks,
            "plain_l_eq_p": plain_lp,
            "batched": batched,
            "surrogate": surrogate,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
