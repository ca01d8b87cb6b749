"""Generate the golden fixtures in tests/golden/ from the reference itself.

Everything here comes from code of the reference, compiled for the host by
oracle/build_ref.py (the reference tree must be present, so run this where it is):
  * Threefry-2x64-20 / 2x32-20 blocks from the vendored Random123 header;
  * the C library's srand()/rand() sequence the reference draws its seeds from;
  * host_functions.cpp regeneration of workplaces and weekday/weekend errands;
  * whole runs of the reference's kernels (one-thread grid, canonical order):
    per-day status bins, infected counts, generation counts and state digests.

    python tests/golden/make_golden.py              rng.json, regen.json, runs.json
    python tests/golden/make_golden.py --headline   headline_50M_100d.json
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from oracle.oracle import RefSim, make_params, ref_lib  # noqa: E402

import ctypes  # noqa: E402

# Workloads: config 1 (100k persons x 30 days), and the reference's default scenario
# (constants.csv: R 1.8/1.3, 30/30 seeds) at 0.1 scale with asymptomatic profiles on,
# run to extinction.
RUNS = {
    "c1_100k_30d": (make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10,
                                initial_seasonal=10, people_scaling=0.04248, location_scaling=0.04248), 12345),
    "default_p0.1_asymp": (make_params(max_days=100, people_scaling=0.1, location_scaling=0.1,
                                       percent_symptomatic=0.6, asymp_factor=0.3), 777),
    "small_lscale10": (make_params(max_days=40, r_pandemic=2.0, r_seasonal=1.5, initial_pandemic=5,
                                   initial_seasonal=3, people_scaling=0.01, location_scaling=0.1), 4242),
}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rng_vectors():
    lib = ref_lib()
    rs = np.random.RandomState(20241203)
    out64, out32 = [], []
    edge = [0, 1, 2**32 - 1, 2**32, 2**63, 2**64 - 1]
    pairs = [(a, b) for a in edge for b in edge[:3]]
    for _ in range(40):
        pairs.append((int(rs.randint(0, 2**62)) * 4 + 3, int(rs.randint(0, 2**31))))
    for c, k in pairs:
        ctr = (ctypes.c_uint64 * 2)(c, c)
        key = (ctypes.c_uint64 * 2)(k, (k * 2654435761) & (2**64 - 1))
        o = (ctypes.c_uint64 * 2)()
        lib.ptref_threefry2x64(ctr, key, o)
        out64.append([str(c), str(key[0]), str(key[1]), str(o[0]), str(o[1])])
        c32 = c & 0xFFFFFFFF
        k32 = k & 0xFFFFFFFF
        ctr32 = (ctypes.c_uint32 * 2)(c32, (c32 * 7) & 0xFFFFFFFF)
        key32 = (ctypes.c_uint32 * 2)(k32, (k32 ^ 0x9E3779B9) & 0xFFFFFFFF)
        o32 = (ctypes.c_uint32 * 2)()
        lib.ptref_threefry2x32(ctr32, key32, o32)
        out32.append([ctr32[0], ctr32[1], key32[0], key32[1], o32[0], o32[1]])
    rand = {}
    for seed in [1, 0, 777, 12345, 2**31 + 3, 4294967291]:
        buf = (ctypes.c_int * 64)()
        lib.ptref_libc_rand(seed, 64, buf)
        rand[str(seed)] = list(buf)
    return {"threefry2x64": out64, "threefry2x32": out32, "libc_rand": rand}


def regen_vectors(params, seed, n=800):
    lib = ref_lib()
    sim = RefSim(params, seed)
    sim.setup()
    v = sim.view()
    rs = np.random.RandomState(seed)
    N = v["N"]
    idx = rs.randint(0, N, size=n)
    ages = [int(v["age"][i]) for i in idx]
    wp = [lib.ptref_host_recalc_workplace(int(i), a) for i, a in zip(idx, ages)]
    wd = []
    we = []
    for i, a in zip(idx, ages):
        off = int(rs.randint(0, 2**40))
        d1, d2 = ctypes.c_int(0), ctypes.c_int(0)
        prof = lib.ptref_host_recalc_weekday(off, int(i), a, ctypes.byref(d1), ctypes.byref(d2))
        wd.append([off, int(i), a, prof, d1.value, d2.value])
        out3 = (ctypes.c_int * 3)()
        lib.ptref_host_recalc_weekend(off, int(i), out3)
        we.append([off, int(i), list(out3)])
    res = dict(N=N, H=v["H"], L=v["L"], seeds=v["seeds"], type_count=v["type_count"],
               type_offset=v["type_offset"], workplace_rand_offset=v["workplace_rand_offset"],
               infectiousness=[float(x) for x in v["infectiousness"]],
               workplace=[[int(i), a, w] for i, a, w in zip(idx, ages, wp)], weekday=wd, weekend=we)
    sim.close()
    return res


def run_digest(params, seed):
    sim = RefSim(params, seed)
    sim.setup()
    v0 = sim.view()
    setup = dict(N=v0["N"], H=v0["H"], L=v0["L"], adults=v0["adults"], children=v0["children"],
                 rand_offset=v0["rand_offset"], age=digest(v0["age"]), household=digest(v0["household"]),
                 household_offset=digest(v0["household_offset"]), workplace=digest(v0["workplace"]),
                 workplace_people=digest(v0["workplace_people"]),
                 workplace_offset=digest(v0["workplace_offset"]),
                 status_p=digest(v0["status_p"]), status_s=digest(v0["status_s"]))
    days = []
    while True:
        rc, counts, infected = sim.step_day()
        if rc == 2:
            break
        v = sim.view()
        days.append(dict(rc=rc, counts=counts, infected=infected, rand_offset=v["rand_offset"],
                         status_p=digest(v["status_p"]), status_s=digest(v["status_s"]),
                         day_p=digest(v["day_p"]), day_s=digest(v["day_s"]),
                         gen_p=digest(v["gen_p"]), gen_s=digest(v["gen_s"]),
                         infected_list=digest(v["infected"][:infected]),
                         errand_people=digest(v["errand_people"]) if rc == 0 else None,
                         errand_offset=digest(v["errand_offset"]) if rc == 0 else None))
        if rc == 1:
            break
    gp, gs = sim.gen_counts()
    sim.close()
    return dict(params=params, seed=seed, setup=setup, days=days, gen_p=gp.tolist(), gen_s=gs.tolist())


# The headline workload: 50M persons x 100 days (people_scaling 21.24044, location
# scaling 10x that, R 1.5 / 1.2, 100 + 100 seeds, seed 777).  Too large for per-day
# state digests, so it records every day's bins, infected count and counter, and the
# digests of the setup tables and of the final per-person state.
HEADLINE = (make_params(max_days=100, r_pandemic=1.5, r_seasonal=1.2, initial_pandemic=100, initial_seasonal=100,
                        people_scaling=21.24044, location_scaling=212.4044), 777)


def headline_digest(params, seed):
    sim = RefSim(params, seed)
    sim.setup()
    v0 = sim.view()
    setup = dict(N=v0["N"], H=v0["H"], L=v0["L"], adults=v0["adults"], children=v0["children"],
                 rand_offset=v0["rand_offset"], age=digest(v0["age"]), household=digest(v0["household"]),
                 workplace=digest(v0["workplace"]), workplace_people=digest(v0["workplace_people"]),
                 workplace_offset=digest(v0["workplace_offset"]))
    days = []
    while True:
        rc, counts, infected = sim.step_day()
        if rc == 2:
            break
        days.append(dict(rc=rc, counts=counts, infected=infected, rand_offset=sim.view()["rand_offset"]))
        print("day", len(days) - 1, infected, flush=True)
        if rc == 1:
            break
    v = sim.view()
    final = {k: digest(v[k]) for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s")}
    gp, gs = sim.gen_counts()
    sim.close()
    return dict(params=params, seed=seed, setup=setup, days=days, final=final, gen_p=gp.tolist(),
                gen_s=gs.tolist())


def main():
    if build_ref.build() is None:
        raise SystemExit("the reference tree is needed to generate golden fixtures")
    if "--headline" in sys.argv:
        # about 40 minutes on one host core: the reference kernels run one thread
        g = headline_digest(*HEADLINE)
        path = os.path.join(HERE, "headline_50M_100d.json")
        with open(path + ".tmp", "w") as fh:
            json.dump(g, fh)
        os.replace(path + ".tmp", path)
        return
    with open(os.path.join(HERE, "rng.json"), "w") as fh:
        json.dump(rng_vectors(), fh)
    with open(os.path.join(HERE, "regen.json"), "w") as fh:
        json.dump({"c1": regen_vectors(*RUNS["c1_100k_30d"]),
                   "lscale10": regen_vectors(*RUNS["small_lscale10"]),
                   "c2_shape": regen_vectors(make_params(people_scaling=0.42481, location_scaling=4.2481), 777)},
                  fh)
    runs = {name: run_digest(p, s) for name, (p, s) in RUNS.items()}
    with open(os.path.join(HERE, "runs.json"), "w") as fh:
        json.dump(runs, fh)
    for f in ("rng.json", "regen.json", "runs.json"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
