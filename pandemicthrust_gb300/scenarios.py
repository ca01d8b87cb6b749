"""Scenario lists for batches of simulations.

``batched_workload`` draws the batched replicate/scenario workload: ``count``
instances whose population sizes are log-uniform in [2e5, 4e6] persons (the
reference's generator at people_scaling = N / 2.354e6, expected household size
2.354, and location_scaling = people_scaling), reproduction numbers uniform in
[1.1, 2.0] per strain, 10 + 10 seed infections and seed 1000 + k, 100 days.  The
draws come from a fixed-seed host generator, so the list is the same everywhere.
"""
import csv

import numpy as np

EXPECTED_HOUSEHOLD_SIZE = 2.354  # persons per household of the reference's household table

FIELDS = ("max_days", "r_pandemic", "r_seasonal", "initial_pandemic", "initial_seasonal", "people_scaling",
          "location_scaling", "percent_symptomatic", "asymp_factor")


def scenario(max_days=100, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=30, initial_seasonal=30,
             people_scaling=1.0, location_scaling=1.0, percent_symptomatic=1.0, asymp_factor=0.0):
    """One instance's constants.csv values (the reference's defaults)."""
    return dict(max_days=max_days, r_pandemic=r_pandemic, r_seasonal=r_seasonal,
                initial_pandemic=initial_pandemic, initial_seasonal=initial_seasonal,
                people_scaling=people_scaling, location_scaling=location_scaling,
                percent_symptomatic=percent_symptomatic, asymp_factor=asymp_factor)


def batched_workload(count=256, min_persons=2e5, max_persons=4e6, days=100, seed_infections=10, rng_seed=20240):
    """(params list, core seeds list) of the batched workload."""
    rng = np.random.default_rng(rng_seed)
    params, seeds = [], []
    for k in range(count):
        n = float(np.exp(rng.uniform(np.log(min_persons), np.log(max_persons))))
        p = float(np.float32(n / (EXPECTED_HOUSEHOLD_SIZE * 1e6)))
        params.append(scenario(max_days=days, r_pandemic=float(np.float32(rng.uniform(1.1, 2.0))),
                               r_seasonal=float(np.float32(rng.uniform(1.1, 2.0))),
                               initial_pandemic=seed_infections, initial_seasonal=seed_infections,
                               people_scaling=p, location_scaling=p))
        seeds.append(1000 + k)
    return params, seeds


def write_csv(path, params, seeds):
    """One row per instance: the core seed, then the nine constants.csv values."""
    with open(path, "w", newline="") as fh:
        w = csv.writer(fh)
        w.writerow(("seed",) + FIELDS)
        for p, s in zip(params, seeds):
            w.writerow([s] + [p[f] for f in FIELDS])


def read_csv(path):
    params, seeds = [], []
    with open(path, newline="") as fh:
        for row in csv.DictReader(fh):
            seeds.append(int(row["seed"]))
            params.append({f: (int(row[f]) if f in ("max_days", "initial_pandemic", "initial_seasonal")
                               else float(row[f])) for f in FIELDS})
    return params, seeds
