"""The learned surrogate: scenario parameters -> 100-day epidemic curves.

A small multilayer perceptron (this library's own BF16/FP32 kernels, ``pt_mlp_*``)
maps a scenario -- reproduction number per strain, seed infections, school-closure
start and length, workplace absenteeism and vaccination coverage -- to the daily
infected counts of each strain over 100 days (log1p-scaled), the final attack rate of
each strain and the generational reproduction numbers of the first generations.  It
is trained on data the batched simulator generates (``simulate``) and judged
against the mean of replicate runs.  Scenarios outside the training ranges fall back
to the simulator itself.

The reference has no surrogate and no interventions; both are this build's
extensions, built on the batched engine (``PandemicBatch``) and the intervention
hooks (``pt_set_interventions``).
"""
import ctypes

import numpy as np

from . import PandemicBatch, PtError, load_library, PT_OK

DAYS = 100
GENERATIONS = 8          # generational Rn of generations 0..7 per strain
RN_SCALE = 4.0
OUTPUTS = 2 * DAYS + 2 + 2 * GENERATIONS
EXPECTED_HOUSEHOLD_SIZE = 2.354

# scenario ranges (inclusive); seeds are sampled and encoded on a log scale
RANGES = {
    "r_pandemic": (1.1, 2.0),
    "r_seasonal": (1.1, 2.0),
    "seeds": (10, 1000),
    "closure_start": (0, 60),
    "closure_days": (0, 42),
    "absenteeism": (0.0, 0.3),
    "vaccination": (0.0, 0.5),
}
FEATURES = tuple(RANGES)


class MLP:
    """The surrogate's network on the current CUDA device (``pt_mlp_*``)."""

    def __init__(self, widths, max_batch=4096, seed=0, stream=None):
        self.lib = lib = load_library()
        vp, fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
        lib.pt_mlp_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_uint64, vp,
                                      ctypes.POINTER(vp)]
        lib.pt_mlp_param_count.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
        lib.pt_mlp_set_params.argtypes = [vp, fp]
        lib.pt_mlp_get_params.argtypes = [vp, fp]
        lib.pt_mlp_set_data.argtypes = [vp, fp, fp, ctypes.c_int]
        lib.pt_mlp_train.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint64, fp]
        lib.pt_mlp_gradients.argtypes = [vp, fp, fp, ctypes.c_int, fp, fp]
        lib.pt_mlp_predict.argtypes = [vp, fp, ctypes.c_int, fp]
        lib.pt_mlp_destroy.argtypes = [vp]
        lib.pt_mlp_last_error.argtypes = [vp]
        lib.pt_mlp_last_error.restype = ctypes.c_char_p
        self.widths = [int(w) for w in widths]
        self.max_batch = int(max_batch)
        arr = (ctypes.c_int * len(self.widths))(*self.widths)
        h = vp()
        rc = lib.pt_mlp_create(len(self.widths) - 1, arr, self.max_batch, int(seed), stream, ctypes.byref(h))
        if rc != PT_OK:
            raise PtError(rc, lib.pt_mlp_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc != PT_OK:
            raise PtError(rc, self.lib.pt_mlp_last_error(self.h).decode())

    @staticmethod
    def _f(a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    def param_count(self):
        n = ctypes.c_int64(0)
        self._check(self.lib.pt_mlp_param_count(self.h, ctypes.byref(n)))
        return n.value

    def get_params(self):
        p = np.zeros(self.param_count(), np.float32)
        self._check(self.lib.pt_mlp_get_params(self.h, self._f(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self.lib.pt_mlp_set_params(self.h, self._f(p)))

    def set_data(self, X, Y):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        self._check(self.lib.pt_mlp_set_data(self.h, self._f(X), self._f(Y), len(X)))

    def train(self, epochs, batch=256, lr=1e-3, seed=0):
        loss = ctypes.c_float(0)
        self._check(self.lib.pt_mlp_train(self.h, int(epochs), int(batch), float(lr), int(seed), ctypes.byref(loss)))
        return loss.value

    def gradients(self, X, Y):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float(0)
        self._check(self.lib.pt_mlp_gradients(self.h, self._f(X), self._f(Y), len(X), self._f(g),
                                              ctypes.byref(loss)))
        return g, loss.value

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), self.widths[-1]), np.float32)
        self._check(self.lib.pt_mlp_predict(self.h, self._f(X), len(X), self._f(Y)))
        return Y

    def close(self):
        if getattr(self, "h", None):
            self.lib.pt_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ scenarios
def sample_scenarios(n, rng):
    """n scenarios drawn uniformly in RANGES (seeds log-uniform, closure days integer)."""
    out = []
    for _ in range(n):
        lo, hi = RANGES["seeds"]
        out.append({
            "r_pandemic": float(rng.uniform(*RANGES["r_pandemic"])),
            "r_seasonal": float(rng.uniform(*RANGES["r_seasonal"])),
            "seeds": int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))),
            "closure_start": int(rng.integers(RANGES["closure_start"][0], RANGES["closure_start"][1] + 1)),
            "closure_days": int(rng.integers(RANGES["closure_days"][0], RANGES["closure_days"][1] + 1)),
            "absenteeism": float(rng.uniform(*RANGES["absenteeism"])),
            "vaccination": float(rng.uniform(*RANGES["vaccination"])),
        })
    return out


def in_range(scenarios):
    """True for scenarios inside the training ranges."""
    return np.array([all(RANGES[f][0] <= s[f] <= RANGES[f][1] for f in FEATURES) for s in scenarios])


def features(scenarios):
    """Inputs of the network: each feature scaled to [0, 1] over its range (seeds on a log scale)."""
    X = np.zeros((len(scenarios), len(FEATURES)), np.float32)
    for i, s in enumerate(scenarios):
        for j, f in enumerate(FEATURES):
            lo, hi = RANGES[f]
            v = s[f]
            if f == "seeds":
                v, lo, hi = np.log(v), np.log(lo), np.log(hi)
            X[i, j] = (v - lo) / (hi - lo)
    return X


def _params_and_interventions(s, persons):
    p = persons / (EXPECTED_HOUSEHOLD_SIZE * 1e6)
    params = dict(max_days=DAYS, r_pandemic=s["r_pandemic"], r_seasonal=s["r_seasonal"],
                  initial_pandemic=int(s["seeds"]), initial_seasonal=int(s["seeds"]), people_scaling=p,
                  location_scaling=p, percent_symptomatic=1.0, asymp_factor=0.0)
    iv = dict(school_closure_start=int(s["closure_start"]), school_closure_days=int(s["closure_days"]),
              workplace_absenteeism=float(s["absenteeism"]), vaccination_coverage=float(s["vaccination"]))
    return params, iv


def simulate(scenarios, replicates=1, persons=100_000, seed_base=1000, max_persons_per_batch=300_000_000):
    """Runs every scenario `replicates` times on the batched simulator.

    Returns a dict of arrays indexed [scenario, replicate, ...]: ``daily`` (DAYS x 2
    infected per day and strain, zero after the epidemic ends), ``attack`` (2, the
    fraction ever infected), ``rn`` (GENERATIONS x 2), ``persons``.  Replicate r of
    scenario i uses core seed seed_base + i * replicates + r.
    """
    n, R = len(scenarios), int(replicates)
    daily = np.zeros((n, R, DAYS, 2), np.float64)
    attack = np.zeros((n, R, 2), np.float64)
    rn = np.zeros((n, R, GENERATIONS, 2), np.float64)
    npers = np.zeros((n, R), np.int64)
    jobs = [(i, r) for i in range(n) for r in range(R)]
    per_batch = max(1, min(4096, int(max_persons_per_batch // max(persons, 1))))
    for c0 in range(0, len(jobs), per_batch):
        chunk = jobs[c0:c0 + per_batch]
        params, ivs, seeds = [], [], []
        for i, r in chunk:
            p, iv = _params_and_interventions(scenarios[i], persons)
            params.append(p)
            ivs.append(iv)
            seeds.append(seed_base + i * R + r)
        b = PandemicBatch(params, seeds)
        b.set_interventions(ivs)
        b.setup()
        b.run()
        gp, gs = b.final_gen_counts()
        for k, (i, r) in enumerate(chunk):
            counts, infected = b.counts(k)
            N = b.info(k)["number_people"]
            npers[i, r] = N
            d = len(counts)
            daily[i, r, :d, 0] = counts[:, 2:8].sum(axis=1)
            daily[i, r, :d, 1] = counts[:, 10:16].sum(axis=1)
            for s_, g in enumerate((gp[k], gs[k])):
                attack[i, r, s_] = (N - g[255]) / N
                size = g[:GENERATIONS].astype(np.float64)
                nxt = g[1:GENERATIONS + 1].astype(np.float64)
                rn[i, r, :, s_] = np.where(size > 0, nxt / np.maximum(size, 1), 0.0)
        b.close()
    return {"daily": daily, "attack": attack, "rn": rn, "persons": npers}


def targets(sim):
    """Network targets, one row per (scenario, replicate): log1p(daily) / log1p(N) for
    each strain, the attack rates, and Rn / RN_SCALE."""
    n, R = sim["attack"].shape[:2]
    N = sim["persons"].reshape(n, R, 1, 1).astype(np.float64)
    d = np.log1p(sim["daily"]) / np.log1p(N)
    Y = np.concatenate([d[..., 0].reshape(n, R, DAYS), d[..., 1].reshape(n, R, DAYS), sim["attack"],
                        sim["rn"][..., 0] / RN_SCALE, sim["rn"][..., 1] / RN_SCALE], axis=2)
    return Y.astype(np.float32)


def decode(Y, persons):
    """Network outputs -> daily infected (n x DAYS x 2), attack rates (n x 2), Rn."""
    Y = np.asarray(Y, np.float64)
    L = np.log1p(persons)
    daily = np.stack([np.expm1(np.clip(Y[:, :DAYS], 0, None) * L),
                      np.expm1(np.clip(Y[:, DAYS:2 * DAYS], 0, None) * L)], axis=2)
    attack = np.clip(Y[:, 2 * DAYS:2 * DAYS + 2], 0.0, 1.0)
    rn = np.stack([Y[:, 2 * DAYS + 2:2 * DAYS + 2 + GENERATIONS], Y[:, 2 * DAYS + 2 + GENERATIONS:]], axis=2)
    return {"daily": daily, "attack": attack, "rn": rn * RN_SCALE}


def summary(daily, attack):
    """Peak height (infected on the peak day), peak day and attack rate per strain."""
    return {"peak": daily.max(axis=1), "peak_day": daily.argmax(axis=1), "attack": np.asarray(attack)}


def relative_errors(pred, truth, min_attack=0.01):
    """|pred - truth| / truth of peak height and attack rate, for (scenario, strain)
    pairs whose reference attack rate is at least min_attack (an epidemic that dies
    out at once has no meaningful relative error)."""
    mask = truth["attack"] >= min_attack
    pk = np.abs(pred["peak"] - truth["peak"]) / np.maximum(truth["peak"], 1e-9)
    at = np.abs(pred["attack"] - truth["attack"]) / np.maximum(truth["attack"], 1e-9)
    return pk[mask], at[mask]


class Surrogate:
    """MLP surrogate for one population size, with the simulator as fallback."""

    def __init__(self, persons=100_000, hidden=256, depth=4, seed=0, max_batch=4096):
        self.persons = int(persons)
        self.net = MLP([len(FEATURES)] + [hidden] * depth + [OUTPUTS], max_batch=max_batch, seed=seed)

    def fit(self, scenarios, Y, epochs=1500, batch=256, lr=1e-3, seed=0):
        """Trains on one target row per scenario (average replicates before, or pass
        each replicate as its own row)."""
        self.net.set_data(features(scenarios), Y)
        return self.net.train(epochs, batch=batch, lr=lr, seed=seed)

    def predict(self, scenarios, fallback_replicates=4, seed_base=900_000):
        """Decoded predictions; scenarios outside the training ranges are simulated
        instead (mean of fallback_replicates runs).  Also returns the fallback mask."""
        ok = in_range(scenarios)
        out = decode(self.net.predict(features(scenarios)), self.persons)
        if not ok.all():
            idx = np.nonzero(~ok)[0]
            sim = simulate([scenarios[i] for i in idx], fallback_replicates, self.persons, seed_base)
            out["daily"][idx] = sim["daily"].mean(axis=1)
            out["attack"][idx] = sim["attack"].mean(axis=1)
            out["rn"][idx] = sim["rn"].mean(axis=1)
        return out, ~ok

    def close(self):
        self.net.close()


def nearest_neighbour(train_X, train_Y, X):
    """The method without the network: each query takes the targets of the nearest
    training scenario in feature space."""
    d = ((X[:, None, :] - train_X[None, :, :]) ** 2).sum(axis=2)
    return train_Y[d.argmin(axis=1)]
