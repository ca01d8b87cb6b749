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
import json
import os
import time

import numpy as np

from . import PandemicBatch, PtError, load_library, PT_OK

DAYS = 100
GENERATIONS = 8          # generational Rn of generations 0..7 per strain
RN_SCALE = 4.0
# outputs: daily infected (2 x DAYS), then per strain attack rate, peak height and
# peak day, then Rn (2 x GENERATIONS)
OUTPUTS = 2 * DAYS + 6 + 2 * GENERATIONS
# the six summary targets (attack rate, peak height, peak day per strain) are scaled
# up so the squared error weighs them as much as the 200 daily values together
SUMMARY_WEIGHT = 5.0
EXPECTED_HOUSEHOLD_SIZE = 2.354
# the hidden layers' activation, as the kernels evaluate it (pt_mlp.cu): a saved
# network trained with another one is refused
ACTIVATION = "gelu_tanh"

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
# the surrogate shipped with the package (1,000,000 persons per scenario; made by
# `python -m pandemicthrust_gb300.surrogate build --out <this path>`)
SHIPPED_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "surrogate_1m.npz")


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
        lib.pt_mlp_predict_ensemble.argtypes = [ctypes.POINTER(vp), ctypes.c_int, fp, ctypes.c_int, fp]
        lib.pt_mlp_predict_ensemble_device.argtypes = [ctypes.POINTER(vp), ctypes.c_int, vp, ctypes.c_int, vp]
        lib.pt_mlp_set_tcgen05.argtypes = [vp, ctypes.c_int]
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

    def set_tcgen05(self, enabled=True):
        """Inference on the tcgen05 kernel (default) or on the mma.sync kernel training uses."""
        self._check(self.lib.pt_mlp_set_tcgen05(self.h, 1 if enabled else 0))

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


N_DERIVED = 4


def features(scenarios):
    """Inputs of the network: each scenario parameter scaled to [0, 1] over its range
    (seeds on a log scale), then derived inputs that the dynamics depend on directly:
    each strain's reproduction number left after vaccination, R (1 - coverage), the
    day schools reopen, and the closed days within the first 60 days."""
    X = np.zeros((len(scenarios), len(FEATURES) + N_DERIVED), np.float32)
    for i, s in enumerate(scenarios):
        for j, f in enumerate(FEATURES):
            lo, hi = RANGES[f]
            v = s[f]
            if f == "seeds":
                v, lo, hi = np.log(v), np.log(lo), np.log(hi)
            X[i, j] = (v - lo) / (hi - lo)
        j = len(FEATURES)
        X[i, j] = s["r_pandemic"] * (1 - s["vaccination"]) / RANGES["r_pandemic"][1]
        X[i, j + 1] = s["r_seasonal"] * (1 - s["vaccination"]) / RANGES["r_seasonal"][1]
        end = s["closure_start"] + s["closure_days"]
        X[i, j + 2] = end / DAYS
        X[i, j + 3] = max(0, min(end, 60) - min(s["closure_start"], 60)) / 60.0
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
    fraction ever infected), ``rn`` (GENERATIONS x 2), ``persons``, ``days`` (days
    simulated, the statistics rows of the run).  Replicate r of
    scenario i uses core seed seed_base + i * replicates + r.
    """
    n, R = len(scenarios), int(replicates)
    daily = np.zeros((n, R, DAYS, 2), np.float64)
    attack = np.zeros((n, R, 2), np.float64)
    rn = np.zeros((n, R, GENERATIONS, 2), np.float64)
    npers = np.zeros((n, R), np.int64)
    ndays = np.zeros((n, R), np.int64)
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
            ndays[i, r] = d
            daily[i, r, :d, 0] = counts[:, 2:8].sum(axis=1)
            daily[i, r, :d, 1] = counts[:, 10:16].sum(axis=1)
            for s_, g in enumerate((gp[k], gs[k])):
                attack[i, r, s_] = (N - g[255]) / N
                size = g[:GENERATIONS].astype(np.float64)
                nxt = g[1:GENERATIONS + 1].astype(np.float64)
                rn[i, r, :, s_] = np.where(size > 0, nxt / np.maximum(size, 1), 0.0)
        b.close()
    return {"daily": daily, "attack": attack, "rn": rn, "persons": npers, "days": ndays}


def targets(sim):
    """Network targets, one row per (scenario, replicate), each roughly in [0, 1]:
    log1p(daily infected) / log1p(N) for each strain; per strain log1p(attack * N) /
    log1p(N), log1p(peak height) / log1p(N) and peak day / DAYS; Rn / RN_SCALE.  Log
    scales make squared errors behave like relative errors."""
    n, R = sim["attack"].shape[:2]
    N = sim["persons"].reshape(n, R, 1).astype(np.float64)
    L = np.log1p(N)
    d = np.log1p(sim["daily"]) / L[..., None]
    peak = sim["daily"].max(axis=2)                       # n x R x 2
    peak_day = sim["daily"].argmax(axis=2) / DAYS
    w = SUMMARY_WEIGHT
    Y = np.concatenate([d[..., 0], d[..., 1], w * np.log1p(sim["attack"] * N) / L, w * np.log1p(peak) / L,
                        w * peak_day, sim["rn"][..., 0] / RN_SCALE, sim["rn"][..., 1] / RN_SCALE], axis=2)
    return Y.astype(np.float32)


def decode(Y, persons):
    """Network outputs -> daily infected (n x DAYS x 2) and, per strain, attack rate,
    peak height and peak day (n x 2), and Rn (n x GENERATIONS x 2)."""
    Y = np.asarray(Y, np.float64)
    L = np.log1p(persons)
    o = 2 * DAYS
    daily = np.stack([np.expm1(np.clip(Y[:, :DAYS], 0, None) * L),
                      np.expm1(np.clip(Y[:, DAYS:o], 0, None) * L)], axis=2)
    S = Y[:, o:o + 6] / SUMMARY_WEIGHT
    attack = np.clip(np.expm1(np.clip(S[:, 0:2], 0, None) * L) / persons, 0.0, 1.0)
    peak = np.expm1(np.clip(S[:, 2:4], 0, None) * L)
    peak_day = np.clip(np.rint(S[:, 4:6] * DAYS), 0, DAYS - 1)
    rn = np.stack([Y[:, o + 6:o + 6 + GENERATIONS], Y[:, o + 6 + GENERATIONS:]], axis=2)
    return {"daily": daily, "attack": attack, "peak": peak, "peak_day": peak_day, "rn": rn * RN_SCALE}


def truth_summary(sim):
    """The judge of the surrogate: per scenario and strain, the mean over replicates of
    peak height (infected on the peak day), peak day and attack rate."""
    return {"peak": sim["daily"].max(axis=2).mean(axis=1), "peak_day": sim["daily"].argmax(axis=2).mean(axis=1),
            "attack": sim["attack"].mean(axis=1)}


def predicted_summary(pred):
    """The same quantities as the surrogate predicts them."""
    return {"peak": pred["peak"], "peak_day": pred["peak_day"], "attack": pred["attack"]}


def peak_day_errors(pred, truth, min_attack=0.01):
    """|predicted - reference| peak day in days, over the same pairs as
    relative_errors (the reference is the mean peak day of the replicates)."""
    mask = truth["attack"] >= min_attack
    return np.abs(np.asarray(pred["peak_day"], np.float64) - truth["peak_day"])[mask]


def relative_errors(pred, truth, min_attack=0.01):
    """|pred - truth| / truth of peak height and attack rate, for (scenario, strain)
    pairs whose reference attack rate is at least min_attack (an epidemic that dies
    out at once has no meaningful relative error)."""
    mask = truth["attack"] >= min_attack
    pk = np.abs(pred["peak"] - truth["peak"]) / np.maximum(truth["peak"], 1e-9)
    at = np.abs(pred["attack"] - truth["attack"]) / np.maximum(truth["attack"], 1e-9)
    return pk[mask], at[mask]


class Surrogate:
    """MLP surrogate for one population size (an ensemble of `members` networks
    averaged in target space), with the simulator as fallback."""

    # fractions of the epochs and their learning rates: a stepped decay
    SCHEDULE = ((0.5, 1e-3), (0.3, 3e-4), (0.2, 1e-4))

    def __init__(self, persons=100_000, hidden=256, depth=4, seed=0, max_batch=4096, members=1):
        self.persons = int(persons)
        self.nets = [MLP([len(FEATURES) + N_DERIVED] + [hidden] * depth + [OUTPUTS], max_batch=max_batch,
                         seed=seed + 7919 * i)
                     for i in range(members)]

    def fit(self, scenarios, Y, epochs=400, batch=512, val_fraction=0.1, checks=16, seed=0, average_last=None):
        """Trains every member on one target row per scenario (average replicates
        before, or pass each replicate as its own row), holding out val_fraction of
        the rows; the learning rate follows SCHEDULE over `epochs`.

        Each member ends with the average of its weights after each of the last
        `average_last` epochs (Polyak averaging; by default the last phase of
        SCHEDULE).  The targets are single noisy runs, so the checkpoint that best
        fits the held-out runs is not the one closest to the replicate mean, and the
        average is: on 131,072 scenarios it halves a single network's error against
        the replicate mean.  average_last=0 keeps the checkpoint with the best
        validation loss instead, measured `checks` times.  Returns the mean final
        validation loss."""
        X = np.asarray(features(scenarios), np.float32)
        Y = np.asarray(Y, np.float32)
        order = np.random.default_rng(seed).permutation(len(X))
        nv = int(len(X) * val_fraction)
        val, trn = order[:nv], order[nv:]
        rates = [r for f, r in self.SCHEDULE for _ in range(max(1, int(round(epochs * f))))]
        total = len(rates)
        avg = int(round(epochs * self.SCHEDULE[-1][0])) if average_last is None else int(average_last)
        avg = max(0, min(avg, total))
        start_avg = total - avg
        step = max(1, epochs // checks)
        losses = []
        for i, net in enumerate(self.nets):
            net.set_data(X[trn], Y[trn])
            best, best_params = np.inf, net.get_params()
            acc, nacc = None, 0
            e = 0
            while e < total:
                n = 1
                if e < start_avg:   # whole chunks of equal rate up to the next check
                    while n < step and e + n < start_avg and rates[e + n] == rates[e]:
                        n += 1
                net.train(n, batch=batch, lr=rates[e], seed=seed + 101 * i + 7 * e)
                e += n
                if e > start_avg:
                    p = net.get_params().astype(np.float64)
                    acc = p if acc is None else acc + p
                    nacc += 1
                elif nv and not avg:
                    v = float(np.mean((net.predict(X[val]) - Y[val]) ** 2))
                    if v < best:
                        best, best_params = v, net.get_params()
            if avg:
                net.set_params((acc / nacc).astype(np.float32))
            elif nv:
                net.set_params(best_params)
            losses.append(float(np.mean((net.predict(X[val]) - Y[val]) ** 2)) if nv else float("nan"))
        return float(np.mean(losses))

    def raw(self, scenarios):
        """Ensemble mean of the network outputs (target space) for scenario dicts."""
        return self.raw_features(features(scenarios))

    def raw_features(self, X):
        """The same for rows of features() already computed.  The members' mean is
        formed on the device (`pt_mlp_predict_ensemble`) and copied back once."""
        X = np.ascontiguousarray(X, np.float32)
        net0 = self.nets[0]
        Y = np.zeros((len(X), net0.widths[-1]), np.float32)
        members = (ctypes.c_void_p * len(self.nets))(*[net.h.value for net in self.nets])
        net0._check(net0.lib.pt_mlp_predict_ensemble(members, len(self.nets), MLP._f(X), len(X), MLP._f(Y)))
        return Y

    def raw_device(self, x_ptr, n, y_ptr):
        """The ensemble mean on device buffers (float32, n x inputs -> n x outputs),
        queued on the first network's stream without copies or synchronisation."""
        net0 = self.nets[0]
        members = (ctypes.c_void_p * len(self.nets))(*[net.h.value for net in self.nets])
        net0._check(net0.lib.pt_mlp_predict_ensemble_device(members, len(self.nets), ctypes.c_void_p(x_ptr), int(n),
                                                             ctypes.c_void_p(y_ptr)))

    def predict(self, scenarios, fallback_replicates=4, seed_base=900_000):
        """Decoded predictions; scenarios outside the training ranges are simulated
        instead (mean of fallback_replicates runs).  Also returns the fallback mask."""
        ok = in_range(scenarios)
        out = decode(self.raw(scenarios), self.persons)
        if not ok.all():
            idx = np.nonzero(~ok)[0]
            sim = simulate([scenarios[i] for i in idx], fallback_replicates, self.persons, seed_base)
            t = truth_summary(sim)
            out["daily"][idx] = sim["daily"].mean(axis=1)
            out["attack"][idx] = t["attack"]
            out["peak"][idx] = t["peak"]
            out["peak_day"][idx] = t["peak_day"]
            out["rn"][idx] = sim["rn"].mean(axis=1)
        return out, ~ok

    # ------------------------------------------------------------ saved models
    def _meta(self):
        return dict(_encoding(), persons=self.persons, widths=self.nets[0].widths, members=len(self.nets))

    def save(self, path, **info):
        """Writes every member's parameters as inference uses them: weight matrices as
        BF16, biases in FP32 (the GEMM epilogue adds the FP32 bias), with the model's
        shape and target encoding (and any `info`, e.g. how it was trained)."""
        mask = _bias_mask(self.nets[0].widths)
        p = [net.get_params() for net in self.nets]
        meta = dict(self._meta(), info=info)
        np.savez_compressed(path, params=np.stack([_bf16_bits(q) for q in p]),
                            biases=np.stack([q[mask] for q in p]), meta=np.array(json.dumps(meta)))

    @classmethod
    def load(cls, path, max_batch=4096):
        """A surrogate saved by save(); refuses a file whose features, ranges or
        target encoding differ from this module's."""
        z = np.load(path)
        meta = json.loads(str(z["meta"]))
        for k, v in _encoding().items():
            if meta.get(k) != v:
                raise ValueError("%s: %s is %r, this module has %r" % (path, k, meta.get(k), v))
        w = meta["widths"]
        if w[0] != len(FEATURES) + N_DERIVED or w[-1] != OUTPUTS or len(set(w[1:-1])) != 1:
            raise ValueError("%s: layer widths %r do not fit this module's network" % (path, w))
        s = cls(meta["persons"], hidden=w[1], depth=len(w) - 2, max_batch=max_batch, members=meta["members"])
        mask = _bias_mask(w)
        for net, bits, bias in zip(s.nets, z["params"], z["biases"]):
            v = _bf16_values(bits)
            v[mask] = bias
            net.set_params(v)
        s.info = meta.get("info", {})
        return s

    def close(self):
        for net in self.nets:
            net.close()


def _encoding():
    """What a saved surrogate must share with this module: its inputs and targets."""
    return dict(features=list(FEATURES), ranges={k: list(v) for k, v in RANGES.items()}, days=DAYS,
                generations=GENERATIONS, rn_scale=RN_SCALE, summary_weight=SUMMARY_WEIGHT, n_derived=N_DERIVED,
                outputs=OUTPUTS, activation=ACTIVATION)


def _bias_mask(widths):
    """Bias positions in the parameter array: each layer stores W (out x in), then b."""
    return np.concatenate([np.r_[np.zeros(widths[i] * widths[i + 1], bool), np.ones(widths[i + 1], bool)]
                           for i in range(len(widths) - 1)])


def _bf16_bits(a):
    """float32 -> BF16 bit patterns, rounded to nearest even (as the device rounds)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_values(bits):
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def nearest_neighbour(train_X, train_Y, X):
    """The method without the network: each query takes the targets of the nearest
    training scenario in feature space."""
    T = np.asarray(train_X, np.float64)
    Q = np.asarray(X, np.float64)
    tn = (T * T).sum(axis=1)
    best = np.empty(len(Q), np.int64)
    step = max(1, (1 << 24) // max(len(T), 1))   # about 128 MB of distances at a time
    for q0 in range(0, len(Q), step):
        q = Q[q0:q0 + step]
        # |q - t|^2 = |q|^2 - 2 q.t + |t|^2; |q|^2 does not change the argmin
        best[q0:q0 + step] = (tn[None, :] - 2.0 * (q @ T.T)).argmin(axis=1)
    return np.asarray(train_Y)[best]


def evaluate(surrogate, scenarios, replicates, seed_base):
    """Errors of a surrogate against the mean of `replicates` simulator runs of each
    scenario, and the time both took."""
    t0 = time.time()
    sim = simulate(scenarios, replicates, surrogate.persons, seed_base=seed_base)
    t_sim = time.time() - t0
    t0 = time.time()
    pred = decode(surrogate.raw(scenarios), surrogate.persons)
    t_pred = time.time() - t0
    truth = truth_summary(sim)
    pk, at = relative_errors(predicted_summary(pred), truth)
    pd = peak_day_errors(pred, truth)
    return {"pairs": int(len(pk)), "peak_median": float(np.median(pk)), "peak_mean": float(np.mean(pk)),
            "attack_median": float(np.median(at)), "attack_mean": float(np.mean(at)),
            "peak_day_abs_median": float(np.median(pd)), "peak_day_abs_mean": float(np.mean(pd)),
            "simulate_s": t_sim, "predict_s": t_pred}


# ------------------------------------------------------------------ intervention search
# Scenarios of the search: the pandemic and seasonal strains at R 1.5 / 1.2 with fixed
# seeding, and the four interventions drawn from their ranges, school closure capped
# by the closure-days budget.
SEARCH_R = (1.5, 1.2)
SEARCH_SEEDS_PER_MILLION = 20


def search_scenarios(n, rng, budget_days, vaccination=0.2):
    """n intervention scenarios for the search: R fixed at SEARCH_R, seeds fixed (per
    million persons; the surrogate takes them in its own population's numbers), the
    vaccination coverage fixed (the doses at hand), closure start uniform in its
    range, closure length uniform in [0, budget_days], absenteeism uniform in its
    range."""
    lo, hi = RANGES["closure_start"]
    out = []
    for _ in range(n):
        out.append({
            "r_pandemic": SEARCH_R[0], "r_seasonal": SEARCH_R[1], "seeds": SEARCH_SEEDS_PER_MILLION,
            "closure_start": int(rng.integers(lo, hi + 1)),
            "closure_days": int(rng.integers(0, budget_days + 1)),
            "absenteeism": float(rng.uniform(*RANGES["absenteeism"])),
            "vaccination": float(vaccination),
        })
    return out


def scaled(scenario, persons, model_persons):
    """The scenario for a population of `persons`: seed infections scale with the
    population (same infected fraction at the start), everything else is kept."""
    s = dict(scenario)
    s["seeds"] = max(1, int(round(scenario["seeds"] * persons / model_persons)))
    return s


def transfer(pred, persons, model_persons):
    """Predictions made at the model's population, carried to `persons` in fractions:
    the network's population and the target's have the same structure per person
    (households, schools, workplaces and errand locations all scale with persons), so
    daily infected and peak height scale by persons / model_persons and attack rate
    and peak day are kept."""
    f = persons / float(model_persons)
    out = dict(pred)
    out["daily"] = pred["daily"] * f
    out["peak"] = pred["peak"] * f
    return out


def search(surrogate, persons=50_000_000, candidates=100_000, budget_days=28, top_fraction=0.01, judge_top=None,
           replicates=32, seed=2026, seed_base=300_000_000, max_persons_per_batch=700_000_000, vaccination=0.2,
           transfer_sample=4):
    """Surrogate-screened intervention search.

    Scores `candidates` random intervention scenarios with the surrogate (minimal
    attack rate, both strains summed, under the closure-days budget), keeps the top
    `top_fraction`, and re-simulates the best `judge_top` of those (default: all of
    them) with `replicates` runs each at `persons` on the batched simulator, which
    judges the surrogate (peak height and attack rate errors against the replicate
    mean, over every judged scenario and strain) and makes the final choice (the
    fallback: the simulator's best, not the surrogate's, is returned).  The best
    scenarios often stop the epidemic early, and so do most candidates of the search
    (R 1.5 / 1.2 with 20% vaccinated), so `transfer_sample` scenarios drawn from the
    surrogate's whole training ranges are simulated the same way at `persons` and
    their errors reported apart: the error of the model trained at its own population
    when carried to this one (pairs with a simulated attack rate of at least 1%).
    Returns a dict of the timings, errors and choices."""
    rng = np.random.default_rng(seed)
    scen = search_scenarios(candidates, rng, budget_days, vaccination)
    X = features(scen)
    surrogate.raw_features(X[:min(len(X), 4096)])   # warm-up
    t0 = time.time()
    Y = surrogate.raw_features(X)
    t_score = time.time() - t0
    pred = transfer(decode(Y, surrogate.persons), persons, surrogate.persons)
    score = pred["attack"].sum(axis=1)
    order = np.argsort(score, kind="stable")
    top = order[:max(1, int(round(candidates * top_fraction)))]
    judged = top if judge_top is None else top[:max(1, int(judge_top))]
    sample = sample_scenarios(int(transfer_sample), rng) if transfer_sample else []
    pred_sample = transfer(decode(surrogate.raw_features(features(sample)), surrogate.persons), persons,
                           surrogate.persons) if sample else None
    big = [scaled(scen[i], persons, surrogate.persons) for i in judged] + \
        [scaled(x, persons, surrogate.persons) for x in sample]
    t0 = time.time()
    sim = simulate(big, replicates, persons, seed_base=seed_base, max_persons_per_batch=max_persons_per_batch)
    t_sim = time.time() - t0
    truth = truth_summary(sim)
    nj = len(judged)

    def errs(p, rows_pred, rows_truth, min_attack):
        if p is None:
            return {"pairs": 0, "min_attack": min_attack}
        sub = {k: np.asarray(v)[rows_pred] for k, v in p.items()}
        t = {k: v[rows_truth] for k, v in truth.items()}
        pk, at = relative_errors(predicted_summary(sub), t, min_attack)
        if not len(pk):
            return {"pairs": 0, "min_attack": min_attack}
        return {"peak_height_median": float(np.median(pk)), "peak_height_mean": float(np.mean(pk)),
                "attack_rate_median": float(np.median(at)), "attack_rate_mean": float(np.mean(at)),
                "pairs": int(len(pk)), "min_attack": min_attack}

    person_days = float((sim["persons"] * sim["days"]).sum())
    abm_score = truth["attack"][:nj].sum(axis=1)
    best_abm = int(np.argmin(abm_score))
    return {
        "persons": int(sim["persons"].mean()), "candidates": candidates, "budget_closure_days": budget_days,
        "vaccination": vaccination,
        "top": int(len(top)), "judged": nj, "transfer_sample": int(len(sample)), "replicates": replicates,
        "surrogate_scenarios_per_s": candidates / t_score, "surrogate_seconds": t_score,
        "abm_seconds": t_sim, "abm_runs": int(len(big) * replicates),
        "abm_person_days_per_s": person_days / t_sim,
        "error_judged": errs(pred, judged, np.arange(nj), 0.0),
        "error_transfer": errs(pred_sample, np.arange(len(sample)), np.arange(nj, len(big)), 0.01),
        "transfer_scenarios": sample,
        "surrogate_choice": dict(scen[int(judged[0])], predicted_attack=[float(x) for x in pred["attack"][judged[0]]],
                                 simulated_attack=[float(x) for x in truth["attack"][0]]),
        "abm_choice": dict(scen[int(judged[best_abm])], simulated_attack=[float(x) for x in truth["attack"][best_abm]]),
        "seeds_at_persons": big[0]["seeds"],
    }


def main(argv=None):
    """python -m pandemicthrust_gb300.surrogate build|evaluate|search ...

    build: samples scenarios, simulates each once on the batched simulator, trains
    an ensemble and saves it.  evaluate: scores a saved surrogate against fresh
    simulations (mean of replicates).  search: the surrogate-screened intervention
    search (``search``), by default 100,000 candidates at 50,000,000 persons with the
    top 1% judged by 32 simulator replicates each."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m pandemicthrust_gb300.surrogate")
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("build")
    b.add_argument("--out", required=True)
    b.add_argument("--persons", type=int, default=1_000_000)
    b.add_argument("--train", type=int, default=131072)
    b.add_argument("--members", type=int, default=4)
    b.add_argument("--epochs", type=int, default=200)
    b.add_argument("--batch", type=int, default=512)
    b.add_argument("--hidden", type=int, default=256)
    b.add_argument("--depth", type=int, default=4)
    b.add_argument("--average-last", type=int, default=None,
                   help="epochs whose weights are averaged (default: the last phase of the schedule; 0: best checkpoint)")
    b.add_argument("--seed", type=int, default=7, help="scenario sampling and network initialisation")
    b.add_argument("--seed-base", type=int, default=1_000_000, help="core seed of the first simulation")
    e = sub.add_parser("evaluate")
    e.add_argument("--model", required=True)
    e.add_argument("--test", type=int, default=1024)
    e.add_argument("--replicates", type=int, default=32)
    e.add_argument("--seed", type=int, default=99)
    e.add_argument("--seed-base", type=int, default=70_000_000)
    f = sub.add_parser("infer", help="time ensemble inference on random scenarios (no simulation)")
    f.add_argument("--model", default=SHIPPED_MODEL)
    f.add_argument("--rows", type=int, default=262144)
    f.add_argument("--repeats", type=int, default=3)
    f.add_argument("--mma-sync", action="store_true", help="the mma.sync kernel instead of tcgen05")
    f.add_argument("--chunk", type=int, default=262144, help="rows per inference launch")
    q = sub.add_parser("search")
    q.add_argument("--model", default=SHIPPED_MODEL)
    q.add_argument("--persons", type=int, default=50_000_000)
    q.add_argument("--candidates", type=int, default=100_000)
    q.add_argument("--budget-days", type=int, default=28, help="closure-days budget")
    q.add_argument("--top-fraction", type=float, default=0.01)
    q.add_argument("--judge-top", type=int, default=None, help="re-simulate only the best N of the top fraction")
    q.add_argument("--replicates", type=int, default=32)
    q.add_argument("--seed", type=int, default=2026)
    a = ap.parse_args(argv)
    if a.cmd == "build":
        scen = sample_scenarios(a.train, np.random.default_rng(a.seed))
        t0 = time.time()
        sim = simulate(scen, 1, a.persons, seed_base=a.seed_base)
        t_sim = time.time() - t0
        s = Surrogate(a.persons, hidden=a.hidden, depth=a.depth, seed=a.seed, members=a.members)
        t0 = time.time()
        val = s.fit(scen, targets(sim)[:, 0, :], epochs=a.epochs, batch=a.batch, average_last=a.average_last)
        t_fit = time.time() - t0
        avg = int(round(a.epochs * Surrogate.SCHEDULE[-1][0])) if a.average_last is None else a.average_last
        info = {"train_scenarios": a.train, "persons": a.persons, "epochs": a.epochs, "batch": a.batch,
                "averaged_epochs": avg,
                "scenario_seed": a.seed, "seed_base": a.seed_base, "val_loss": val, "simulate_s": t_sim,
                "fit_s": t_fit}
        s.save(a.out, **info)
        s.close()
        print(json.dumps(info))
    elif a.cmd == "infer":
        s = Surrogate.load(a.model, max_batch=a.chunk)
        for net in s.nets:
            net.set_tcgen05(not a.mma_sync)
        X = features(sample_scenarios(a.rows, np.random.default_rng(5)))
        times = []
        for _ in range(a.repeats):
            t0 = time.time()
            s.raw_features(X)
            times.append(time.time() - t0)
        # device time with inputs and outputs resident (CUDA events on the networks'
        # stream, the legacy default stream)
        device = []
        try:
            import torch
            xd = torch.from_numpy(X).cuda()
            yd = torch.empty((len(X), OUTPUTS), dtype=torch.float32, device="cuda")
            s.raw_device(xd.data_ptr(), len(X), yd.data_ptr())
            for _ in range(a.repeats):
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(torch.cuda.default_stream())
                s.raw_device(xd.data_ptr(), len(X), yd.data_ptr())
                ev1.record(torch.cuda.default_stream())
                torch.cuda.synchronize()
                device.append(ev0.elapsed_time(ev1) / 1000.0)
        except ImportError:
            pass
        s.close()
        print(json.dumps({"rows": a.rows, "members": len(s.nets), "kernel": "mma.sync" if a.mma_sync else "tcgen05",
                          "chunk": a.chunk,
                          "seconds": times, "scenarios_per_s": a.rows / min(times), "device_seconds": device,
                          "device_scenarios_per_s": a.rows / min(device) if device else None}))
    elif a.cmd == "search":
        s = Surrogate.load(a.model, max_batch=65536)
        r = search(s, a.persons, a.candidates, a.budget_days, a.top_fraction, a.judge_top, a.replicates, a.seed)
        s.close()
        print(json.dumps(r))
    else:
        s = Surrogate.load(a.model)
        scen = sample_scenarios(a.test, np.random.default_rng(a.seed))
        r = evaluate(s, scen, a.replicates, a.seed_base)
        s.close()
        print(json.dumps(dict(r, test_scenarios=a.test, replicates=a.replicates)))


if __name__ == "__main__":
    main()
