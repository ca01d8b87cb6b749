"""Host-side pieces of the surrogate: BF16 weight files and the target encoding."""
import json

import numpy as np
import pytest

from pandemicthrust_gb300 import surrogate as sg


def test_bf16_bits_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.standard_normal(10000).astype(np.float32) * 10.0 ** rng.integers(-6, 6, 10000),
                        np.array([1.0, 1.00390625, 1.01171875, -1.00390625, 0.0, -0.0], np.float32)])
    want = torch.tensor(a).bfloat16().float().numpy()
    got = sg._bf16_values(sg._bf16_bits(a))
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_targets_decode_round_trip():
    rng = np.random.default_rng(1)
    n, N = 5, 1_000_000
    daily = np.zeros((n, 1, sg.DAYS, 2))
    for i in range(n):
        t = np.arange(sg.DAYS)
        for s in range(2):
            daily[i, 0, :, s] = np.rint(rng.uniform(1e3, 1e5) * np.exp(-((t - rng.uniform(20, 90)) / 15.0) ** 2))
    sim = {"daily": daily, "attack": rng.uniform(0.01, 0.9, (n, 1, 2)), "rn": rng.uniform(0, 3, (n, 1, 8, 2)),
           "persons": np.full((n, 1), N)}
    d = sg.decode(sg.targets(sim)[:, 0, :], N)
    np.testing.assert_allclose(d["attack"], sim["attack"][:, 0], rtol=1e-5)
    np.testing.assert_allclose(d["peak"], daily[:, 0].max(axis=1), rtol=1e-5)
    np.testing.assert_array_equal(d["peak_day"], daily[:, 0].argmax(axis=1))
    np.testing.assert_allclose(d["rn"], sim["rn"][:, 0], rtol=1e-5)


def test_shipped_model_matches_this_module():
    """The committed surrogate was trained for these features, ranges and outputs."""
    import os
    path = sg.SHIPPED_MODEL
    if not os.path.exists(path):
        pytest.skip("no shipped surrogate")
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    assert meta["features"] == list(sg.FEATURES)
    assert meta["ranges"] == {k: list(v) for k, v in sg.RANGES.items()}
    assert meta["outputs"] == sg.OUTPUTS and meta["summary_weight"] == sg.SUMMARY_WEIGHT
    assert meta["activation"] == sg.ACTIVATION
    w = meta["widths"]
    n = sum(w[i] * w[i + 1] + w[i + 1] for i in range(len(w) - 1))
    assert z["params"].shape == (meta["members"], n) and z["params"].dtype == np.uint16
    nb = sum(w[1:])
    assert z["biases"].shape == (meta["members"], nb) and z["biases"].dtype == np.float32
    assert sg._bias_mask(w).sum() == nb


class _FakeNet:
    """Stands in for MLP: its 'weights' count the epochs trained so far."""

    def __init__(self):
        self.calls, self.p, self.widths = [], np.zeros(3, np.float32), [11, 4, sg.OUTPUTS]

    def set_data(self, X, Y):
        pass

    def get_params(self):
        return self.p.copy()

    def set_params(self, p):
        self.p = np.array(p, np.float32)

    def train(self, n, batch, lr, seed):
        self.calls.append((n, lr))
        self.p = self.p + n

    def predict(self, X):
        return np.zeros((len(X), sg.OUTPUTS), np.float32)


@pytest.mark.parametrize("epochs,average_last", [(400, None), (200, 40), (50, 0), (7, None)])
def test_fit_follows_the_schedule_and_averages_the_last_epochs(epochs, average_last):
    s = sg.Surrogate.__new__(sg.Surrogate)
    s.persons, s.nets = 1, [_FakeNet(), _FakeNet()]
    scen = sg.sample_scenarios(40, np.random.default_rng(0))
    s.fit(scen, np.zeros((40, sg.OUTPUTS), np.float32), epochs=epochs, checks=16, average_last=average_last)
    rates = [r for f, r in sg.Surrogate.SCHEDULE for _ in range(max(1, int(round(epochs * f))))]
    for net in s.nets:
        # every epoch trained once, at its scheduled rate
        assert [lr for n, lr in net.calls for _ in range(n)] == rates
        avg = int(round(epochs * sg.Surrogate.SCHEDULE[-1][0])) if average_last is None else average_last
        if avg:
            # the weights are the mean over the last `avg` epochs
            want = np.mean(np.arange(len(rates) - avg + 1, len(rates) + 1))
            np.testing.assert_allclose(net.p, want, rtol=1e-6)
        else:
            assert net.p[0] == net.calls[0][0]   # equal validation losses keep the first checkpoint


def test_load_refuses_a_model_for_other_targets(tmp_path):
    """Checked before any device memory is taken."""
    meta = dict(sg._encoding(), persons=1000, widths=[len(sg.FEATURES) + sg.N_DERIVED, 8, sg.OUTPUTS], members=1,
                info={})
    for key, value in (("summary_weight", sg.SUMMARY_WEIGHT + 1.0), ("days", sg.DAYS + 1),
                       ("ranges", dict(meta["ranges"], vaccination=[0.0, 0.9])),
                       ("activation", "gelu_erf"), ("activation", None)):   # None: a file from before the key
        bad = dict(meta, **{key: value})
        path = tmp_path / ("bad_%s_%s.npz" % (key, value is None))
        np.savez(path, params=np.zeros((1, 10), np.uint16), biases=np.zeros((1, 10), np.float32),
                 meta=np.array(json.dumps(bad)))
        with pytest.raises(ValueError, match=key):
            sg.Surrogate.load(path)
    wrong = dict(meta, widths=[3, 8, sg.OUTPUTS])
    path = tmp_path / "bad_widths.npz"
    np.savez(path, params=np.zeros((1, 10), np.uint16), biases=np.zeros((1, 10), np.float32),
             meta=np.array(json.dumps(wrong)))
    with pytest.raises(ValueError, match="widths"):
        sg.Surrogate.load(path)


def test_nearest_neighbour_matches_brute_force():
    rng = np.random.default_rng(11)
    T = rng.random((40000, 11)).astype(np.float32)   # enough rows that the queries go in several chunks
    Y = np.arange(len(T))[:, None] * np.ones((1, 3))
    X = rng.random((700, 11)).astype(np.float32)
    want = np.concatenate([((X[i:i + 20, None, :].astype(np.float64) - T[None, :, :]) ** 2).sum(axis=2).argmin(axis=1)
                           for i in range(0, len(X), 20)])
    got = sg.nearest_neighbour(T, Y, X)[:, 0].astype(int)
    # ties aside (none in random data), the same training row
    np.testing.assert_array_equal(got, want)


def test_search_scenarios_respect_the_budget_and_fixed_strains():
    scen = sg.search_scenarios(2000, np.random.default_rng(3), budget_days=21)
    assert all(s["closure_days"] <= 21 and s["r_pandemic"] == 1.5 and s["r_seasonal"] == 1.2 for s in scen)
    assert max(s["closure_days"] for s in scen) == 21 and min(s["closure_days"] for s in scen) == 0
    assert sg.in_range(scen).all()   # every candidate is inside the network's training ranges


def test_transfer_to_a_larger_population_keeps_fractions():
    pred = {"daily": np.ones((2, sg.DAYS, 2)) * 10.0, "peak": np.array([[5.0, 6.0], [7.0, 8.0]]),
            "attack": np.array([[0.1, 0.2], [0.3, 0.4]]), "peak_day": np.array([[30.0, 40.0], [50.0, 60.0]])}
    out = sg.transfer(pred, 50_000_000, 1_000_000)
    np.testing.assert_array_equal(out["peak"], pred["peak"] * 50)
    np.testing.assert_array_equal(out["daily"], pred["daily"] * 50)
    np.testing.assert_array_equal(out["attack"], pred["attack"])
    np.testing.assert_array_equal(out["peak_day"], pred["peak_day"])
    s = sg.scaled({"seeds": 20, "closure_days": 3}, 50_000_000, 1_000_000)
    assert s["seeds"] == 1000 and s["closure_days"] == 3
