"""The surrogate's network and pipeline: gradients of the hand-written BF16/FP32 kernels
against an FP64 reference on the CPU, training, and the trained surrogate against the
method without it (nearest neighbour in the training set), judged by the mean of 32
simulator replicates."""
import numpy as np
import pytest

from pandemicthrust_gb300 import surrogate as sg

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


C0, C1 = np.sqrt(2 / np.pi), np.sqrt(2 / np.pi) * 0.044715


def gelu(z):
    """GELU in its tanh form, as the kernels (which use the hardware tanh)."""
    return 0.5 * z * (1 + np.tanh(z * (C0 + C1 * z * z)))


def gelu_grad(z):
    t = np.tanh(z * (C0 + C1 * z * z))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * (C0 + 3 * C1 * z * z)


def reference_gradients(params, widths, X, Y):
    """FP64 forward / backward of the same network; weights and inputs rounded to
    BF16 as the kernels read them, nothing rounded in between."""
    Ws, bs, off = [], [], 0
    for l in range(len(widths) - 1):
        n = widths[l + 1] * widths[l]
        Ws.append(bf16(params[off:off + n]).reshape(widths[l + 1], widths[l]))
        off += n
        bs.append(params[off:off + widths[l + 1]].astype(np.float64))
        off += widths[l + 1]
    H, Hs, Zs = bf16(X), [], []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Hs.append(H)
        Z = H @ W.T + b
        Zs.append(Z)
        H = gelu(Z) if l + 1 < len(Ws) else Z
    D = H - Y
    loss = np.mean(D * D)
    dZ = 2 * D / D.size
    grads = [None] * (2 * len(Ws))
    for l in reversed(range(len(Ws))):
        grads[2 * l] = (dZ.T @ Hs[l]).ravel()
        grads[2 * l + 1] = dZ.sum(axis=0)
        if l > 0:
            dZ = (dZ @ Ws[l]) * gelu_grad(Zs[l - 1])
    return np.concatenate(grads), loss


@pytest.mark.parametrize("widths,batch", [([7, 32, 48, 24], 40), ([7, 256, 256, 222], 128)])
def test_mlp_gradients_match_fp64_reference(native_lib, widths, batch):
    rng = np.random.default_rng(7)
    net = sg.MLP(widths, max_batch=256, seed=3)
    params = net.get_params()
    params[:] += rng.normal(0, 0.02, params.size).astype(np.float32)  # non-zero biases too
    net.set_params(params)
    X = rng.uniform(0, 1, (batch, widths[0])).astype(np.float32)
    Y = rng.normal(0, 1, (batch, widths[-1])).astype(np.float32)
    g, loss = net.gradients(X, Y)
    ref, ref_loss = reference_gradients(params, widths, X, Y)
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    off = 0
    for l in range(len(widths) - 1):
        for n in (widths[l + 1] * widths[l], widths[l + 1]):
            a, b = g[off:off + n].astype(np.float64), ref[off:off + n]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert rel < 3e-2, (l, n, rel)  # BF16 activations and gradients between layers
            off += n
    net.close()


def test_mlp_learns_a_smooth_map(native_lib):
    rng = np.random.default_rng(1)
    X = rng.uniform(0, 1, (2048, 7)).astype(np.float32)
    Y = np.stack([np.sin(3 * X[:, 0]) * X[:, 1], np.cos(2 * X[:, 2] + X[:, 3]), X[:, 4] * X[:, 5] - X[:, 6]],
                 axis=1).astype(np.float32)
    net = sg.MLP([7, 128, 128, 3], max_batch=512, seed=5)
    net.set_data(X, Y)
    first = net.train(1, batch=256, lr=1e-3)
    last = net.train(300, batch=256, lr=1e-3)
    assert last < first / 20
    pred = net.predict(X[:100])
    assert np.sqrt(np.mean((pred - Y[:100]) ** 2)) < 0.1
    net.close()


def test_surrogate_beats_nearest_neighbour_and_falls_back(native_lib):
    persons = 20_000
    rng = np.random.default_rng(2024)
    train = sg.sample_scenarios(384, rng)
    test = sg.sample_scenarios(12, rng)
    tr = sg.simulate(train, 1, persons, seed_base=10_000)
    te = sg.simulate(test, 32, persons, seed_base=50_000)
    Ytr = sg.targets(tr)[:, 0, :]
    s = sg.Surrogate(persons, hidden=256, depth=4, seed=1)
    s.fit(train, Ytr, epochs=600, batch=128, checks=6)
    pred, fb = s.predict(test)
    assert not fb.any()
    truth = sg.truth_summary(te)
    mine = sg.predicted_summary(pred)
    nn = sg.decode(sg.nearest_neighbour(sg.features(train), Ytr, sg.features(test)), persons)
    base = sg.predicted_summary(nn)
    pk, at = sg.relative_errors(mine, truth)
    pk0, at0 = sg.relative_errors(base, truth)
    assert len(pk) >= 6
    assert np.median(at) < np.median(at0) and np.median(pk) < np.median(pk0), (np.median(pk), np.median(at),
                                                                             np.median(pk0), np.median(at0))
    # an out-of-range scenario is simulated instead
    odd = dict(test[0], r_pandemic=2.6)
    p2, fb2 = s.predict([odd, test[1]], fallback_replicates=2, seed_base=77)
    assert list(fb2) == [True, False]
    direct = sg.simulate([odd], 2, persons, seed_base=77)
    assert np.allclose(p2["attack"][0], direct["attack"].mean(axis=1)[0])
    s.close()


def test_saved_surrogate_predicts_the_same(native_lib, tmp_path):
    rng = np.random.default_rng(3)
    scen = sg.sample_scenarios(64, rng)
    s = sg.Surrogate(20_000, hidden=32, depth=2, seed=5, members=2)
    Y = rng.random((64, sg.OUTPUTS)).astype(np.float32)
    s.fit(scen, Y, epochs=4, batch=16, checks=2)
    path = tmp_path / "model.npz"
    s.save(path, note="test")
    before = s.raw(scen)
    s.close()
    t = sg.Surrogate.load(path)
    assert t.persons == 20_000 and len(t.nets) == 2 and t.info == {"note": "test"}
    # the saved weights are the BF16 values inference uses: predictions are identical
    np.testing.assert_array_equal(t.raw(scen), before)
    t.close()


def test_shipped_surrogate_on_fresh_scenarios(native_lib):
    """The shipped ensemble against simulations it never saw (new draws, new seeds).
    A small sample with a loose bound; the full evaluation (1,024 scenarios x 32
    replicates) gives 3.9% / 3.4% median peak / attack error."""
    import os
    if not os.path.exists(sg.SHIPPED_MODEL):
        pytest.skip("no shipped surrogate")
    s = sg.Surrogate.load(sg.SHIPPED_MODEL)
    assert s.persons == 1_000_000 and len(s.nets) >= 1
    scen = sg.sample_scenarios(48, np.random.default_rng(4242))
    r = sg.evaluate(s, scen, 8, seed_base=90_000_000)
    s.close()
    assert r["pairs"] >= 10
    assert r["peak_median"] < 0.08 and r["attack_median"] < 0.08, r
    assert r["peak_day_abs_median"] <= 3, r


def test_ensemble_mean_on_device_matches_the_members(native_lib):
    rng = np.random.default_rng(8)
    s = sg.Surrogate(20_000, hidden=32, depth=2, seed=3, members=3, max_batch=64)
    X = sg.features(sg.sample_scenarios(200, rng))   # more rows than max_batch: several chunks
    want = np.mean([net.predict(X) for net in s.nets], axis=0)
    np.testing.assert_allclose(s.raw_features(X), want, rtol=1e-5, atol=1e-6)
    assert s.raw_features(X[:0]).shape == (0, sg.OUTPUTS)
    s.close()


def test_intervention_search_screens_then_judges_with_the_simulator(native_lib):
    """The surrogate-screened search end to end at a small size: every candidate is
    scored, the top fraction is kept, its best are re-simulated with replicates, and
    the simulator's pick is among the judged candidates and within the budget."""
    import os
    if not os.path.exists(sg.SHIPPED_MODEL):
        pytest.skip("no shipped surrogate")
    s = sg.Surrogate.load(sg.SHIPPED_MODEL, max_batch=4096)
    r = sg.search(s, persons=300_000, candidates=3000, budget_days=14, top_fraction=0.01, judge_top=2,
                  replicates=3, transfer_sample=2, seed_base=400_000_000)
    s.close()
    assert r["candidates"] == 3000 and r["top"] == 30 and r["judged"] == 2 and r["transfer_sample"] == 2
    assert len(r["transfer_scenarios"]) == 2 and all(sg.in_range(r["transfer_scenarios"]))
    assert r["abm_runs"] == 12 and r["abm_person_days_per_s"] > 0 and r["surrogate_scenarios_per_s"] > 0
    assert r["abm_choice"]["closure_days"] <= 14 and r["abm_choice"]["vaccination"] == 0.2
    assert r["seeds_at_persons"] == 6   # 20 per million, scaled to 300,000 persons
    assert r["error_judged"]["pairs"] == 4
    # the best candidates by the surrogate hold the epidemic down in the simulator too
    assert sum(r["abm_choice"]["simulated_attack"]) < 0.2
