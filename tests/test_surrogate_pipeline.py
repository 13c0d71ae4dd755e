"""What the trained surrogate gains over the methods without it (GPU).

Sequences of 1024 beads are simulated by the batched engine into 256 x 256
contact-probability maps (one replica each, 2 x 10^4 Heun steps after a
burn-in); the network is trained on most of them with its own tensor-core
kernels. One simulated map remembers its start (its P(s) is ~15 % off its
sequence's expectation), so held-out sequences are each simulated by 32
fresh replicas and their mean map is the truth. Against it the trained
network is closer, in P(s) error and in map error, than
  * the training set's mean map (what is known without reading the sequence),
  * a power law P(s) fitted to that mean (a P(s)-only model),
  * one more simulation of the same sequence (what simulating instead gives),
and much closer than the untrained network; predicting a map costs a small
fraction of simulating it. The P(s) error is surrogate.ps_error: the mean
over separation octaves [1,2) .. [64,128) bins of |P_pred - P_ref| / P_ref;
the map error is surrogate.map_log_error.

The screening test runs surrogate.screen (c4's protocol) on a small network:
every sequence that is re-simulated is either in the random sample or
predicted outside the training envelope, and each of those is.
"""
import time

import numpy as np
import pytest


@pytest.mark.gpu
def test_trained_surrogate_beats_methods_without_it(engine_lib):
    from tfm_gb300 import surrogate as S

    n, L, M = 2048, 1024, 256
    steps, burn, every = 20000, 5000, 200
    types, lad, _ = S.make_sequences(n, L, 21)
    t0 = time.perf_counter()
    maps, frames = S.simulate_maps(types, lad, M, steps, burn, every, seed=300)
    sim_s_per_map = (time.perf_counter() - t0) / n
    assert frames == steps // every
    nh = 64
    ntr = n - nh
    k = 32
    held = slice(ntr, ntr + k)
    truth, _ = S.simulate_maps(types[held], lad[held], M, steps, burn, every, seed=9000, reps=32)

    epochs = 20
    total = epochs * (ntr // 32)
    with S.Surrogate("lr 1e-3\nlr_min 1e-4\nlr_steps %d\n" % total, seed=4) as net:
        net.set_dataset(types, lad, maps)
        rows = np.arange(ntr, ntr + k, dtype=np.int32)
        untrained = S.ps_error(net.predict_rows(rows), truth).mean()
        S.train(net, ntr, epochs, seed=8)
        pred = net.predict_rows(rows)
        net.predict_rows(rows)  # warm
        t1 = time.perf_counter()
        net.predict_rows(np.arange(0, 256, dtype=np.int32))
        pred_s_per_map = (time.perf_counter() - t1) / 256
        assert net.error_flags() == 0

    assert np.all(np.isfinite(pred)) and pred.min() >= 0.0 and pred.max() <= 1.0
    rep = lambda m: np.repeat(m, k, 0)
    cands = {"surrogate": pred, "training mean map": rep(maps[:ntr].mean(axis=0, keepdims=True)),
             "power-law P(s)": rep(S.powerlaw_map(maps[:ntr])), "one simulation": maps[held]}
    ps = {c: S.ps_error(m, truth).mean() for c, m in cands.items()}
    me = {c: S.map_log_error(m, truth).mean() for c, m in cands.items()}
    print("\nP(s) error / map error against the 32-replica truth:")
    for c in cands:
        print("  %-18s %.4f  %.4f" % (c, ps[c], me[c]))
    for c in ("training mean map", "power-law P(s)", "one simulation"):
        assert ps["surrogate"] < ps[c], (c, ps)
        assert me["surrogate"] < me[c], (c, me)
    assert ps["surrogate"] < 0.5 * untrained, (ps["surrogate"], untrained)
    assert pred_s_per_map * 20 < sim_s_per_map, (pred_s_per_map, sim_s_per_map)


@pytest.mark.gpu
def test_screen_resimulates_random_and_out_of_envelope(engine_lib):
    from tfm_gb300 import surrogate as S

    L, M = 256, 128
    cfg = "seq_len %d\nbins %d\nbatch 8\nenc_layers 2\nhead_layers 2\ndilations 1,2\n" % (L, M)
    sim = lambda t, l: S.simulate_maps(t, l, M, 2000, 500, 100, seed=77)[0]
    types, lad, _ = S.make_sequences(64, L, 5)
    maps = sim(types, lad)
    env = S.envelope(maps)
    st, sl, _ = S.make_sequences(600, L, 6)
    calls = []

    def counting_sim(t, l):
        calls.append(len(t))
        return sim(t, l)

    with S.Surrogate(cfg, seed=2) as net:
        net.set_dataset(types, lad, maps)
        S.train(net, 64, 3, seed=1)
        rep, fb = S.screen(net, st, sl, env, 0.01, seed=3, sim=counting_sim, chunk=256)
        maps_pred = net.predict(st, sl)
        pb = S.ps_log_bins(maps_pred)
        # the device-side P(s) equals the host reduction of the same maps
        ps_dev = net.predict_ps(st, sl)
        assert np.allclose(ps_dev, S.ps_curve(maps_pred), rtol=1e-5, atol=1e-9)
        assert net.error_flags() == 0
    lo, hi = env
    out = np.any((pb < lo) | (pb > hi), axis=1)
    assert rep["sequences"] == 600 and rep["fallback_random"] == 6
    assert rep["fallback_out_of_envelope"] == int(out.sum())
    assert calls == [len(fb)] and rep["simulated"] == len(fb)
    assert np.array_equal(fb, np.unique(fb))
    # every out-of-envelope sequence is re-simulated; the rest of the
    # re-simulated ones are the random sample
    assert set(np.nonzero(out)[0]) <= set(fb.tolist())
    assert len(set(fb.tolist()) - set(np.nonzero(out)[0])) <= 6
    err = rep["ps_error_random_sample"]
    assert np.isfinite([err["mean"], err["median"], err["p90"]]).all()
    # the per-bin map error of the random sample, overall and by separation octave
    me = rep["map_log10_error_random_sample"]
    assert np.isfinite([me["mean"], me["median"], me["p90"]]).all() and me["mean"] >= 0
    assert len(me["by_separation_octave"]) == int(np.log2(M // 2))
