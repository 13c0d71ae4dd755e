"""What the trained surrogate gains over simulating (GPU).

Sequences of 1024 beads are simulated by the batched engine into 256 x 256
contact-probability maps; the network is trained on most of them with its own
tensor-core kernels. On held-out sequences, each also simulated by three
fresh replicas, the reference is the replicas' mean map. Against it:
  * the trained network's P(s) (per separation octave) is closer than that of
    one more simulation of the same sequence, the map a user gets by
    simulating instead, and much closer than the untrained network's;
  * predicting a map costs a small fraction of simulating it.
The error metric is surrogate.ps_error: the mean over separation octaves
[1,2) .. [64,128) of |P_pred - P_ref| / P_ref.
"""
import time

import numpy as np
import pytest


@pytest.mark.gpu
def test_trained_surrogate_beats_one_more_simulation(engine_lib):
    from tfm_gb300 import surrogate as S

    n, L, M = 384, 1024, 256
    steps, burn, every = 8000, 2000, 100
    types, lad, _ = S.make_sequences(n, L, 21)
    t0 = time.perf_counter()
    maps, frames = S.simulate_maps(types, lad, M, steps, burn, every, seed=300)
    sim_s_per_map = (time.perf_counter() - t0) / n
    assert frames == steps // every
    nh = 64
    ntr = n - nh
    k = 32
    held = slice(ntr, ntr + k)
    reps = [S.simulate_maps(types[held], lad[held], M, steps, burn, every, seed=900 + 13 * r)[0]
            for r in range(3)]
    ref = np.mean(reps, axis=0)

    epochs = 40
    total = epochs * (ntr // 32)
    with S.Surrogate("lr 1e-3\nlr_min 1e-4\nlr_steps %d\n" % total, seed=4) as net:
        net.set_dataset(types, lad, maps)
        rows = np.arange(ntr, ntr + k, dtype=np.int32)
        untrained = S.ps_error(net.predict_rows(rows), ref).mean()
        S.train(net, ntr, epochs, seed=8)
        pred = net.predict_rows(rows)
        net.predict_rows(rows)  # warm
        t1 = time.perf_counter()
        net.predict_rows(np.arange(0, 256, dtype=np.int32))
        pred_s_per_map = (time.perf_counter() - t1) / 256
        assert net.error_flags() == 0

    trained = S.ps_error(pred, ref).mean()
    one_more = S.ps_error(maps[held], ref).mean()
    assert np.all(np.isfinite(pred)) and pred.min() >= 0.0 and pred.max() <= 1.0
    assert trained < one_more, (trained, one_more)
    assert trained < 0.5 * untrained, (trained, untrained)
    assert pred_s_per_map * 20 < sim_s_per_map, (pred_s_per_map, sim_s_per_map)
