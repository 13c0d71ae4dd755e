"""Trajectory output overlapped with the steps (chrsim::run_simulation,
chrsim.cu:558-593, writes each frame after a blocking copy; here frame k is
copied on a separate stream and written while frame k+1 computes).

  * every frame delivered to the callback is the state at the end of its
    frame: the same system stepped frame by frame with run_steps and read
    back with positions() gives the same frames (to the trajectories' own
    FP32 drift; a frame from the wrong step would be ~0.3 sigma away);
  * a writer that takes 80 % of a frame's compute time is hidden: the run
    takes about one frame longer than without it, not 1.8 times as long.
"""
import time

import numpy as np
import pytest

from helpers import ccp_params


@pytest.mark.gpu
def test_frames_are_frame_end_states(engine_lib):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(2048)
    extra = "frames_per_file 6\nsteps_per_frame 500\n"
    a = ChrSim(txt + extra, seed=2)
    a.generate_initial_condition()
    b = ChrSim(txt + extra, seed=2)
    b.set_types(a.types())
    b.set_lbs(a.lbs())
    b.set_positions(a.positions())
    got = []
    a.run_simulation(None, on_frame=lambda i_f, t, x: got.append((i_f, t, x)))
    assert [g[0] for g in got] == list(range(1, 7))
    for k in range(6):
        b.run_steps(500)
        d = np.abs(got[k][2] - b.positions()).max()
        assert d < 1e-2, (k, d)
    assert np.array_equal(got[-1][2], a.positions())
    assert np.isclose(got[-1][1], a.info().time)


@pytest.mark.gpu
def test_slow_writer_is_hidden(engine_lib):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(2048)
    sim = ChrSim(txt + "frames_per_file 8\nsteps_per_frame 2000\n", seed=3)
    sim.generate_initial_condition()
    sim.run_simulation(None)  # graphs built
    plain = []
    for _ in range(2):
        t0 = time.perf_counter()
        sim.run_simulation(None)
        plain.append(time.perf_counter() - t0)
    t_plain = min(plain)
    tf = t_plain / 8
    t0 = time.perf_counter()
    sim.run_simulation(None, on_frame=lambda i_f, t, x: time.sleep(0.8 * tf))
    t_slow = time.perf_counter() - t0
    print("8 frames: %.1f ms plain, %.1f ms with a writer of %.1f ms per frame (serial: %.1f ms)"
          % (1e3 * t_plain, 1e3 * t_slow, 0.8e3 * tf, 1e3 * (t_plain + 8 * 0.8 * tf)))
    assert t_slow < t_plain + 3 * 0.8 * tf
