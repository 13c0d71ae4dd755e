"""ccp-analyze's outputs from the GPU observables against the analysis oracle
(oracle/analysis_oracle.py, whose statistics are pinned character for
character against the reference's own sostat.cu).

A 2048-bead ccp system runs two simulations of 24 frames each. Checked:
  * the per-frame series (centre-of-mass distance, gyration radius squared,
    nematic order, nucleus fraction, 3 x 64 radial densities) against the
    oracle's FP64 observables of the same positions: relative 1e-5 (the GPU
    sums FP32 shell volumes), the nucleus fraction exactly;
  * analysis-XXX.dat: the statistics lines equal, character for character,
    what the oracle writes for the same series; the contact-probability block
    equals the oracle's (identical contact counts); the spatial-distance
    block within 1e-5 relative (FP32 partial distance sums on the GPU);
  * analysis-fin.dat over both simulations, within the same tolerances;
  * contact-map.bin: the mean of the per-simulation map averages, from the
    oracle's own contact counts, within 1e-12 relative.
"""
import math

import numpy as np
import pytest

from helpers import ccp_params


def _compare_text(got, want, rtol):
    gl, wl = got.splitlines(), want.splitlines()
    assert len(gl) == len(wl)
    for g, w in zip(gl, wl):
        gt, wt = g.split(), w.split()
        assert len(gt) == len(wt), (g, w)
        finite = [abs(float(x)) for x in wt if "." in x and math.isfinite(float(x))]
        scale = max(finite) if finite else 0.0
        for a, b in zip(gt, wt):
            try:
                fa, fb = float(a), float(b)
            except ValueError:
                assert a == b, (g, w)
                continue
            if "." not in b:  # integers: separation index, block count, thermalisation index
                assert a == b, (g, w)
            elif math.isnan(fa) or math.isnan(fb):
                # a variance that cancels to rounding size prints nan on one side
                # (square root of a tiny negative) and ~0 on the other
                other = fb if math.isnan(fa) else fa
                assert math.isnan(other) or abs(other) <= rtol * scale + 2e-6, (g, w)
            else:
                assert abs(fa - fb) <= rtol * abs(fb) + 2e-6, (g, w)


@pytest.mark.gpu
def test_analysis_outputs_match_oracle(engine_lib, orc):
    from oracle import analysis_oracle as ao
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(2048)
    sim = ChrSim(txt, seed=3)
    sim.generate_initial_condition()
    si, info = sim.system_info(0), sim.info()
    L = si.n_beads
    types = (sim.types() & 1).astype(int)
    R_n = float(si.nucleus_radius)
    nod = math.sqrt(R_n * R_n - float(si.opening_radius) ** 2)
    cut = info.contact_cutoff
    nb, px, ncop = si.contact_bins, si.map_len // si.contact_bins, si.n_copies
    diag = np.zeros(nb * (nb + 1) // 2)
    b = np.arange(nb)
    diag[b * (b + 1) // 2 + b] = px * ncop

    stats, sd_sims, cp_sims, cm_sims = [], [], [], []
    for run in range(2):
        xs = []
        for f in range(24):
            if f:
                sim.run_steps(100)
            sim.analysis_frame()
            xs.append(sim.positions().copy())
        ser = sim.analysis_series(0)
        assert ser.shape == (4 + 3 * 64, 24)
        # per-frame observables
        ref = [ao.frame_observables(x, types, R_n, nod) for x in xs]
        for k in range(4):
            r = np.array([o[k] for o in ref], np.float64)
            if k == 3:
                assert np.array_equal(ser[k], r.astype(np.float32))
            else:
                assert np.allclose(ser[k], r, rtol=1e-5, atol=1e-6), k
        rcd = np.array([o[4] for o in ref]).reshape(24, -1).T
        assert np.allclose(ser[4:], rcd, rtol=1e-5, atol=1e-5 * np.abs(rcd).max())
        # frame-averaged basic observables from the oracle's own counts and distances
        mcnt = np.zeros(nb * (nb + 1) // 2)
        pcnt = np.zeros(L // 2 + 1)
        dsum = np.zeros(L // 2 + 1)
        for x in xs:
            m, ps, _ = orc.contacts(x, cut, nb, si.map_len, si.copy_len, ncop, [0])
            mcnt += m
            pcnt += ps
            dsum += orc.sdist(x)
        s = np.arange(1, L // 2 + 1)
        cp = 1000.0 * pcnt[1:] / (24.0 * (L - s))
        sd = dsum[1:] / (24.0 * (L - s))
        cm = 1000.0 * (mcnt / 24.0 + diag) / (ncop * px * px)
        sim.analysis_end_simulation()
        got = sim.analysis_txt(0).decode()
        series = [(ser[0, f], ser[1, f], ser[2, f], ser[3, f], ser[4:, f].reshape(3, 64)) for f in range(24)]
        want, st = ao.analysis_txt(series, R_n, [list(sd)], [list(cp)])
        # statistics and contact probability: as written by the oracle; distances within 1e-5
        gl, wl = got.splitlines(), want.splitlines()
        heads = [i for i, l in enumerate(wl) if l == "     s         avg"]
        assert len(heads) == 12  # six sd blocks, six cp blocks
        assert gl[:heads[0]] == wl[:heads[0]]
        _compare_text(got, want, 1e-5)
        assert gl[heads[6]:] == wl[heads[6]:]
        stats.append(st)
        sd_sims.append([list(sd)])
        cp_sims.append([list(cp)])
        cm_sims.append(cm)
        assert sim.analysis_series(0).shape[1] == 0  # series cleared

    fin = sim.analysis_fin_txt().decode()
    _compare_text(fin, ao.analysis_fin_txt(stats, R_n, sd_sims, cp_sims), 1e-5)
    cmb = np.frombuffer(sim.contact_map_bin(), np.float64)
    ref_cm = (cm_sims[0] + cm_sims[1]) / 2.0
    assert cmb.shape == ref_cm.shape
    assert np.allclose(cmb, ref_cm, rtol=1e-12, atol=0)
