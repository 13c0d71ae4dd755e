"""Statistical agreement with ccp's own dynamics.

ccp seeds its noise with the time, so its trajectories cannot be reproduced
bit for bit; what must agree is what they sample. M replicas of ccp's model
(2048 beads, chromatin volume fraction 0.2, lamina area fraction 0.25, ccp's
force field) start from the engine's initial conditions. Each start is run
twice for the same number of Heun steps: by the reference's own kernels
(oracle/ccp_gpu_ref.py: begin_iter, the cell list, exec_RK_1/2 compiled from
the reference's sources, cuRAND noise) and by the engine (batched, Philox
noise). Per frame the same code measures both: the gyration radius squared
and the radial chromatin density (chrana.cu:390-480, as the analysis oracle
restates it, in 8 groups of 8 of ccp's 64 equal-volume shells) and the
contact probability by separation octave (the contact rule of calc_sd_cp,
chrana.cu:13-45, at aco = 2).

Error bars are ccp's own (sostat.cu:136-204, restated by the pinned analysis
oracle): per replica the marginal-standard-error thermalisation and the
blocking standard error, then the inverse-variance combination over
replicas. Each observable must satisfy |mean_ref - mean_engine| <=
3 sqrt(sem_ref^2 + sem_engine^2). Because a replica's two runs share their
start, the difference per replica is also tested directly (paired: the
start's contribution cancels there). Its bound is 5 standard errors over the
16 replicas: with 15 degrees of freedom and 18 observables a bound of 4 would
fail by chance in ~2 % of runs, one of 5 in ~0.3 %.
"""
import math

import numpy as np
import pytest

from helpers import ccp_params

pytestmark = pytest.mark.gpu

M = 16            # replicas
N = 2048          # beads
FRAMES = 100      # frames per run
SPF = 100         # Heun steps per frame (10^4 steps = 4.9 time units)
OCTAVES = range(1, 10)  # separations [2^k, 2^(k+1)), k = 1..9
ACO = 2.0


def _octave_ids(n, device):
    import torch

    i = torch.arange(n, device=device)
    s = (i[None, :] - i[:, None]).abs()
    ids = torch.full_like(s, -1)
    for k in OCTAVES:
        ids[(s >= 2 ** k) & (s < 2 ** (k + 1))] = k - OCTAVES[0]
    ids[torch.tril(torch.ones_like(s, dtype=torch.bool))] = -1  # each pair once
    sel = ids >= 0
    flat = ids[sel]
    return sel, flat, torch.bincount(flat, minlength=len(OCTAVES)).double()


def _contact_octaves(r, sel, flat, pairs):
    import torch

    d = torch.cdist(r.double(), r.double())
    c = (d < ACO)[sel]
    return (torch.bincount(flat[c], minlength=len(OCTAVES)).double() / pairs).cpu().numpy()


def _frame(r_dev, types, R_n, oct_args):
    from oracle import analysis_oracle as ao

    x = r_dev.cpu().numpy()
    _, rg2, _, _, rcd = ao.frame_observables(x, types, R_n, R_n)
    rad = rcd[2].astype(np.float64).reshape(8, 8).mean(axis=1)
    return np.concatenate([[rg2], _contact_octaves(r_dev, *oct_args), rad])


NAMES = (["Rg^2"] + ["P(s), s in [%d, %d)" % (2 ** k, 2 ** (k + 1)) for k in OCTAVES]
         + ["radial density, shells %d-%d" % (8 * g + 1, 8 * g + 8) for g in range(8)])


def test_engine_samples_what_ccp_samples(engine_lib):
    import torch

    from oracle import analysis_oracle as ao
    from oracle import ccp_gpu_ref as ref
    from tfm_gb300.ccpgpu import Batch

    try:
        mod = ref.Module()
    except FileNotFoundError as e:
        pytest.skip(str(e))
    dev = torch.device("cuda")
    txt, R_n, n_l = ccp_params(N)
    eng = Batch(txt, [N] * M, seeds=np.arange(M, dtype=np.uint64) + 101)
    eng.generate_initial_condition()
    x0, types, lbs = eng.positions(), eng.types(), eng.lbs()
    infos = [eng.system_info(s) for s in range(M)]
    oct_args = _octave_ids(N, dev)

    # the reference: one system per replica on its own stream, a CUDA graph of
    # SPF steps each (ccp's launches captured once, replayed per frame)
    streams = [torch.cuda.Stream() for _ in range(M)]
    systems, graphs = [], []
    for s in range(M):
        si = infos[s]
        sl = slice(si.bead_offset, si.bead_offset + si.n_beads)
        ls = lbs[si.lbs_offset:si.lbs_offset + si.n_lbs]
        sysr = ref.System(mod, x0[sl], types[sl], ls, si.nucleus_radius, seed=7001 + s,
                          stream=streams[s])
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=streams[s]):
            for _ in range(SPF):
                sysr.step()
        systems.append(sysr)
        graphs.append(g)
    torch.cuda.synchronize()
    # capture does not run the steps: every system is still at its start
    series_ref = [[] for _ in range(M)]
    series_eng = [[] for _ in range(M)]
    for f in range(FRAMES):
        for s in range(M):
            with torch.cuda.stream(streams[s]):
                graphs[s].replay()
        eng.run_steps(SPF)
        torch.cuda.synchronize()
        xe = torch.tensor(eng.positions(), device=dev)
        for s in range(M):
            sysr, si = systems[s], infos[s]
            # a bead outside ccp's grid would be an out-of-range cell index in
            # the reference's own cell list: stop before the next replay
            rmax = sysr.max_radius()
            assert math.isfinite(rmax) and rmax < sysr.grid_half - 1.0, (s, f, rmax)
            sl = slice(si.bead_offset, si.bead_offset + si.n_beads)
            series_ref[s].append(_frame(sysr.r, types[sl], si.nucleus_radius, oct_args))
            series_eng[s].append(_frame(xe[sl], types[sl], si.nucleus_radius, oct_args))
    flags, _ = eng.error_flags()
    assert not flags[:4].any(), flags
    eng.close()
    mod.close()

    sr = np.asarray(series_ref)  # (M, FRAMES, observables)
    se = np.asarray(series_eng)
    worst = 0.0
    print("\nobservable: ccp mean +- sem | engine mean +- sem | z | paired z")
    for k, name in enumerate(NAMES):
        st_r = [ao.stats_ts(sr[s, :, k]) for s in range(M)]
        st_e = [ao.stats_ts(se[s, :, k]) for s in range(M)]
        mr, _, er = ao.combine_ts(st_r)
        me, _, ee = ao.combine_ts(st_e)
        z = abs(mr - me) / math.sqrt(er * er + ee * ee)
        # paired: per replica the difference of the two runs' averages
        d = [a[0] - b[0] for a, b in zip(st_r, st_e)]
        md, _, ed = ao.combine_basic(d)
        zp = abs(md) / ed if ed > 0 else 0.0
        print("%-34s %.6g +- %.2g | %.6g +- %.2g | %.2f | %.2f" % (name, mr, er, me, ee, z, zp))
        worst = max(worst, z)
        assert z <= 3.0, (name, mr, er, me, ee)
        assert zp <= 5.0, (name, md, ed)
    print("largest |difference| / combined sem: %.2f" % worst)
