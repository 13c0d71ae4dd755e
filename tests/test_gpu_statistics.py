"""Statistical agreement with ccp's own dynamics.

ccp seeds its noise with the time, so its trajectories cannot be reproduced
bit for bit; what must agree is what they sample. M replicas of ccp's model
(chromatin volume fraction 0.2, lamina area fraction 0.25, ccp's force
field) start from the engine's initial conditions: one chain of 2048 beads,
and ccp's diploid model of 30386 beads in 12 chromosomes (the bond limits of
chrdat.cuh:28-31, the cone walk of chrsim.cu:694-703; its type sequence,
which ccp reads from a file, is a seeded two-type block sequence here). Each start is run
twice for the same number of Heun steps: by the reference's own kernels
(oracle/ccp_gpu_ref.py: begin_iter, the cell list, exec_RK_1/2 compiled from
the reference's sources, cuRAND noise) and by the engine (batched, Philox
noise). Per frame the same code measures both: the gyration radius squared
and the radial chromatin density (chrana.cu:390-480, in 8 groups of 8 of
ccp's 64 equal-volume shells; computed on the GPU by the formulas of the
analysis oracle, which a CPU check here ties to the oracle's own frame
function) and the contact probability by separation octave over the pairs
of one chromosome (the contact rule of calc_sd_cp, chrana.cu:13-45, at
aco = 2).

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

M = 16            # replicas
SPF = 100         # Heun steps per frame
FRAMES = {2048: 100, 30386: 60}  # 10^4 and 6000 steps (4.9 and 2.9 time units)
OCTAVES = range(1, 10)  # separations [2^k, 2^(k+1)), k = 1..9
ACO = 2.0
N_SHELLS = 64


def _chain_limits(n):
    from oracle.oracle import CHR_LIM

    return list(CHR_LIM) if n == CHR_LIM[-1] else [0, n]


def _band(n, limits, device):
    """Index tables for the pairs (i, i + s), s in [2, 1024), inside one chain."""
    import torch

    s = torch.arange(2 ** OCTAVES[0], 2 ** (OCTAVES[-1] + 1), device=device)
    i = torch.arange(n, device=device)
    cid = torch.zeros(n, dtype=torch.long, device=device)
    for c, a in enumerate(limits[1:-1]):
        cid[a:] = c + 1
    j = i[:, None] + s[None, :]
    jc = j.clamp(max=n - 1)
    valid = (j < n) & (cid[:, None] == cid[jc])
    octave = torch.floor(torch.log2(s.double())).long() - OCTAVES[0]
    pairs = torch.zeros(len(OCTAVES), dtype=torch.float64, device=device)
    pairs.index_add_(0, octave, valid.sum(0).double())
    return jc, valid, octave, pairs


def _contact_octaves(r, band):
    import torch

    jc, valid, octave, pairs = band
    x = r.double()
    d2 = ((x[jc] - x[:, None, :]) ** 2).sum(-1)
    per_s = ((d2 < ACO * ACO) & valid).sum(0).double()
    c = torch.zeros(len(OCTAVES), dtype=torch.float64, device=r.device)
    c.index_add_(0, octave, per_s)
    return c / pairs


def _rg2_and_density(r, R_n):
    """Rg^2 and the radial chromatin density of all beads over ccp's 64
    equal-volume shells: the overlap volume of a sphere of radius rco / 2
    around each bead with each shell (chrana.cu:390-468), as
    analysis_oracle.frame_observables computes it, in FP64 on the device."""
    import torch

    from oracle.analysis_oracle import RCO

    x = r.double()
    rg2 = ((x - x.mean(0)) ** 2).sum(1).mean()
    a = RCO / 2.0
    rb = R_n * ((torch.arange(N_SHELLS, device=r.device, dtype=torch.float64) + 1.0)
                / N_SHELLS) ** (1.0 / 3)
    dr = x.norm(dim=1)[:, None]
    rr = rb[None, :]
    ca = (dr * dr + a * a - rr * rr) / (2.0 * dr * a)
    cb = (rr * rr + dr * dr - a * a) / (2.0 * rr * dr)
    v = (math.pi / 3.0) * a ** 3 * (2.0 + ca) * (1.0 - ca) ** 2 \
        + (math.pi / 3.0) * rr ** 3 * (2.0 + cb) * (1.0 - cb) ** 2
    v = torch.where(dr - a > rr, torch.zeros_like(v),
                    torch.where(dr + a < rr, torch.full_like(v, (4.0 / 3.0) * math.pi * a ** 3), v))
    dv = torch.diff(v, dim=1, prepend=torch.zeros_like(v[:, :1]))
    rcd = dv.sum(0) / ((4.0 / 3.0) * math.pi * R_n ** 3 / N_SHELLS)
    return rg2, rcd


def _frame(r_dev, R_n, band):
    rg2, rcd = _rg2_and_density(r_dev, R_n)
    rad = rcd.reshape(8, 8).mean(dim=1)
    return np.concatenate([[float(rg2)], _contact_octaves(r_dev, band).cpu().numpy(),
                           rad.cpu().numpy()])


NAMES = (["Rg^2"] + ["P(s), s in [%d, %d)" % (2 ** k, 2 ** (k + 1)) for k in OCTAVES]
         + ["radial density, shells %d-%d" % (8 * g + 1, 8 * g + 8) for g in range(8)])


def _block_sequence(n, seed, mean_block=16.0):
    """Two-type block sequence ('A'/'B' per bead), block lengths geometric."""
    rng = np.random.default_rng(seed)
    out, t = [], rng.integers(2)
    while len(out) < n:
        out += ["AB"[t]] * int(rng.geometric(1.0 / mean_block))
        t = 1 - t
    return "".join(out[:n])


def test_frame_observables_follow_the_oracle():
    """The device-side Rg^2, radial density and octave contacts equal the
    analysis oracle's frame function and an all-pairs count on CPU tensors."""
    torch = pytest.importorskip("torch")

    from oracle import analysis_oracle as ao

    rng = np.random.default_rng(3)
    n, R_n = 3000, 12.0
    x = rng.normal(size=(n, 3))
    x *= (R_n * rng.random(n) ** (1 / 3) / np.linalg.norm(x, axis=1))[:, None]
    t = torch.tensor(x, dtype=torch.float32)
    rg2, rcd = _rg2_and_density(t, R_n)
    _, rg2_o, _, _, rcd_o = ao.frame_observables(t.numpy(), np.zeros(n, np.int32), R_n, R_n)
    assert abs(float(rg2) - float(rg2_o)) <= 1e-6 * float(rg2_o)
    assert np.allclose(rcd.numpy(), rcd_o[2].astype(np.float64), rtol=1e-5, atol=1e-6)
    limits = [0, 1000, 3000]
    c = _contact_octaves(t, _band(n, limits, t.device)).numpy()
    xd = t.numpy().astype(np.float64)
    d = np.linalg.norm(xd[:, None, :] - xd[None, :, :], axis=2)
    cid = np.repeat([0, 1], [1000, 2000])
    sep = np.abs(np.arange(n)[:, None] - np.arange(n)[None, :])
    same = (cid[:, None] == cid[None, :]) & (np.arange(n)[:, None] < np.arange(n)[None, :])
    for k, o in enumerate(OCTAVES):
        sel = same & (sep >= 2 ** o) & (sep < 2 ** (o + 1))
        assert c[k] == (d[sel] < ACO).sum() / sel.sum()


@pytest.mark.gpu
@pytest.mark.parametrize("N", [2048, 30386])
def test_engine_samples_what_ccp_samples(engine_lib, tmp_path, N):
    import torch

    from oracle import analysis_oracle as ao
    from oracle import ccp_gpu_ref as ref
    from tfm_gb300.ccpgpu import Batch

    try:
        mod = ref.Module()
    except FileNotFoundError as e:
        pytest.skip(str(e))
    dev = torch.device("cuda")
    frames = FRAMES[N]
    txt, R_n, n_l = ccp_params(N)
    limits = _chain_limits(N)
    if len(limits) > 2:  # ccp's diploid model reads its sequence from a file
        seq = tmp_path / "sequence.txt"
        seq.write_text(_block_sequence(N, seed=11))
        txt += "sequence_file %s\n" % seq
    eng = Batch(txt, [N] * M, seeds=np.arange(M, dtype=np.uint64) + 101)
    eng.generate_initial_condition()
    x0, types, lbs = eng.positions(), eng.types(), eng.lbs()
    infos = [eng.system_info(s) for s in range(M)]
    assert all(si.n_chains == len(limits) - 1 for si in infos)
    band = _band(N, limits, dev)

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
    for f in range(frames):
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
            series_ref[s].append(_frame(sysr.r, si.nucleus_radius, band))
            series_eng[s].append(_frame(xe[sl], si.nucleus_radius, band))
    flags, _ = eng.error_flags()
    assert not flags[:4].any(), flags
    eng.close()
    mod.close()

    sr = np.asarray(series_ref)  # (M, frames, observables)
    se = np.asarray(series_eng)
    worst = 0.0
    print("\nN = %d, %d replicas x %d Heun steps" % (N, M, frames * SPF))
    print("observable: ccp mean +- sem | engine mean +- sem | z | paired z")
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
