"""CPU oracle of ccp-analyze's outputs — TEST INFRASTRUCTURE.

Only tests/ import this module. It restates, from positions and contact
counts, what the reference's analysis writes:
  per-frame observables   chrana::calc_observables (Program/src/chrana.cu:371-512):
                          centre-of-mass distance, gyration radius squared,
                          nematic order parameter, nucleus chromatin fraction,
                          radial chromatin density (64 equal-volume shells,
                          A / B / all beads)
  basic observables       the per-frame spatial distance and contact
                          probability by separation (calc_sd_cp, chrana.cu:13-45)
                          and contact map (calc_cm, chrana.cu:48-84), averaged
                          over frames
  statistics              sostat.cu:68-237: plain moments, blocking for the
                          standard error of correlated data, the marginal
                          standard error rule for thermalisation, and the
                          inverse-variance combination of simulations
  files                   analysis-XXX.dat (chrana.cu:205-256), analysis-fin.dat
                          (chrana.cu:306-360), contact-map.bin (chrana.cu:362-369)
The statistics are pinned by tests/golden/sostat.json, printed by the
reference's own sostat.cu (oracle/ref/build_sostat.sh). Floating-point steps
that ccp takes in single precision (the stored series, squares of series
values, pairwise block averages) are taken in single precision here too.
One deliberate difference: for a series too short to block (fewer than 4
values after thermalisation) ccp prints an uninitialised block count and
standard error; here they are the series length and sqrt(var / n).
"""
import math

import numpy as np


def _sqrt(x):
    """sqrt that propagates a NaN's sign and makes a new NaN for x < 0 the way
    the hardware does (C++'s sqrt)."""
    with np.errstate(invalid="ignore"):
        return float(np.sqrt(np.float64(x)))

N_SHELLS = 64
RCO = 1.154701
F32 = np.float32


# ---------------------------------------------------------------- statistics

def stats_id(v):
    """(avg, var, sem) of float values, sostat.cu:69-88."""
    v = np.asarray(v, F32)
    n = len(v)
    m1 = float(np.cumsum(v.astype(np.float64))[-1]) / n
    m2 = float(np.cumsum((v * v).astype(np.float64))[-1]) / n
    with np.errstate(divide="ignore", invalid="ignore"):
        var = float(np.float64(m2 - m1 * m1) / np.float64(1.0 - 1.0 / n))
        sem = _sqrt(np.float64(var) / n)
    return m1, var, sem


def stats_cd(v):
    """(avg, var, sem, n_blocks) of correlated values by blocking, sostat.cu:90-134."""
    av = np.asarray(v, F32).copy()
    avg, var, _ = stats_id(av)
    n = len(av)
    ivm = var / n
    ul = ivm * (1.0 + math.sqrt(2.0 / (n - 1.0))) if n > 1 else float("inf")  # n = 1: no blocking
    sem, fnb = _sqrt(ivm), n
    while n >= 4:
        nb = n // 2
        av = ((av[0:2 * nb:2] + av[1:2 * nb:2]) * F32(0.5)).astype(F32)
        n = nb
        _, bvar, _ = stats_id(av)
        ivm = bvar / n
        sem, fnb = _sqrt(ivm), n
        if ivm > ul:
            ul = ivm * (1.0 + math.sqrt(2.0 / (n - 1.0)))
        else:
            break
    return avg, var, sem, fnb


def stats_ts(v):
    """Time-series statistics, sostat.cu:136-174: (avg, var, sem, n_blocks,
    thermalisation index, thermalised)."""
    v = np.asarray(v, F32)
    n0 = len(v)
    best, it = float("inf"), n0 // 2
    d = 2
    while d < 128:
        i_t = n0 // d
        av = v[i_t:]
        ne = len(av)
        _, var, _ = stats_id(av)
        mse = var * (ne - 1) / (ne * ne)
        if mse < best:
            best, it = mse, i_t
        d *= 2
    avg, var, sem, fnb = stats_cd(v[it:])
    return avg, var, sem, fnb, it, it != n0 // 2


def combine_ts(stats):
    """Inverse-variance combination of per-simulation statistics, sostat.cu:176-204."""
    m1 = m2 = w1 = w2 = 0.0
    for s in stats:
        with np.errstate(divide="ignore", invalid="ignore"):
            w = float(np.float64(1.0) / np.float64(s[2] * s[2]))
        if not math.isfinite(w):
            w = 1.0
        m1 += w * s[0]
        m2 += w * s[0] * s[0]
        w1 += w
        w2 += w * w
    m1 /= w1
    m2 /= w1
    with np.errstate(divide="ignore", invalid="ignore"):
        var = float(np.float64(m2 - m1 * m1) / np.float64(1.0 - w2 / (w1 * w1)))
        sem = _sqrt(np.float64(var) * w2 / (w1 * w1))
    return m1, var, sem


def combine_basic(avgs):
    """Plain combination of per-simulation averages, sostat.cu:206-224."""
    m1 = m2 = 0.0
    for a in avgs:
        m1 += a
        m2 += a * a
    n = len(avgs)
    m1 /= n
    m2 /= n
    with np.errstate(divide="ignore", invalid="ignore"):
        var = float(np.float64(m2 - m1 * m1) / np.float64(1.0 - 1.0 / n))
        sem = _sqrt(np.float64(var) / n)
    return m1, var, sem


def f6(x):
    """%12.6f as C's printf writes it, including the sign of a NaN."""
    if math.isnan(x):
        return "%12s" % ("-nan" if math.copysign(1.0, x) < 0 else "nan")
    return "%12.6f" % x


def ts_line(s):
    """save_last_is_stat, sostat.cu:20-26."""
    return (f6(s[0]) + f6(_sqrt(s[1])) + f6(s[2])
            + "%8d" % s[3] + "%8d" % s[4] + (" yes" if s[5] else "  no") + "\n")


def ts_line_s(s):
    """save_last_is_stat_s, sostat.cu:28-34."""
    return f6(s[0]) + f6(_sqrt(s[1])) + f6(s[2]) + "\n"


def fin_line(s):
    """save_cs_final_stat, sostat.cu:36-41."""
    return f6(s[0]) + f6(_sqrt(s[1])) + f6(s[2]) + "\n"


# ---------------------------------------------------------------- observables

def frame_observables(xyz, types, R_n, nod):
    """Per-frame scalars and radial densities of one system (chrana.cu:371-468),
    in FP64, stored as float32 like ccp's series: (dcm, rg2, nop, ncf, rcd[3][64])."""
    x = np.asarray(xyz, np.float64)
    n = len(x)
    cm = x.mean(axis=0)
    dcm = np.linalg.norm(cm)
    rg2 = ((x - cm) ** 2).sum(axis=1).mean()
    b = x[1:] - x[:-1]
    cos = (b * x[:-1]).sum(axis=1) / (np.linalg.norm(b, axis=1) * np.linalg.norm(x[:-1], axis=1))
    nop = (0.5 * (3.0 * cos * cos - 1.0)).mean()
    ncf = np.count_nonzero(x[:, 2] < nod) / n
    a = RCO / 2.0
    rb = R_n * ((np.arange(N_SHELLS) + 1.0) / N_SHELLS) ** (1.0 / 3)
    dr = np.linalg.norm(x, axis=1)[:, None]
    r = rb[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        ca = (dr * dr + a * a - r * r) / (2.0 * dr * a)
        cb = (r * r + dr * dr - a * a) / (2.0 * r * dr)
        v = (math.pi / 3.0) * a ** 3 * (2.0 + ca) * (1.0 - ca) ** 2 + (math.pi / 3.0) * r ** 3 * (2.0 + cb) * (1.0 - cb) ** 2
    v = np.where(dr - a > r, 0.0, np.where(dr + a < r, (4.0 / 3.0) * math.pi * a ** 3, v))
    dv = np.diff(np.concatenate([np.zeros((n, 1)), v], axis=1), axis=1)
    t = np.asarray(types)
    rcd = np.stack([dv[t == 0].sum(axis=0), dv[t == 1].sum(axis=0), dv.sum(axis=0)])
    rcd /= (4.0 / 3.0) * math.pi * R_n ** 3 / N_SHELLS
    return (F32(dcm), F32(rg2), F32(nop), F32(ncf), rcd.astype(F32))


def analysis_txt(series, R_n, sd, cp, n_blocks=6):
    """analysis-XXX.dat of one simulation. series: list of frame_observables
    tuples; sd, cp: per block, the frame-averaged values for s = 1, 2, ...
    Returns (text, time-series statistics for analysis_fin_txt)."""
    cols = [np.array([f[k] for f in series], F32) for k in range(4)]
    rcd = np.array([f[4] for f in series], F32)  # [frames][3][64]
    out = "         avg   sqrt(var)         sem   f_n_b     i_t ter\n"
    st = {"scalars": [], "rcd": np.empty((3, N_SHELLS), object)}
    for c in cols:
        s = stats_ts(c)
        st["scalars"].append(s)
        out += ts_line(s)
    out += "\n\n"
    for t in range(3):
        out += "         r_b         avg   sqrt(var)         sem\n"
        out += "    0.000000    0.000000    0.000000    0.000000\n"
        for b in range(N_SHELLS):
            s = stats_ts(rcd[:, t, b])
            st["rcd"][t, b] = s
            out += f6(float(F32(R_n)) * ((b + 1.0) / N_SHELLS) ** (1.0 / 3)) + ts_line_s(s)
        out += "\n\n"
    for arr in (sd, cp):
        for blk in range(n_blocks):
            out += "     s         avg\n"
            vals = arr[blk] if blk < len(arr) else []
            for i, v in enumerate(vals):
                out += "%6d" % (i + 1) + f6(v) + "\n"
            out += "\n\n"
    return out, st


def analysis_fin_txt(stats, R_n, sd_sims, cp_sims, n_blocks=6):
    """analysis-fin.dat over simulations: stats from analysis_txt, and per
    simulation its sd / cp block averages."""
    out = "         avg   sqrt(var)         sem\n"
    for k in range(4):
        out += fin_line(combine_ts([s["scalars"][k] for s in stats]))
    out += "\n\n"
    for t in range(3):
        out += "         r_b         avg   sqrt(var)         sem\n"
        out += "    0.000000    0.000000    0.000000    0.000000\n"
        for b in range(N_SHELLS):
            out += f6(float(F32(R_n)) * ((b + 1.0) / N_SHELLS) ** (1.0 / 3))
            out += fin_line(combine_ts([s["rcd"][t, b] for s in stats]))
        out += "\n\n"
    for sims in (sd_sims, cp_sims):
        for blk in range(n_blocks):
            out += "     s         avg   sqrt(var)         sem\n"
            n_s = len(sims[0][blk]) if blk < len(sims[0]) else 0
            for i in range(n_s):
                out += "%6d" % (i + 1) + fin_line(combine_basic([s[blk][i] for s in sims]))
            out += "\n\n"
    return out
