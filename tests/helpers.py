"""Shared set-up of the parity tests: ccp parameter texts, engine <-> oracle
glue and the force-error measures."""
import math

import numpy as np

RCO = 1.154701


def ccp_params(N, cvf=0.2, laf=0.25, extra=""):
    """adjustable-parameters text as Scripts/makeallsim.py:44-87 derives it."""
    R = RCO / 2 + RCO / 2 * (N / cvf) ** (1 / 3)
    n_l = int(math.floor(laf * 4 / ((0.5 / (R - RCO)) ** 2)))
    txt = "number_of_particles %05d\nnucleus_radius %09.6f\nnumber_of_lbs %05d\n" % (N, R, n_l)
    return txt + extra, R, n_l


def baseline_params(N, extra=""):
    return "force_field baseline\nnumber_of_particles %d\n" % N + extra


def heads_of(sim, s=0):
    si = sim.system_info(s)
    L = si.n_beads // si.n_chains
    return [c * L for c in range(si.n_chains)]


def force_errors(f_gpu, f_ref, absum):
    """(max relative error |dF|/|F| over beads with |F| >= 1e-3 * S, and the
    max of |dF| / S) where S is the sum of the magnitudes of the force terms."""
    d = np.linalg.norm(np.asarray(f_gpu, np.float64) - f_ref, axis=1)
    n = np.linalg.norm(f_ref, axis=1)
    big = n >= 1e-3 * absum
    rel = (d[big] / n[big]).max() if big.any() else 0.0
    scaled = (d / np.maximum(absum, 1e-30)).max()
    return rel, scaled


def at_cutoff(x, fl, lbs, ff, tol=1e-6):
    """Beads with a pair or a lamina-binding site within tol of its cutoff
    (A-A pairs at rc_att, other pairs at rc_rep). A truncated force jumps at
    its cutoff, and FP32 and FP64 distances can fall on opposite sides of it
    (tol covers a few FP32 ulps of the distance), so the two forces differ by
    the jump there: the baseline Lennard-Jones at 2.5 sigma (~0.02), and the
    Wang-Frenkel at the FP32 cutoff 1.154701, 4.6e-7 beyond its zero at
    2/sqrt(3) (~1e-5; ccp's relaxation leaves many pairs exactly there).
    Such beads are checked against the jump's size instead."""
    from scipy.spatial import cKDTree

    x = np.asarray(x, np.float64)
    fl = np.asarray(fl)
    hit = np.zeros(len(x), bool)
    t = cKDTree(x)
    rmax = max(ff["rc_att"], ff["rc_rep"]) + tol
    for i, j in t.query_pairs(rmax, output_type="ndarray"):
        aa = (fl[i] & 1) and (fl[j] & 1)
        rc = ff["rc_att"] if aa else ff["rc_rep"]
        if abs(np.linalg.norm(x[i] - x[j]) - rc) < tol:
            hit[i] = hit[j] = True
    lad = np.flatnonzero(fl & 2)
    if len(lad) and len(lbs):
        t = cKDTree(np.asarray(lbs, np.float64).reshape(-1, 3))
        for k, near in enumerate(t.query_ball_point(x[lad], ff["lco"] + tol)):
            for l in near:
                if abs(np.linalg.norm(x[lad[k]] - t.data[l]) - ff["lco"]) < tol:
                    hit[lad[k]] = True
    return hit
