"""Parity at the full sizes of the benchmark configurations, through checks
that do not grow with the system beyond what the oracle does in seconds:

  * one 131072-bead system (16 chains of 8192, baseline force field): every
    bead's force against the FP64 oracle after 200 steps (cell-list oracle,
    O(N)) within the 1e-5 bound;
  * the 512-replica ensemble (2.79 M beads, log-uniform sizes 1024-16384):
    after the initial condition and 200 steps no device flag is set (no
    non-finite position, no bead outside its grid, no counting-sort slot
    outside its replica, no exhausted noise redraw), every position is
    inside its own nucleus, and for replicas spread over the size range the
    forces meet the oracle bound and the contact counts equal the oracle's
    all-pairs counts.
"""
import math

import numpy as np
import pytest

from helpers import at_cutoff

FORCE_RTOL = 1e-5
PARAMS = ("force_field baseline\ncontact_bins 256\ncontact_cutoff 1.5\n"
          "steps_per_frame 100\npacking_fraction 0.2\n")


def _force_ratio(f, f64, sa):
    """Per bead |F - F_64| / max(|F_64|, 0.1 S, 1)."""
    d = np.linalg.norm(np.asarray(f, np.float64) - f64, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f64, axis=1), 0.1 * sa), 1.0)
    return d / scale


def _force_bound(f, f64, sa, skip):
    e = _force_ratio(f, f64, sa)
    return e[~skip].max(), e.max()


def _replica_sizes(n_rep, seed=2026):
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(1024), math.log(16384), n_rep))).astype(np.int32)


@pytest.mark.gpu
def test_c1_system_forces(engine_lib, orc):
    from tfm_gb300.ccpgpu import Batch

    n = 131072
    b = Batch(PARAMS.replace("contact_bins 256", "contact_bins 1024"), [n], n_chains=[16],
              seeds=[42])
    b.generate_initial_condition()
    b.run_steps(200)
    x, pt, lbs = b.positions(), b.types(), b.lbs()
    si = b.system_info(0)
    heads = [c * (n // 16) for c in range(16)]
    fl = orc.flags_from_types(pt, heads, "baseline")
    ff = orc.baseline_ff()
    geo = orc.geo_vec(si.nucleus_radius, csl=2.5)
    f64, sa = orc.forces(x, fl, lbs, ff, geo, with_abs=True, cells=True)
    fg = b.forces()
    edge = at_cutoff(x, fl, lbs, ff)
    e = _force_ratio(fg, f64, sa)
    inner, every = e[~edge].max(), e.max()
    above = int((e[~edge] > FORCE_RTOL).sum())
    print("c1 forces: bound %.3g, %d beads above %g (%d of %d beads at a cutoff)"
          % (inner, above, FORCE_RTOL, edge.sum(), n))
    worst = np.flatnonzero(~edge)[np.argsort(e[~edge])[-3:]]
    for i in worst:  # the tail beads: error, |F_64| and the sum of term magnitudes S
        print("  bead %d: ratio %.3g  |dF| %.3g  |F| %.4g  S %.4g" % (
            i, e[i], np.linalg.norm(fg[i] - f64[i]), np.linalg.norm(f64[i]), sa[i]))
    assert above == 0 and inner <= FORCE_RTOL and every <= 1e-2
    b.close()


@pytest.mark.gpu
def test_c2_ensemble_invariants_and_samples(engine_lib, orc):
    from tfm_gb300.ccpgpu import Batch

    sizes = _replica_sizes(512)
    b = Batch(PARAMS, sizes, seeds=np.arange(512, dtype=np.uint64) + 1)
    b.generate_initial_condition()
    b.run_steps(200, observe_every=100)
    flags, rc = b.error_flags()
    assert not flags[:4].any(), flags
    x = b.positions()
    assert np.isfinite(x).all()
    pt, lbs = b.types(), b.lbs()
    assert b.info().n_beads == int(sizes.sum())
    # every replica's beads inside its own nucleus (the WCA wall at R_n)
    for s in range(512):
        si = b.system_info(s)
        r = np.linalg.norm(x[si.bead_offset:si.bead_offset + si.n_beads], axis=1)
        assert r.max() < si.nucleus_radius + 0.1, s
    # forces and contact counts of replicas across the size range
    ff = orc.baseline_ff()
    f = b.forces()
    order = np.argsort(sizes)
    picks = [int(order[k]) for k in (0, 128, 256, 384, 511)]
    b.reset_observables()
    b.observe()
    for s in picks:
        si = b.system_info(s)
        sl = slice(si.bead_offset, si.bead_offset + si.n_beads)
        fl = orc.flags_from_types(pt[sl], [0], "baseline")
        geo = orc.geo_vec(si.nucleus_radius, csl=2.5)
        ls = lbs[si.lbs_offset:si.lbs_offset + si.n_lbs]
        f64, sa = orc.forces(x[sl], fl, ls, ff, geo, with_abs=True, cells=True)
        edge = at_cutoff(x[sl], fl, ls, ff)
        inner, every = _force_bound(f[sl], f64, sa, edge)
        assert inner <= FORCE_RTOL and every <= 1e-2, (s, inner, every)
        m, ps, _ = orc.contacts(x[sl], 1.5, si.contact_bins, si.map_len, si.copy_len,
                                si.n_copies, [0])
        assert np.array_equal(b.contact_counts(s), m), s
    b.close()
