"""Edge cases of the batched engine against the FP64 oracle: systems of one,
two and three beads; chains of a single bead (no bonds at all); and one batch
that mixes such systems with a 2048-bead one. Each goes through the GPU
initial condition, 50 Heun steps, then forces (oracle bound) and contact
counts (bit-exact)."""
import numpy as np
import pytest

from helpers import at_cutoff, ccp_params

FORCE_RTOL = 1e-5


def _check_system(b, s, orc, ff, preset, heads, csl):
    x, pt, lbs = b.positions(), b.types(), b.lbs()
    si = b.system_info(s)
    sl = slice(si.bead_offset, si.bead_offset + si.n_beads)
    fl = orc.flags_from_types(pt[sl], heads, preset)
    geo = orc.geo_vec(si.nucleus_radius, csl=csl)
    ls = lbs[si.lbs_offset:si.lbs_offset + si.n_lbs]
    f64, sa = orc.forces(x[sl], fl, ls, ff, geo, with_abs=True, cells=True)
    f = b.forces()[sl]
    assert np.isfinite(f).all()
    d = np.linalg.norm(f.astype(np.float64) - f64, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f64, axis=1), 0.1 * sa), 1.0)
    e = d / scale
    edge = at_cutoff(x[sl], fl, ls, ff)
    assert e[~edge].max(initial=0.0) <= FORCE_RTOL and e.max(initial=0.0) <= 1e-2
    return x[sl]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_ccp_systems(engine_lib, orc, n):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(n)
    sim = ChrSim(txt + "number_of_lbs 0\n", seed=3)
    sim.generate_initial_condition()
    sim.run_steps(50)
    x = sim.positions()
    assert x.shape == (n, 3) and np.isfinite(x).all()
    assert np.linalg.norm(x, axis=1).max() < R
    _check_system(sim, 0, orc, orc.ccp_ff(), "ccp", [0], 2.0)
    sim.reset_observables()
    sim.observe()
    si = sim.system_info(0)
    m, ps, _ = orc.contacts(x, 2.0, si.contact_bins, si.map_len, si.copy_len, si.n_copies, [0])
    assert np.array_equal(sim.contact_counts(0), m)


@pytest.mark.gpu
def test_single_bead_chains_and_a_mixed_batch(engine_lib, orc):
    """Chains of one bead have no bonds; in a batch of 1, 2, 5 and 2048 beads
    (the 5-bead system as five one-bead chains) every system meets the
    oracle bound and no device flag is set."""
    from tfm_gb300.ccpgpu import Batch

    sizes = [1, 2, 5, 2048]
    chains = [1, 1, 5, 4]
    radii = [2.5, 2.5, 3.0, 0.5 * (2048 / 0.2) ** (1 / 3)]
    b = Batch("force_field baseline\ncontact_bins 64\n", sizes, n_chains=chains, radii=radii,
              seeds=[11, 12, 13, 14])
    b.generate_initial_condition()
    b.run_steps(50)
    flags, rc = b.error_flags()
    assert not flags[:4].any(), flags
    for s, (n, nc) in enumerate(zip(sizes, chains)):
        heads = [c * (n // nc) for c in range(nc)]
        x = _check_system(b, s, orc, orc.baseline_ff(), "baseline", heads, 2.5)
        assert np.isfinite(x).all()
