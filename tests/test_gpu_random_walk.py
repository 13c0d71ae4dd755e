"""The GPU confined random walk of the initial condition against the oracle's
sequential restatement (oracle/ccp_oracle.c orc_random_walk) of
chrsim::set_particle_positons + perform_random_walk (chrsim.cu:678-802).

Both walk in FP64 on the same Philox stream, so every acceptance decision
agrees: each chain's attempt count must be equal and every position equal to
FP32 rounding.
  * ccp's 30386-bead diploid model: 12 chromosomes in cones around the
    shuffled icosahedral directions;
  * three 2048-bead ccp systems batched: each walks as the oracle says, and
    exactly as the same system created alone;
  * a dense nucleus, where the wall rejects attempts;
  * a walk that can never finish ends at its draw budget with an error.
"""
import math

import numpy as np
import pytest

from helpers import ccp_params

MIS32 = float(np.float32(0.838732))


def _oracle_chain(orc, n, seed, c, axis, cos_mda, R_n, kT):
    return orc.random_walk(n, seed, c, axis, cos_mda, R_n, kT=kT, k_b=1.0, k_e=128.0, l_0=1.0,
                           mis=MIS32)


@pytest.mark.gpu
def test_diploid_walk_matches_oracle(engine_lib, orc):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(orc.N_DEF)
    sim = ChrSim(txt, seed=5)
    si, info = sim.system_info(0), sim.info()
    assert si.n_chains == 12
    rng = np.random.default_rng(0)
    sim.set_types(rng.integers(0, 2, orc.N_DEF).astype(np.int32))
    draws = sim.random_walk()
    x = sim.positions()
    axes, cos_mda = orc.walk_axes(5, True, 12)
    R_n = float(si.nucleus_radius)
    for c in range(12):
        a, b = orc.CHR_LIM[c], orc.CHR_LIM[c + 1]
        ref, used = _oracle_chain(orc, b - a, 5, c, axes[c], cos_mda, R_n, float(info.kT))
        assert used == int(draws[c]), c
        assert np.allclose(x[a:b], ref, rtol=0, atol=2e-5), c
        # cone of the chromosome
        ax = np.asarray(axes[c]) / np.linalg.norm(axes[c])
        cosang = (x[a:b] @ ax) / np.linalg.norm(x[a:b], axis=1)
        assert (cosang >= cos_mda - 1e-5).mean() >= 0.999
    r = np.linalg.norm(x, axis=1)
    assert (R_n - r >= MIS32 - 1e-4).mean() >= 0.999


@pytest.mark.gpu
def test_batched_walk_equals_single_and_oracle(engine_lib, orc):
    from tfm_gb300.ccpgpu import Batch, ChrSim

    txt, R, n_l = ccp_params(2048)
    seeds = [11, 12, 13]
    bt = Batch(txt, [2048] * 3, seeds=seeds)
    draws = bt.random_walk()
    xb = bt.positions()
    kT = float(bt.info().kT)
    for s, seed in enumerate(seeds):
        si = bt.system_info(s)
        assert si.n_chains == 1
        o = si.bead_offset
        ref, used = _oracle_chain(orc, 2048, seed, 0, (0.0, 0.0, 0.0), -1.0,
                                  float(si.nucleus_radius), kT)
        assert used == int(draws[s])
        assert np.allclose(xb[o:o + 2048], ref, rtol=0, atol=2e-5)
    one = ChrSim(txt, seed=12)
    d1 = one.random_walk()
    assert int(d1[0]) == int(draws[1])
    o = bt.system_info(1).bead_offset
    assert np.array_equal(one.positions(), xb[o:o + 2048])
    # the walk leaves a state that relaxes like generate_initial_condition's
    assert bt.overlaps().sum() >= 0


@pytest.mark.gpu
def test_dense_nucleus_walk_rejects(engine_lib, orc):
    """4096 beads at the largest chromatin volume fraction the parameters
    allow (0.4, nucleus radius 13.2): attempts that cross the wall are
    rejected (about 9 % of all attempts)."""
    from tfm_gb300.ccpgpu import ChrSim

    n = 4096
    txt = "number_of_particles %05d\nnucleus_radius %09.6f\nnumber_of_lbs %05d\n" % (n, 13.2, 16)
    sim = ChrSim(txt, seed=21)
    draws = sim.random_walk()
    x = sim.positions()
    si, info = sim.system_info(0), sim.info()
    ref, used = _oracle_chain(orc, n, 21, 0, (0.0, 0.0, 0.0), -1.0, float(si.nucleus_radius),
                              float(info.kT))
    assert used == int(draws[0])
    assert used > 1.05 * n
    assert np.allclose(x, ref, rtol=0, atol=2e-5)


@pytest.mark.gpu
def test_stuck_walk_ends_with_error(engine_lib):
    """At temperature 0 every bond is straight and of length 1: a chain that
    meets the wall can never turn (the reference's walk loops forever there).
    The kernel stops at its draw budget, the call returns ERR_STATE with
    device flag [4] set, and the engine stays usable."""
    from tfm_gb300.ccpgpu import ERR_STATE, CcpError, ChrSim

    txt, R, n_l = ccp_params(256, extra="temperature 0\n")
    sim = ChrSim(txt, seed=4)
    with pytest.raises(CcpError) as ei:
        sim.random_walk()
    assert ei.value.code == ERR_STATE
    flags, rc = sim.error_flags(clear=True)
    assert flags[4] == 1
    assert sim.error_flags()[0][4] == 0
    ok = ChrSim(ccp_params(2048)[0], seed=4)
    ok.generate_initial_condition()
    assert ok.overlaps().sum() == 0


@pytest.mark.gpu
def test_diploid_batch_walks_like_single_systems(engine_lib, orc):
    """A batch of ccp's 30386-bead model defaults to its 12 chromosomes at
    ccp's limits, like a single system created from the same text: each
    system's walk equals that system's walk alone."""
    from tfm_gb300.ccpgpu import Batch, ChrSim

    txt, R, n_l = ccp_params(orc.N_DEF)
    bt = Batch(txt, [orc.N_DEF] * 2, seeds=[5, 6])
    assert [bt.system_info(s).n_chains for s in range(2)] == [12, 12]
    draws = bt.random_walk()
    xb = bt.positions()
    one = ChrSim(txt, seed=6)
    d1 = one.random_walk()
    assert np.array_equal(d1, draws[12:])
    o = bt.system_info(1).bead_offset
    assert np.array_equal(one.positions(), xb[o:o + orc.N_DEF])


@pytest.mark.gpu
def test_large_ccp_relaxation_stays_confined(engine_lib):
    """Relaxing 16 walks of 30385 beads in ccp's force field ends with no
    overlapping pair and every bead inside its nucleus. Without the cap on a
    relaxation stage's displacement, beads pushed close to the wall got a
    Wang-Frenkel wall force that threw them out of the nucleus (positions up
    to 1e17) in 10 of these 16 systems."""
    from tfm_gb300.ccpgpu import Batch

    n, m = 30385, 16
    txt, R, n_l = ccp_params(n)
    bt = Batch(txt, [n] * m, seeds=np.arange(m, dtype=np.uint64) + 101)
    bt.generate_initial_condition()
    flags, _ = bt.error_flags()
    assert not flags[:4].any(), flags
    assert int(bt.overlaps().sum()) == 0
    x = bt.positions()
    for s in range(m):
        si = bt.system_info(s)
        r = np.linalg.norm(x[si.bead_offset:si.bead_offset + si.n_beads], axis=1)
        assert r.max() < si.nucleus_radius, s
