"""The oracle's confined random walk (oracle/ccp_oracle.c orc_random_walk)
against the distributions chrsim::perform_random_walk (chrsim.cu:719-802)
draws from. The reference seeds cuRAND's host generator with time(nullptr)
(chrsim.cu:474-475), so its walks are not reproducible; the restatement is
pinned to what the reference's formulas sample:
  * bond length l_0 + sqrt(2 kT / k_e) erfinv(2u - 1): the Boltzmann
    distribution of the harmonic bond, normal with mean l_0 and standard
    deviation sqrt(kT / k_e);
  * bond angle acos(1 + ln(1 - (1 - e^(-1/kT)) u) / (0.5/kT)): cos(theta)
    with density proportional to exp(cos(theta) / (2 kT)) on [-1, 1];
  * the new direction's azimuth about the old one uniform;
  * every accepted bead at least mis inside the wall and inside its cone;
  * ccp's 12 cone axes a permutation of the icosahedral directions.
"""
import math

import numpy as np
import pytest

scipy_stats = pytest.importorskip("scipy.stats")


def _bonds(x):
    b = np.diff(x, axis=0)
    return b, np.linalg.norm(b, axis=1)


def test_bond_length_is_boltzmann(orc):
    for kT, k_e in ((1.0, 128.0), (0.5, 100.0)):
        x, used = orc.random_walk(20000, 3, 0, (0, 0, 0), -1.0, 1.0e4, kT=kT, k_e=k_e)
        assert used == 20000  # nothing to reject far from the wall
        _, L = _bonds(x)
        sd = math.sqrt(kT / k_e)
        p = scipy_stats.kstest((L - 1.0) / sd, scipy_stats.norm.cdf).pvalue
        assert p > 1e-3, (kT, k_e, p)


def test_bond_angle_is_boltzmann(orc):
    for kT in (1.0, 0.25):
        x, _ = orc.random_walk(20000, 5, 0, (0, 0, 0), -1.0, 1.0e4, kT=kT)
        b, L = _bonds(x)
        u = b / L[:, None]
        c = np.clip((u[1:] * u[:-1]).sum(1), -1.0, 1.0)
        a = 0.5 / kT  # density exp(a cos) on [-1, 1]
        cdf = lambda t: (np.exp(a * t) - math.exp(-a)) / (math.exp(a) - math.exp(-a))
        p = scipy_stats.kstest(c, cdf).pvalue
        assert p > 1e-3, (kT, p)
        # azimuth of bond k+1 about bond k, measured from a fixed reference
        # perpendicular: uniform on [0, 2 pi)
        ref = np.cross(u[:-1], np.array([0.3, -0.5, 0.81]))
        ref /= np.linalg.norm(ref, axis=1)[:, None]
        ort = np.cross(u[:-1], ref)
        w = u[1:] - c[:, None] * u[:-1]
        phi = np.arctan2((w * ort).sum(1), (w * ref).sum(1)) % (2 * math.pi)
        p = scipy_stats.kstest(phi / (2 * math.pi), lambda t: np.clip(t, 0.0, 1.0)).pvalue
        assert p > 1e-3, (kT, p)


def test_confinement_and_cones(orc):
    R_n = 13.2
    x, used = orc.random_walk(4096, 1, 0, (0, 0, 0), -1.0, R_n)
    assert used > 4096
    assert (R_n - np.linalg.norm(x, axis=1) >= orc.MIS - 1e-12).all()
    axes, cos_mda = orc.walk_axes(9, True, 12)
    assert math.isclose(cos_mda, math.cos(math.pi / 2 - math.atan((1 + 5 ** 0.5) / 2)))
    for c in (0, 5, 11):
        x, _ = orc.random_walk(2000, 9, c, axes[c], cos_mda, 17.0)
        a = np.asarray(axes[c]) / np.linalg.norm(axes[c])
        cosang = (x @ a) / np.linalg.norm(x, axis=1)
        assert (cosang >= cos_mda - 1e-12).all()
        assert (17.0 - np.linalg.norm(x, axis=1) >= orc.MIS - 1e-12).all()


def test_cone_axes_are_a_shuffle(orc):
    phi = (1 + 5 ** 0.5) / 2
    ico = {(0, 1, phi), (1, phi, 0), (phi, 0, 1), (0, 1, -phi), (1, -phi, 0), (-phi, 0, 1),
           (0, -1, phi), (-1, phi, 0), (phi, 0, -1), (0, -1, -phi), (-1, -phi, 0), (-phi, 0, -1)}
    seen = set()
    for seed in range(4):
        axes, _ = orc.walk_axes(seed, True, 12)
        assert set(axes) == ico
        seen.add(tuple(axes))
    assert len(seen) == 4
    axes, cm = orc.walk_axes(0, False, 3)
    assert axes == [(0.0, 0.0, 0.0)] * 3 and cm == -1.0


def test_walk_is_deterministic_and_bounded(orc):
    a, ua = orc.random_walk(500, 7, 2, (0, 0, 0), -1.0, 10.0)
    b, ub = orc.random_walk(500, 7, 2, (0, 0, 0), -1.0, 10.0)
    c, _ = orc.random_walk(500, 7, 3, (0, 0, 0), -1.0, 10.0)
    assert ua == ub and np.array_equal(a, b)
    assert not np.allclose(a, c)
    # a budget smaller than the chain ends the walk with -1
    _, u = orc.random_walk(500, 7, 2, (0, 0, 0), -1.0, 10.0, max_draws=100)
    assert u == -1
