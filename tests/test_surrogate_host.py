"""Host-side helpers of the surrogate pipeline (tfm_gb300/surrogate.py) on
CPU: P(s) by diagonal, its octave means, the power-law baseline, the
envelope and the error measures the tests and bench.py score with."""
import numpy as np


def _maps(rng, n, M, b=-1.2):
    d = np.abs(np.arange(M)[:, None] - np.arange(M)[None, :])
    base = 0.6 * np.maximum(d, 1.0) ** b
    np.fill_diagonal(base, 0.9)
    noise = np.exp(0.05 * rng.standard_normal((n, M, M)))
    m = base[None] * noise
    return ((m + m.transpose(0, 2, 1)) / 2).astype(np.float32)


def test_ps_curve_is_the_diagonal_mean():
    from tfm_gb300 import surrogate as S

    m = _maps(np.random.default_rng(0), 3, 128)
    ps = S.ps_curve(m)
    for s in (0, 1, 7, 64, 127):
        assert np.allclose(ps[:, s], [np.diagonal(x, s).astype(np.float64).mean() for x in m])
    assert np.allclose(S.ps_curve(m, 64), ps[:, :64])


def test_octaves_and_errors():
    from tfm_gb300 import surrogate as S

    m = _maps(np.random.default_rng(1), 4, 128)
    ps = S.ps_curve(m)
    oc = S.ps_octaves(ps, 128)
    # octaves [1, 2), [2, 4), ..., [32, 64) of a 128-bin map
    assert oc.shape == (4, 6)
    assert np.allclose(oc[:, 0], ps[:, 1]) and np.allclose(oc[:, 5], ps[:, 32:64].mean(axis=1))
    assert np.array_equal(S.ps_log_bins(m), oc)
    assert np.allclose(S.ps_error(m, m), 0.0) and np.allclose(S.map_log_error(m, m), 0.0)
    # a map 10 % high everywhere is 10 % off in every octave
    assert np.allclose(S.ps_error(1.1 * m, m), 0.1, rtol=1e-4)


def test_powerlaw_baseline_recovers_an_exact_power_law():
    from tfm_gb300 import surrogate as S

    M = 128
    d = np.abs(np.arange(M)[:, None] - np.arange(M)[None, :])
    exact = (0.6 * np.maximum(d, 1.0) ** -1.3).astype(np.float32)
    np.fill_diagonal(exact, 0.9)
    pl = S.powerlaw_map(np.repeat(exact[None], 3, 0))
    assert pl.shape == (1, M, M)
    assert np.allclose(pl[0], exact, rtol=1e-4)


def test_envelope_widens_the_range_of_the_octaves():
    from tfm_gb300 import surrogate as S

    m = _maps(np.random.default_rng(2), 8, 128)
    lo, hi = S.envelope(m, margin=0.25)
    pb = S.ps_log_bins(m)
    assert np.allclose(lo, pb.min(axis=0) * 0.75) and np.allclose(hi, pb.max(axis=0) * 1.25)
    assert ((pb >= lo) & (pb <= hi)).all()
