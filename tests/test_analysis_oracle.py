"""The analysis oracle against the reference's own analysis code: its
statistics against sostat.cu (tests/golden/sostat.json, printed by
oracle/_ref/sostat_driver built from the reference sources), the
per-simulation time-series line, its summary form, the basic average and the
combined lines, character for character; and its per-frame observables
against chrana::calc_observables (tests/golden/observables_ccp.npz, printed
by oracle/_ref/chrana_driver)."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _cases():
    with open(os.path.join(HERE, "golden", "sostat.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("k", range(30))
def test_statistics_match_reference_lines(k):
    import numpy as np

    from oracle import analysis_oracle as ao

    case = _cases()[k]
    want = case["lines"]
    got, ts, bs = [], [], []
    for s in case["series"]:
        v = np.asarray(s, np.float32)
        st = ao.stats_ts(v)
        ts.append(st)
        got.append("ts " + ao.ts_line(st).rstrip("\n"))
        got.append("ts_s " + ao.ts_line_s(st).rstrip("\n"))
        avg = float(np.cumsum(v.astype(np.float64))[-1]) / len(v)
        bs.append(avg)
        got.append("b " + ao.f6(avg))
    got.append("ts_fin " + ao.fin_line(ao.combine_ts(ts)).rstrip("\n"))
    got.append("b_fin " + ao.fin_line(ao.combine_basic(bs)).rstrip("\n"))
    assert got == want


def _observable_cases():
    import numpy as np

    g = np.load(os.path.join(HERE, "golden", "observables_ccp.npz"))
    return [{k[len("c%d_" % c):]: g[k] for k in g.files if k.startswith("c%d_" % c)}
            for c in range(int(g["n_cases"]))]


@pytest.mark.parametrize("k", range(2))
def test_frame_observables_match_reference(k):
    """Per-frame observables of the analysis oracle (FP64) and of the C oracle
    the engine's GPU observables are tested against, on the frames of
    tests/golden/observables_ccp.npz, against what the reference's own
    chrana::calc_observables computed from them (chrana.cu:371-480, run on
    the host by oracle/_ref/chrana_driver). ccp accumulates in FP32 over the
    beads, so the bounds are FP32-accumulation bounds: Rg^2 within 1e-5
    relative, the radial densities within 1e-4 of their largest value."""
    import numpy as np

    from oracle import analysis_oracle as ao
    from oracle import oracle as orc

    c = _observable_cases()[k]
    xs, types, ref = c["xyz"], c["types"], c["series"]
    R, nod = float(c["R_n"]), float(c["nod"])
    n = len(types)
    for f in range(len(xs)):
        dcm, rg2, nop, ncf, rcd = ao.frame_observables(xs[f], types, R, nod)
        r = ref[f]
        rr = r[5:].reshape(3, 64)
        assert abs(dcm - r[1]) <= 1e-6 * R
        assert abs(rg2 - r[2]) <= 1e-5 * r[2]
        assert abs(nop - r[3]) <= 1e-5
        assert abs(ncf - r[4]) <= 1e-6
        assert np.abs(rcd - rr).max() <= 1e-4 * np.abs(rr).max()
        # the C oracle's sums: sum r, sum |r|^2 and shell volumes per type
        o = orc.observables(xs[f], np.where(types == 0, orc.F_A, 0).astype(np.uint32), R)
        cm = o[:3] / n
        assert abs(o[3] / n - (cm ** 2).sum() - r[2]) <= 1e-5 * r[2]
        shells = np.stack([o[4:68], o[68:132], o[132:196]]) / ((4.0 / 3.0) * np.pi * R ** 3 / 64)
        assert np.abs(shells - rr).max() <= 1e-4 * np.abs(rr).max()
