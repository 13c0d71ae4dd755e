"""The analysis oracle's statistics against the reference's own sostat.cu
(tests/golden/sostat.json, printed by oracle/_ref/sostat_driver built from
the reference sources): the per-simulation time-series line, its summary
form, the basic average, and the combined lines, character for character."""
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
