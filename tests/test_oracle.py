"""CPU tests of the oracle: published known-answer vectors, internal
cross-checks, and the golden fixtures produced by the reference's own kernels."""
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_philox_known_answers(orc):
    # Philox4x32-10 known-answer vectors published with Random123 (Salmon et al. 2011)
    assert [hex(v) for v in orc.philox([0, 0, 0, 0], [0, 0])] == [
        "0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == [
        "0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                       [0xA4093822, 0x299F31D0])] == [
        "0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_noise_is_truncated_standard_normal(orc):
    z = np.array([orc.noise(b, s, 99) for b in range(300) for s in range(40)])
    assert np.abs(z).max() <= 5.0
    assert abs(z.mean()) < 0.02
    assert abs(z.std() - 1.0) < 0.02
    # counter-based: the same (bead, step, seed) gives the same triple
    assert np.array_equal(orc.noise(7, 123, 5), orc.noise(7, 123, 5))
    assert not np.array_equal(orc.noise(7, 123, 5), orc.noise(7, 124, 5))


def _walk(n, R, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 3), np.float32)
    for i in range(1, n):
        while True:
            d = rng.normal(size=3)
            p = x[i - 1] + d / np.linalg.norm(d)
            if np.linalg.norm(p) < R - 1.0:
                break
        x[i] = p
    return x + rng.normal(scale=0.05, size=x.shape).astype(np.float32)


@pytest.mark.parametrize("preset", ["ccp", "baseline"])
def test_cell_list_equals_all_pairs(orc, preset):
    n, R = 600, 8.0
    x = _walk(n, R, 3)
    pt = (np.arange(n) // 17 % 2).astype(np.int32)
    if preset == "baseline":
        pt |= np.where(np.arange(n) % 10 == 0, 2, 0).astype(np.int32)
    fl = orc.flags_from_types(pt, [0, 300], preset)
    lbs = (np.array([[0, 0, 1.0]]) * (R - 1.1547)).astype(np.float32)
    ff = orc.ccp_ff() if preset == "ccp" else orc.baseline_ff()
    geo = orc.geo_vec(R, csl=2.0 if preset == "ccp" else 2.5)
    a = orc.forces(x, fl, lbs, ff, geo)
    b = orc.forces(x, fl, lbs, ff, geo, cells=True)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-9)


def test_pair_forces_sum_to_zero(orc):
    """Newton's third law of the pair terms (no bonds, wall or sites)."""
    n, R = 400, 7.0
    x = _walk(n, R, 4)
    ff = dict(orc.ccp_ff(), k_e=0.0, k_b=0.0, e_w=0.0, e_l=0.0)
    fl = orc.flags_from_types(np.zeros(n, np.int32), [0])
    f = orc.forces(x, fl, np.zeros((0, 3), np.float32), ff, orc.geo_vec(R))
    assert np.abs(f.sum(axis=0)).max() < 1e-8 * np.abs(f).sum()


def test_bonded_force_is_minus_gradient(orc):
    """Elastic + bending forces (bending on every bead) equal -dV/dr of
    V = sum k_e/2 (d - l0)^2 + k_b (1 - cos) by central differences."""
    n = 12
    x = _walk(n, 50.0, 5).astype(np.float64)
    ff = dict(orc.baseline_ff(), e_att=0.0, e_rep=0.0, e_w=0.0, e_l=0.0)
    fl = orc.flags_from_types(np.zeros(n, np.int32), [0])

    def V(y):
        b = np.diff(y, axis=0)
        d = np.linalg.norm(b, axis=1)
        c = (b[1:] * b[:-1]).sum(1) / (d[1:] * d[:-1])
        return 0.5 * ff["k_e"] * ((d - 1) ** 2).sum() + ff["k_b"] * (1 - c).sum()

    f = orc.forces(x.astype(np.float32), fl, np.zeros((0, 3), np.float32), ff,
                   orc.geo_vec(100.0, csl=2.5))
    xf = x.astype(np.float32).astype(np.float64)
    h = 1e-6
    g = np.zeros_like(xf)
    for i in range(n):
        for k in range(3):
            p, m = xf.copy(), xf.copy()
            p[i, k] += h
            m[i, k] -= h
            g[i, k] = -(V(p) - V(m)) / (2 * h)
    assert np.allclose(f, g, rtol=1e-5, atol=1e-5)


def test_contacts_and_overlaps_brute_force(orc):
    x = _walk(300, 6.0, 6)
    m, ps, ps_off = orc.contacts(x, 2.0, 75, 300, 300, 1, [0])
    # brute force in numpy with the same FP32 predicate
    d2 = None
    cnt = 0
    for i in range(300):
        dx = (x[i] - x[i + 1:]).astype(np.float32)
        dd = np.sqrt(np.float32(dx[:, 2]) * dx[:, 2] + (dx[:, 1] * dx[:, 1] + dx[:, 0] * dx[:, 0]))
        cnt += int((dd < 2.0).sum())
    tri_total = m.sum() - m[np.arange(75) * (np.arange(75) + 1) // 2 + np.arange(75)].sum() // 2
    assert abs(int(tri_total) - cnt) <= 2  # predicate rounding differs from numpy's order
    assert ps[ps_off[0] + 1] == 299  # every bonded neighbour is in contact
    assert orc.overlaps(x) >= 0


def _golden():
    return sorted(glob.glob(os.path.join(GOLDEN, "ccp_*.npz")))


@pytest.mark.parametrize("path", _golden(), ids=os.path.basename)
def test_oracle_matches_reference_forces(orc, path):
    """The FP64 oracle reproduces the reference's own calc_bf + calc_cf +
    calc_srf (run on a GPU from the reference sources) within the reference's
    FP32 rounding."""
    g = np.load(path)
    n = len(g["xyz"])
    heads = list(orc.CHR_LIM[:12]) if n == orc.N_DEF else [0]
    fl = orc.flags_from_types(g["pt"], heads)
    geo = orc.geo_vec(*[float(v) for v in g["geo"]], csl=2.0)
    f64, sa = orc.forces(g["xyz"], fl, g["lbs"], orc.ccp_ff(), geo, with_abs=True, cells=True)
    # ccp's FP32 forms (1 - l0/d, R/d - 1, the unfactored Wang-Frenkel
    # polynomial) carry up to ~1.5e-4 of rounding relative to this scale
    d = np.linalg.norm(g["f_dst"].astype(np.float64) - f64, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f64, axis=1), 0.1 * sa), 1.0)
    assert (d / scale).max() < 3e-4
    if "f_icg" in g:
        fi, si = orc.forces(g["xyz"], fl, g["lbs"], orc.ccp_ff(), geo, mode=orc.MODE_ICG,
                            with_abs=True, cells=True)
        d = np.linalg.norm(g["f_icg"].astype(np.float64) - fi, axis=1)
        scale = np.maximum(np.maximum(np.linalg.norm(fi, axis=1), 0.1 * si), 1.0)
        assert (d / scale).max() < 3e-4


@pytest.mark.parametrize("path", _golden(), ids=os.path.basename)
def test_oracle_matches_reference_contact_map(orc, path):
    """Contact counts of the oracle reproduce the reference's calc_cm values
    exactly: value = 1000 (count + self) / (copies * 16)."""
    g = np.load(path)
    n = len(g["xyz"])
    ncop = 2 if n == orc.N_DEF else 1
    copy_len = n // ncop
    cms = copy_len // 4
    heads = list(orc.CHR_LIM[:12]) if n == orc.N_DEF else [0]
    m, ps, ps_off = orc.contacts(g["xyz"], 2.0, cms, cms * 4, copy_len, ncop, heads)
    b = np.arange(cms)
    cnt = m.astype(np.int64)
    cnt[b * (b + 1) // 2 + b] += 4 * ncop
    val = (np.float32(1000.0) * cnt.astype(np.float32)) / np.float32(ncop * 16)
    ref = np.zeros(int(g["cm_len"]), np.float32)
    ref[g["cm_idx"]] = g["cm_val"]
    assert np.array_equal(val.astype(np.float32), ref)


@pytest.mark.parametrize("path", _golden(), ids=os.path.basename)
def test_oracle_cell_keys_match_reference(orc, path):
    """The reference's calc_indexes keys (sugrid.cu:15-35) restated."""
    g = np.load(path)
    x = g["xyz"].astype(np.float32)
    cps = int(g["cps"])
    ir = np.floor(x / np.float32(2.0)).astype(np.int64)
    key = (cps // 2) * (1 + cps + cps * cps) + ir[:, 0] + ir[:, 1] * cps + ir[:, 2] * cps * cps
    assert np.array_equal(key.astype(np.uint32), g["cell_keys"])
