"""GPU parity of the engine (through the C ABI) against the FP64 oracle and the
reference's own kernels (golden fixtures made by tests/golden/make_golden.py).

Force tolerance: per bead, |F_gpu - F_64| <= 1e-5 * max(|F_64|, 0.1 * S, 1)
where S is the sum of the magnitudes of the bead's force terms (bonds, angles,
pairs, wall, lamina sites) and 1 is one kT/sigma. For beads whose terms do not
cancel (|F| >= 0.1 S) and whose force is not below 1 kT/sigma this is the plain
1e-5 relative bound; where the terms cancel, no FP32 sum can hold a bound
relative to the small remainder, and the bound is relative to the terms; and a
bead whose every term is below 1 kT/sigma (a relaxed start: bonds at l_0, pairs
at the potential's zero) is held to 1e-5 kT/sigma.
"""
import glob
import os

import numpy as np
import pytest

from helpers import at_cutoff, baseline_params, ccp_params, force_errors

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORCE_RTOL = 1e-5


def _force_ok(fg, f64, sa, skip=None):
    d = np.linalg.norm(np.asarray(fg, np.float64) - f64, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f64, axis=1), 0.1 * sa), 1.0)
    e = d / scale
    return (e[~skip] if skip is not None else e).max()




@pytest.fixture(scope="module")
def ccp_sim(engine_lib):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(2048, laf=0.3)
    sim = ChrSim(txt + "steps_per_frame 256\n", seed=7)
    sim.generate_initial_condition()
    return sim, R


@pytest.fixture(scope="module")
def base_sim(engine_lib):
    from tfm_gb300.ccpgpu import ChrSim

    sim = ChrSim(baseline_params(2048, "number_of_chains 4\nsteps_per_frame 200\n"), seed=11)
    sim.generate_initial_condition()
    return sim


def _oracle_forces(orc, sim, ff, csl, heads):
    si = sim.system_info(0)
    fl = orc.flags_from_types(sim.types(), heads,
                              "ccp" if sim.info().preset == 0 else "baseline")
    geo = orc.geo_vec(si.nucleus_radius, si.opening_radius, si.bleb_radius, csl)
    return orc.forces(sim.positions(), fl, sim.lbs(), ff, geo, with_abs=True, cells=True), fl, geo


def test_initial_condition_has_no_overlaps(ccp_sim, orc):
    sim, R = ccp_sim
    x = sim.positions()
    assert np.isfinite(x).all()
    assert orc.overlaps(x) == 0
    assert int(sim.overlaps()[0]) == 0
    assert np.linalg.norm(x, axis=1).max() < R


@pytest.mark.parametrize("steps", [0, 2000])
def test_forces_ccp_match_fp64_oracle(ccp_sim, orc, steps):
    sim, R = ccp_sim
    if steps:
        sim.run_steps(steps)
    (f64, sa), fl, geo = _oracle_forces(orc, sim, orc.ccp_ff(), 2.0, [0])
    fg = sim.forces()
    edge = at_cutoff(sim.positions(), fl, sim.lbs(), orc.ccp_ff())
    err = _force_ok(fg, f64, sa, skip=edge)
    rel, scaled = force_errors(fg, f64, sa)
    print("ccp forces: bound %.3g (%d beads at a cutoff)  rel(|F|>=1e-3S) %.3g  |dF|/S %.3g"
          % (err, edge.sum(), rel, scaled))
    assert err <= FORCE_RTOL
    assert _force_ok(fg, f64, sa) <= 1e-2


@pytest.mark.parametrize("steps", [0, 2000])
def test_forces_baseline_match_fp64_oracle(base_sim, orc, steps):
    sim = base_sim
    if steps:
        sim.run_steps(steps)
    heads = [0, 512, 1024, 1536]
    (f64, sa), fl, geo = _oracle_forces(orc, sim, orc.baseline_ff(), 2.5, heads)
    fg = sim.forces()
    edge = at_cutoff(sim.positions(), fl, sim.lbs(), orc.baseline_ff())
    err = _force_ok(fg, f64, sa, skip=edge)
    print("baseline forces: bound %.3g (%d beads at a cutoff)" % (err, edge.sum()))
    assert err <= FORCE_RTOL
    assert _force_ok(fg, f64, sa) <= 1e-2


@pytest.mark.parametrize("kernel,half_cells",
                         [(0, False), (1, False), (2, False), (2, True), (3, False), (3, True),
                          (4, False), (4, True)])
def test_pair_kernels_agree(ccp_sim, base_sim, orc, kernel, half_cells):
    """Full-shell thread-per-bead (0), warp-per-cell (1), half-shell (2, 3)
    and typed half-shell (4: A beads and the others in separate grids) pair
    kernels, the half-shell ones also on cells of half the cutoff (5x5x5
    neighbourhood), all meet the force bound, for both presets."""
    from tfm_gb300.ccpgpu import ChrSim

    sim, R = ccp_sim
    txt, _, _ = ccp_params(2048, laf=0.3)
    for ref, text, ff, csl, heads in (
            (sim, txt, orc.ccp_ff(), 2.0, [0]),
            (base_sim, baseline_params(2048, "number_of_chains 4\n"), orc.baseline_ff(), 2.5,
             [0, 512, 1024, 1536])):
        extra = "pair_kernel %d\n" % kernel
        if half_cells:
            extra += "cell_side %r\n" % (csl / 2)
        other = ChrSim(text + extra, seed=7)
        other.set_types(ref.types())
        other.set_lbs(ref.lbs())
        other.set_positions(ref.positions())
        (f64, sa), fl, geo = _oracle_forces(orc, ref, ff, csl, heads)
        edge = at_cutoff(ref.positions(), fl, ref.lbs(), ff)
        fo = other.forces()
        assert _force_ok(fo, f64, sa, skip=edge) <= FORCE_RTOL
        assert _force_ok(fo, f64, sa) <= 1e-2


@pytest.mark.parametrize("kernel,lanes", [(2, 1), (2, 2), (2, 4), (2, 8), (4, 1), (4, 2), (4, 4),
                                          (4, 8)])
def test_pair_lanes_agree(ccp_sim, base_sim, orc, kernel, lanes):
    """The half-shell kernels (one grid, 2; typed layout, 4) with 1, 2, 4 or
    8 lanes per bead (rows dealt to the lanes, partial forces combined by
    shuffles; batches below 16384 beads default to 8) meet the force bound,
    on cells of half the cutoff."""
    from tfm_gb300.ccpgpu import ChrSim

    sim, R = ccp_sim
    txt, _, _ = ccp_params(2048, laf=0.3)
    for ref, text, ff, csl, heads in (
            (sim, txt, orc.ccp_ff(), 2.0, [0]),
            (base_sim, baseline_params(2048, "number_of_chains 4\n"), orc.baseline_ff(), 2.5,
             [0, 512, 1024, 1536])):
        other = ChrSim(text + "pair_kernel %d\npair_lanes %d\ncell_side %r\n"
                       % (kernel, lanes, csl / 2), seed=7)
        other.set_types(ref.types())
        other.set_lbs(ref.lbs())
        other.set_positions(ref.positions())
        (f64, sa), fl, geo = _oracle_forces(orc, ref, ff, csl, heads)
        edge = at_cutoff(ref.positions(), fl, ref.lbs(), ff)
        fo = other.forces()
        assert _force_ok(fo, f64, sa, skip=edge) <= FORCE_RTOL
        assert _force_ok(fo, f64, sa) <= 1e-2


def _golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "ccp_*.npz")))


def _sim_from_golden(path):
    from tfm_gb300.ccpgpu import ChrSim

    g = np.load(path)
    n = len(g["xyz"])
    R_n, R_o, R_b = (float(v) for v in g["geo"])
    txt = ("number_of_particles %d\nnucleus_radius %r\nopening_radius %r\nbleb_radius %r\n"
           "number_of_lbs %d\n" % (n, R_n, R_o, R_b, len(g["lbs"])))
    sim = ChrSim(txt, seed=1)
    sim.set_types(g["pt"])
    sim.set_lbs(g["lbs"])
    sim.set_positions(g["xyz"])
    return sim, g


@pytest.mark.parametrize("path", _golden_cases(), ids=os.path.basename)
def test_forces_match_reference_kernels(engine_lib, orc, path):
    """Engine forces vs the reference's calc_bf + calc_cf + calc_srf run on the
    same positions (both FP32) and vs the FP64 oracle."""
    sim, g = _sim_from_golden(path)
    n = len(g["xyz"])
    heads = list(orc.CHR_LIM[:12]) if n == orc.N_DEF else [0]
    fl = orc.flags_from_types(g["pt"], heads)
    geo = orc.geo_vec(*[float(v) for v in g["geo"]], csl=2.0)
    f64, sa = orc.forces(g["xyz"], fl, g["lbs"], orc.ccp_ff(), geo, with_abs=True, cells=True)
    fg = sim.forces()
    assert _force_ok(fg, f64, sa) <= FORCE_RTOL
    # the reference's FP32 forces are within their own rounding of FP64
    # the reference's own FP32 forces are within its rounding (3e-4) of FP64
    fr = g["f_dst"].astype(np.float64)
    d = np.linalg.norm(fg - fr, axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f64, axis=1), 0.1 * sa), 1.0)
    print(os.path.basename(path), "engine vs reference kernels: %.3g" % (d / scale).max())
    assert (d / scale).max() <= 3e-4


@pytest.mark.parametrize("path", _golden_cases(), ids=os.path.basename)
def test_contact_map_bit_exact_vs_reference(engine_lib, orc, path):
    """Per-frame contact map values 1000 * (count + self) / (copies * 16) equal
    the reference's calc_cm output exactly, and the counts equal the oracle's."""
    sim, g = _sim_from_golden(path)
    n = len(g["xyz"])
    si = sim.system_info(0)
    sim.reset_observables()
    sim.observe()
    cnt = sim.contact_counts(0).astype(np.int64)
    heads = list(orc.CHR_LIM[:12]) if n == orc.N_DEF else [0]
    m, ps, ps_off = orc.contacts(g["xyz"], 2.0, si.contact_bins, si.map_len, si.copy_len,
                                 si.n_copies, heads)
    assert np.array_equal(cnt, m.astype(np.int64))
    nb = si.contact_bins
    px = si.map_len // nb
    diag = np.zeros(len(cnt), np.int64)
    b = np.arange(nb)
    diag[b * (b + 1) // 2 + b] = px * si.n_copies
    val = (np.float32(1000.0) * (cnt + diag).astype(np.float32)) / np.float32(
        si.n_copies * px * px)
    ref = np.zeros(int(g["cm_len"]), np.float32)
    ref[g["cm_idx"]] = g["cm_val"]
    assert np.array_equal(val.astype(np.float32), ref)


@pytest.mark.parametrize("kernel", [2, 4])
def test_contacts_on_half_cells_bit_exact(engine_lib, orc, kernel):
    """Contact counts from the 5x5x5 neighbourhood (cells of half the cutoff)
    equal the oracle's all-pairs counts, with one grid (2) and with the typed
    layout's two grids (4); the run also relaxes and steps with that kernel."""
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(2048)
    sim = ChrSim(txt + "cell_side 1.0\npair_kernel %d\n" % kernel, seed=9)
    sim.generate_initial_condition()
    sim.run_steps(500)
    sim.reset_observables()
    sim.observe()
    si = sim.system_info(0)
    m, ps, ps_off = orc.contacts(sim.positions(), 2.0, si.contact_bins, si.map_len, si.copy_len,
                                 si.n_copies, [0])
    assert np.array_equal(sim.contact_counts(0), m)
    cc, _ = sim.separation_counts(0, 2048)
    assert np.array_equal(cc, ps[:len(cc)])


@pytest.mark.parametrize("path", _golden_cases(), ids=os.path.basename)
def test_separation_observables_vs_reference(engine_lib, orc, path):
    sim, g = _sim_from_golden(path)
    n = len(g["xyz"])
    heads = list(orc.CHR_LIM[:12]) if n == orc.N_DEF else [0]
    sim.reset_observables()
    sim.observe(with_sdist=True)
    lens = np.diff(np.append(heads, n))
    ncop = 2 if n == orc.N_DEF else 1
    nh = len(heads) // ncop
    off = 0
    for c in range(nh):
        L = int(lens[c])
        cnt = np.zeros(L // 2 + 1, np.int64)
        dst = np.zeros(L // 2 + 1, np.float64)
        for k in range(ncop):
            cc, dd = sim.separation_counts(c + k * nh, L)
            cnt += cc
            dst += dd
        s = np.arange(1, L // 2 + 1)
        cp = (np.float32(1000.0) * cnt[1:].astype(np.float32)) / (ncop * (L - s)).astype(np.float32)
        ls = int(g["sd_len"][c])
        ref_cp = g["cp"][off:off + ls]
        ref_sd = g["sd"][off:off + ls].astype(np.float64)
        off += ls
        assert np.array_equal(cp.astype(np.float32), ref_cp)
        sd = dst[1:] / (ncop * (L - s))
        # the reference accumulates d(s) in FP32; the engine in FP64
        assert np.allclose(sd, ref_sd, rtol=1e-3)
        first = heads[c]
        ods = orc.sdist(g["xyz"][first:first + L])
        if ncop == 1:
            assert np.allclose(dst, ods, rtol=2e-5, atol=1e-9)


def test_observables_match_oracle(ccp_sim, orc):
    sim, R = ccp_sim
    sim.reset_observables()
    sim.observe()
    got = sim.observable_sums(0)
    fl = orc.flags_from_types(sim.types(), [0])
    want = orc.observables(sim.positions(), fl, sim.system_info(0).nucleus_radius)
    assert np.allclose(got[:4], want[:4], rtol=1e-9)
    vfull = 4.0 / 3.0 * np.pi * (orc.RCO / 2) ** 3
    assert np.allclose(got[4:], want[4:], rtol=0, atol=2e-5 * vfull * 64)
    # radial density integrates to the bead volume inside the nucleus
    assert abs(got[4 + 128:].sum() - want[4 + 128:].sum()) < 1e-3 * want[4 + 128:].sum()


@pytest.mark.parametrize("persistent", [0, 1])
def test_trajectory_matches_oracle_1000_steps(engine_lib, orc, persistent):
    """Same seed, same Philox stream, same start: 1000 Heun steps on the GPU vs
    the FP64 oracle, on the graph path and on the persistent per-system
    kernel. Stated drift: max |dr| < 2e-3 sigma (FP32 rounding amplified by
    the chaotic dynamics)."""
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(1024, laf=0.3)
    sim = ChrSim(txt + "persistent %d\n" % persistent, seed=1234)
    assert (sim.info().persistent_reach > 0) == bool(persistent)
    sim.generate_initial_condition()
    x0 = sim.positions()
    pt = sim.types()
    lbs = sim.lbs()
    step0 = sim.info().step
    sim.run_steps(1000)
    xg = sim.positions().astype(np.float64)
    fl = orc.flags_from_types(pt, [0])
    geo = orc.geo_vec(sim.system_info(0).nucleus_radius, csl=2.0)
    x64 = orc.run(x0, fl, lbs, orc.ccp_ff(), geo, 1234, step0, 1000, prec=64)
    drift = np.linalg.norm(xg - x64, axis=1)
    rms_step = np.sqrt(3) * orc.ccp_ff()["sd"]
    print("1000-step drift: max %.3g  mean %.3g  (noise rms/step %.3g)" % (
        drift.max(), drift.mean(), rms_step))
    assert drift.max() < 2e-3


@pytest.mark.parametrize("persistent", [0, 1])
def test_trajectory_baseline_matches_oracle_1000_steps(engine_lib, orc, persistent):
    """The same for the baseline force field (Lennard-Jones A-A attraction,
    WCA, lamina sites, the displacement cap) on its default typed pair
    kernel and on the persistent kernel: 1000 Heun steps vs the FP64 oracle,
    max |dr| < 2e-3 sigma."""
    from tfm_gb300.ccpgpu import ChrSim

    sim = ChrSim(baseline_params(1024, "persistent %d\n" % persistent), seed=4321)
    assert (sim.info().persistent_reach > 0) == bool(persistent)
    assert "pair_kernel" not in baseline_params(1024)  # the preset's default (typed)
    sim.generate_initial_condition()
    x0, pt, lbs = sim.positions(), sim.types(), sim.lbs()
    step0 = sim.info().step
    sim.run_steps(1000)
    xg = sim.positions().astype(np.float64)
    fl = orc.flags_from_types(pt, [0], "baseline")
    geo = orc.geo_vec(sim.system_info(0).nucleus_radius, csl=2.5)
    x64 = orc.run(x0, fl, lbs, orc.baseline_ff(), geo, 4321, step0, 1000, prec=64)
    drift = np.linalg.norm(xg - x64, axis=1)
    print("baseline 1000-step drift: max %.3g  mean %.3g" % (drift.max(), drift.mean()))
    assert drift.max() < 2e-3


def test_batch_matches_single_systems(engine_lib):
    from tfm_gb300.ccpgpu import Batch, ChrSim

    txt = "force_field baseline\ncontact_bins 64\n"
    sizes = [1024, 1536, 2048]
    b = Batch(txt, sizes, seeds=[5, 6, 7])
    b.generate_initial_condition()
    x0 = b.positions()
    b.run_steps(200)
    xb = b.positions()
    off = 0
    for k, n in enumerate(sizes):
        s = ChrSim("force_field baseline\nnumber_of_particles %d\ncontact_bins 64\n" % n,
                   seed=5 + k)
        s.generate_initial_condition()
        assert np.array_equal(s.types(), b.types()[off:off + n])
        s.set_positions(x0[off:off + n])
        s.run_steps(200)
        d = np.abs(s.positions() - xb[off:off + n]).max()
        assert d < 1e-3, (k, d)
        off += n


def test_ensemble_split_matches_whole_batch(engine_lib):
    """A fixed ensemble split over two ranks by bead count (each rank's share
    a batch of its own, replicas keeping their seeds) reproduces the whole
    batch: same types and lamina sites, and after 200 steps from the same
    start the same positions to FP32 summation order."""
    from tfm_gb300 import replicas
    from tfm_gb300.ccpgpu import Batch

    txt = "force_field baseline\ncontact_bins 64\n"
    sizes = np.array([1024, 3000, 1536, 2048, 1100], dtype=np.int32)
    seeds = np.arange(len(sizes), dtype=np.uint64) + 21
    b = Batch(txt, sizes, seeds=seeds)
    b.generate_initial_condition()
    x0, pt, lbs = b.positions(), b.types(), b.lbs()
    b.run_steps(200)
    xb = b.positions()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for rank in range(2):
        idx, sz, sd = replicas.local_replicas(sizes, seeds, 2, rank)
        part = Batch(txt, sz, seeds=sd)
        part.generate_initial_condition()
        rows = np.concatenate([np.arange(off[k], off[k + 1]) for k in idx])
        assert np.array_equal(part.types(), pt[rows])
        for j, k in enumerate(idx):
            si, sj = b.system_info(int(k)), part.system_info(j)
            assert np.array_equal(part.lbs()[sj.lbs_offset:sj.lbs_offset + sj.n_lbs],
                                  lbs[si.lbs_offset:si.lbs_offset + si.n_lbs])
        part.set_positions(x0[rows])
        part.run_steps(200)
        d = np.abs(part.positions() - xb[rows]).max()
        assert d < 1e-3, (rank, d)
        part.close()
    b.close()


def test_autotune_keeps_state_and_forces(engine_lib, orc):
    """The autotuner picks a pair kernel, re-grids size classes and picks a
    tile size without changing positions or time, and forces stay within the
    bound afterwards."""
    from tfm_gb300.ccpgpu import Batch

    sizes = [1100, 1500, 2600, 3000, 5000]
    b = Batch("force_field baseline\ncontact_bins 64\n", sizes, seeds=[1, 2, 3, 4, 5])
    b.generate_initial_condition()
    b.run_steps(100)
    x0, step0 = b.positions(), b.info().step
    rep = b.autotune(reps=3)
    assert len(rep["classes"]) == 3 and rep["tile"] in (64, 128, 256)
    assert rep["pair_kernel"] in (2, 4) and len(rep["kernels_tried"]) == 2
    assert rep["lanes"] in (1, 2, 4, 8) and rep["tile"] * rep["lanes"] <= 512
    assert np.array_equal(b.positions(), x0) and b.info().step == step0
    f = b.forces()
    pt, lbs = b.types(), b.lbs()
    for s in range(len(sizes)):
        si = b.system_info(s)
        sl = slice(si.bead_offset, si.bead_offset + si.n_beads)
        fl = orc.flags_from_types(pt[sl], [0], "baseline")
        geo = orc.geo_vec(si.nucleus_radius, csl=2.5)
        ls = lbs[si.lbs_offset:si.lbs_offset + si.n_lbs]
        f64, sa = orc.forces(x0[sl], fl, ls, orc.baseline_ff(), geo, with_abs=True, cells=True)
        edge = at_cutoff(x0[sl], fl, ls, orc.baseline_ff())
        assert _force_ok(f[sl], f64, sa, skip=edge) <= FORCE_RTOL
        if edge.any():  # at most the force jump of the truncated potential
            assert _force_ok(f[sl], f64, sa) <= 1e-2
    b.run_steps(200)
    assert np.isfinite(b.positions()).all()


def test_checkpoint_roundtrip_and_resume(ccp_sim, engine_lib):
    from tfm_gb300.ccpgpu import ChrSim

    sim, R = ccp_sim
    ck = sim.checkpoint()
    n = sim.n_beads
    n_l = sim.info().n_lbs
    assert len(ck) == 8 + 16 * n + 12 * n_l
    txt, _, _ = ccp_params(2048, laf=0.3)
    other = ChrSim(txt + "steps_per_frame 256\n", seed=7)
    other.load_checkpoint_bytes(ck)
    assert np.array_equal(other.positions(), sim.positions())
    assert np.array_equal(other.types(), sim.types())
    assert np.array_equal(other.lbs(), sim.lbs())
    assert other.checkpoint() == ck


def test_run_simulation_writes_trr_frames(engine_lib, tmp_path):
    from tfm_gb300.ccpgpu import ChrSim

    txt, R, n_l = ccp_params(512)
    sim = ChrSim(txt + "frames_per_file 3\nsteps_per_frame 64\n", seed=3)
    sim.generate_initial_condition()
    frames = []
    with open(tmp_path / "t.trr", "wb") as f:
        sim.run_simulation(f, on_frame=lambda i, t, x: frames.append((i, t, x)))
    data = (tmp_path / "t.trr").read_bytes()
    fsz = 72 + 12 * 512
    assert len(data) == 3 * fsz
    hdr = np.frombuffer(data[:72], np.uint32)
    assert hdr[0] == 1993 and hdr[13] == 512 and hdr[14] == 1
    assert [f[0] for f in frames] == [1, 2, 3]
    assert np.isclose(frames[-1][1], 3 * 64 / 2048)
    assert np.array_equal(np.frombuffer(data[-12 * 512:], np.float32).reshape(512, 3),
                          sim.positions())
    assert sim.info().frame_index == 3


def test_nan_positions_are_reported(engine_lib):
    from tfm_gb300.ccpgpu import CcpError, ChrSim, ERR_STATE

    txt, R, n_l = ccp_params(512)
    sim = ChrSim(txt, seed=3)
    sim.generate_initial_condition()
    x = sim.positions()
    x[100, 1] = np.nan
    sim.set_positions(x)
    with pytest.raises(CcpError) as e:
        sim.run_steps(2)
    assert e.value.code == ERR_STATE
