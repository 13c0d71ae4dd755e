"""The persistent per-system path (tfm_gb300/csrc/persist.cuh, `persistent 1`):
one CTA per system advances it by a frame of Heun steps in shared memory.
It must step exactly as the graph path does, up to the FP32 summation order
of the pair forces: the same forces, the same Philox noise, the same
displacement cap and relaxation. The oracle trajectory tests of
test_gpu_parity.py run on both paths; here the two paths are compared on
batches, from identical starts."""
import numpy as np
import pytest

from helpers import ccp_params

pytestmark = pytest.mark.gpu

SIZES = [300, 1024, 2048, 2800]


def _pair(text, sizes, seeds, radii=None):
    from tfm_gb300.ccpgpu import Batch

    a = Batch(text + "persistent 0\n", sizes, seeds=seeds, radii=radii)
    b = Batch(text + "persistent 1\n", sizes, seeds=seeds, radii=radii)
    assert a.info().persistent_reach == 0 and b.info().persistent_reach in (1, 2)
    a.generate_initial_condition()
    b.set_types(a.types())
    b.set_lbs(a.lbs())
    b.set_positions(a.positions())
    return a, b


@pytest.mark.parametrize("preset", ["baseline", "ccp"])
def test_persistent_steps_as_the_graph_path(engine_lib, preset):
    radii = None
    if preset == "baseline":
        text = "force_field baseline\ncontact_bins 64\n"
    else:  # ccp's field, each system at chromatin volume fraction 0.2, 40 sites each
        text = "number_of_particles 02048\nnucleus_radius %.6f\nnumber_of_lbs 00040\n" \
               "contact_bins 64\n" % ccp_params(2048)[1]
        radii = [ccp_params(n)[1] for n in SIZES]
    a, b = _pair(text, SIZES, [11, 12, 13, 14], radii)
    # one step: the two differ only by the summation order of the pair forces
    a.run_steps(1)
    b.run_steps(1)
    d1 = np.abs(a.positions() - b.positions()).max()
    assert d1 < 1e-5, d1
    # 300 more steps with contact observation every 100 (FP32 differences grow
    # through the chaotic dynamics, as between any two summation orders)
    a.reset_observables()
    b.reset_observables()
    a.run_steps(300, observe_every=100)
    b.run_steps(300, observe_every=100)
    d = np.abs(a.positions() - b.positions()).max()
    assert d < 1e-3, d
    assert a.info().step == b.info().step == 301
    assert a.info().frames_observed == b.info().frames_observed
    for s in range(len(SIZES)):
        ca, cb = a.contact_counts(s).sum(), b.contact_counts(s).sum()
        assert abs(int(ca) - int(cb)) <= 0.01 * ca, (s, ca, cb)
    for h in (a, b):
        flags, _ = h.error_flags()
        assert not flags[:4].any(), flags
        h.close()


def test_persistent_relaxation_and_fallback(engine_lib):
    from tfm_gb300.ccpgpu import Batch

    # the relaxation (soft repulsion mode) also runs in the persistent kernel
    b = Batch("force_field baseline\ncontact_bins 64\npersistent 1\n", SIZES, seeds=[1, 2, 3, 4])
    assert b.info().persistent_reach > 0
    b.generate_initial_condition()
    assert all(v == 0 for v in b.overlaps()), b.overlaps()
    b.run_steps(100)
    assert np.isfinite(b.positions()).all()
    b.close()
    # a system that does not fit one CTA's shared memory keeps the graph path
    big = Batch("force_field baseline\ncontact_bins 64\npersistent 1\n", [8192], seeds=[5])
    assert big.info().persistent_reach == 0
    big.close()
