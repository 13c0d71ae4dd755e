"""The allocation-free force entry point (ccpgpu_forces_noalloc).

It exists for callers that cannot call cudaMalloc when they need forces (a
host whose memory manager owns all device memory, or a loop that must not
take the device synchronisation of cudaMalloc/cudaFree). Its scratch is one
fixed static device array shared by every call, so this test calls it several
times in a row on different systems (one whose chain count does not divide
its bead count), checks each result against the allocating entry point,
ccpgpu_compute_forces, within the force tolerance of the parity tests, and
reads each call's device flags. The file sorts last so a run that stops at
the first failure has already run every other test; it also passes alone in a
fresh process.
"""
import numpy as np
import pytest

from helpers import at_cutoff, baseline_params, ccp_params

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5


def _reference(orc, text, seed, heads, ff, csl, preset):
    from tfm_gb300.ccpgpu import ChrSim

    sim = ChrSim(text + "number_of_lbs 0\n", seed=seed)
    sim.generate_initial_condition()
    x, pt = sim.positions(), sim.types()
    si = sim.system_info(0)
    fl = orc.flags_from_types(pt, heads, preset)
    geo = orc.geo_vec(si.nucleus_radius, csl=csl)
    f64, sa = orc.forces(x, fl, np.zeros((0, 3), np.float32), ff, geo, with_abs=True, cells=True)
    edge = at_cutoff(x, fl, np.zeros((0, 3)), ff)
    return x, pt, si.nucleus_radius, sim.forces(), f64, sa, edge


def _bound(f, f_ref, sa, skip=None):
    d = np.linalg.norm(np.asarray(f, np.float64) - np.asarray(f_ref, np.float64), axis=1)
    scale = np.maximum(np.maximum(np.linalg.norm(f_ref, axis=1), 0.1 * sa), 1.0)
    e = d / scale
    return (e[~skip] if skip is not None else e).max()


def test_noalloc_forces_match_compute_forces(engine_lib, orc):
    import torch

    from tfm_gb300 import ccpgpu

    txt, _, _ = ccp_params(2048, laf=0.0)
    cases = [
        (0, 2048, 1, _reference(orc, txt, 3, [0], orc.ccp_ff(), 2.0, "ccp")),
        (1, 3000, 3, _reference(orc, baseline_params(3000, "number_of_chains 3\n"), 5,
                                [0, 1000, 2000], orc.baseline_ff(), 2.5, "baseline")),
        # 7 chains do not divide 3001 beads: heads at c * 428, the last chain
        # takes 433 beads, as the allocating engine places them
        (1, 3001, 7, _reference(orc, baseline_params(3001, "number_of_chains 7\n"), 6,
                                [c * 428 for c in range(7)], orc.baseline_ff(), 2.5,
                                "baseline")),
    ]
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    # three systems, then the first again: each call must not see the previous one
    for preset, n, nch, (x, pt, R, f_alloc, f64, sa, edge) in cases + cases[:1]:
        d_x = torch.tensor(x, device=dev)
        d_t = torch.tensor(pt, device=dev)
        d_f = torch.full((n, 3), float("nan"), dtype=torch.float32, device=dev)
        rc = ccpgpu.forces_noalloc(preset, n, nch, R, d_x.data_ptr(), d_t.data_ptr(),
                                   d_f.data_ptr(), stream.cuda_stream)
        assert rc == ccpgpu.OK, ccpgpu.last_error()
        torch.cuda.synchronize()
        f = d_f.cpu().numpy()
        assert np.isfinite(f).all()
        # the two paths run different pair kernels: at a truncation cutoff their
        # FP32 distances may also fall on opposite sides
        assert _bound(f, f_alloc, sa, skip=edge) <= FORCE_RTOL
        # beads within FP32 rounding of a jump of the truncated potential are
        # held to the jump's size (see helpers.at_cutoff)
        assert _bound(f, f64, sa, skip=edge) <= FORCE_RTOL
        assert _bound(f, f64, sa) <= 1e-2
        rc, flags = ccpgpu.noalloc_error_flags(stream.cuda_stream)
        assert rc == ccpgpu.OK and not flags.any(), (rc, flags)

    # device flags of a call are readable: a bead outside the nucleus's grid
    # is clamped and flagged, a non-finite position is a state error
    preset, n, nch, (x, pt, R, *_rest) = cases[0]
    for bad, want_rc, flag in ((3.0 * R, ccpgpu.OK, 1), (float("nan"), ccpgpu.ERR_STATE, 0)):
        xb = np.array(x, np.float32)
        xb[n // 2, 0] = bad
        d_x = torch.tensor(xb, device=dev)
        d_t = torch.tensor(pt, device=dev)
        d_f = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        rc = ccpgpu.forces_noalloc(preset, n, nch, R, d_x.data_ptr(), d_t.data_ptr(),
                                   d_f.data_ptr(), stream.cuda_stream)
        assert rc == ccpgpu.OK, ccpgpu.last_error()
        rc, flags = ccpgpu.noalloc_error_flags(stream.cuda_stream)
        assert rc == want_rc and flags[flag] == 1, (bad, rc, flags)

    # sizes beyond the scratch are refused, not truncated
    big = ccpgpu.NOALLOC_MAX_BEADS + 1
    d_x = torch.zeros((big, 3), dtype=torch.float32, device=dev)
    d_t = torch.zeros(big, dtype=torch.int32, device=dev)
    d_f = torch.zeros((big, 3), dtype=torch.float32, device=dev)
    rc = ccpgpu.forces_noalloc(1, big, 1, 40.0, d_x.data_ptr(), d_t.data_ptr(), d_f.data_ptr(),
                               stream.cuda_stream)
    assert rc == ccpgpu.ERR_ARG
    assert "no-allocation" in ccpgpu.last_error()
    # a nucleus whose grid cannot fit, or that is not finite, is refused
    for radius in (1e6, float("inf")):
        rc = ccpgpu.forces_noalloc(1, 2048, 1, radius, d_x.data_ptr(), d_t.data_ptr(),
                                   d_f.data_ptr(), stream.cuda_stream)
        assert rc == ccpgpu.ERR_ARG, radius
