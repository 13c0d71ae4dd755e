"""Tests of the contact-map surrogate (include/ccpgpu_surrogate.h).

CPU: the library exports every declared symbol and rejects bad
configurations before touching the GPU; the oracle's convolution agrees with
torch's own conv1d/conv2d, and its gradients with finite differences.
GPU: each tensor-core layer (convolution with its fused epilogue, weight and
bias gradients) against the oracle on the same BF16 inputs; the whole network
(forward maps, loss, every parameter's gradient) against the oracle; AdamW
training lowers the loss.

Tolerances. Layers: the GPU accumulates in FP32 and rounds the output to
BF16, so an output may differ from the FP64 oracle rounded to BF16 by one
BF16 step (2^-8 relative) where the FP32 sum lands next to a rounding
boundary (at most one step, on under 1 % of the values); weight gradients (FP32 sums over every pixel) agree within 1e-4 of
the largest entry. Network: forward maps within 2e-2 relative (a one-step
BF16 difference in an early activation propagates), gradients per tensor
within 3e-2 relative L2 and cosine >= 0.999 (the GPU feeds BF16-rounded
gradients to the tensor cores; the oracle's backward is exact FP64).
"""
import ctypes as C
import os
import re
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "ccpgpu_surrogate.h")).read()
    return sorted(set(re.findall(r"\b(ccpsur_[a-z0-9_]+)\s*\(", src)))


def test_surrogate_symbols_exported(engine_lib):
    from tfm_gb300 import surrogate

    decl = _declared()
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(engine_lib, name), name
    assert set(decl) == set(surrogate.SYMBOLS)


@pytest.mark.parametrize("text,msg", [
    ("seq_len 1000\n", "seq_len must be a positive multiple of 128"),
    ("bins 100\n", "bins must be a multiple of 128 dividing seq_len"),
    ("seq_len 1024\nbins 384\n", "bins must be a multiple of 128 dividing seq_len"),
    ("enc_width 96\n", "enc_width must be 128"),
    ("head_width 32\n", "head_width must be 64"),
    ("enc_kernel 4\n", "enc_kernel must be 1, 3 or 5"),
    ("head_layers 3\ndilations 1,2\n", "dilations must list one value per head layer"),
    ("batch 0\n", "batch out of range"),
])
def test_surrogate_config_errors(engine_lib, text, msg):
    from tfm_gb300 import ccpgpu, surrogate

    surrogate.load()
    h = C.c_void_p()
    rc = engine_lib.ccpsur_create(text.encode(), 0, C.byref(h))
    assert rc == ccpgpu.ERR_PARAM
    assert engine_lib.ccpgpu_last_error().decode() == msg
    assert not h


def test_oracle_conv_matches_torch_conv():
    """The oracle's tap convolution is torch's conv2d with dilation and 'same'
    zero padding (and conv1d for the encoder's row taps)."""
    import torch
    import torch.nn.functional as F

    from oracle import surrogate_oracle as so

    rng = np.random.default_rng(1)
    x = torch.as_tensor(rng.standard_normal((2, 9, 11, 5)))
    for d in (1, 2, 4):
        W = torch.as_tensor(rng.standard_normal((9, 3, 5)))
        got = so.conv_taps(x, W, so.head_taps(d))
        k = W.reshape(3, 3, 3, 5).permute(2, 3, 0, 1)  # [co][ci][kh][kw]
        ref = F.conv2d(x.permute(0, 3, 1, 2), k, padding=d, dilation=d).permute(0, 2, 3, 1)
        assert torch.allclose(got, ref, atol=1e-10)
    x1 = torch.as_tensor(rng.standard_normal((2, 1, 17, 4)))
    W1 = torch.as_tensor(rng.standard_normal((5, 6, 4)))
    got = so.conv_taps(x1, W1, so.enc_taps(5))
    ref = F.conv1d(x1[:, 0].permute(0, 2, 1), W1.permute(1, 2, 0), padding=2).permute(0, 2, 1)
    assert torch.allclose(got[:, 0], ref, atol=1e-10)


def test_oracle_gradient_matches_finite_differences():
    import torch

    from oracle import surrogate_oracle as so

    cfg = so.config(seq_len=128, bins=128, enc_layers=2, head_layers=2, enc_kernel=3,
                    dilations=(1, 2))
    rng = np.random.default_rng(2)
    flat = rng.standard_normal(so.n_params(cfg)) * 0.05
    flat[-1] = -3.0  # output bias: predictions stay below the clamp at probability 1
    types = rng.integers(0, 2, (1, 128))
    lad = (rng.random((1, 128)) < 0.1).astype(np.uint8)
    maps = rng.random((1, 128, 128)) * 0.1
    maps = 0.5 * (maps + maps.transpose(0, 2, 1))
    maps[0, 3, 5] = maps[0, 5, 3] = 0.0  # a zero count

    # exact FP64 graph (no BF16 rounding) for the finite-difference check
    orig = so.bf16
    so.bf16 = lambda x: x
    try:
        loss, g = so.loss_and_grads(flat, cfg, types, lad, maps, maps)
        for k in rng.choice(flat.size, 12, replace=False):
            e = np.zeros_like(flat)
            h = 1e-6
            e[k] = h
            lp, _ = so.loss_and_grads(flat + e, cfg, types, lad, maps, maps)
            lm, _ = so.loss_and_grads(flat - e, cfg, types, lad, maps, maps)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])
    finally:
        so.bf16 = orig
    assert np.isfinite(loss)


# ---------------------------------------------------------------- GPU

def _rand_bf16(rng, shape, scale=1.0):
    from tfm_gb300 import surrogate

    return surrogate.to_bf16(rng.standard_normal(shape).astype(np.float32) * scale)


def _ref_conv(x, w, taps, bias, relu, resid):
    import torch

    from oracle import surrogate_oracle as so
    from tfm_gb300 import surrogate

    xt = torch.as_tensor(surrogate.from_bf16(x).astype(np.float64))
    wt = torch.as_tensor(surrogate.from_bf16(w).astype(np.float64))
    pre = so.conv_taps(xt, wt, taps)
    if bias is not None:
        pre = pre + torch.as_tensor(bias.astype(np.float64))
    out = torch.relu(pre) if relu else pre
    if resid is not None:
        out = out + torch.as_tensor(surrogate.from_bf16(resid).astype(np.float64))
    return pre.numpy(), out.numpy()


CONV_CASES = [
    # (B, H, W, cin, cout, taps, relu, resid)
    (2, 4, 128, 64, 64, "head2", True, True),
    (1, 9, 128, 64, 64, "head8", True, True),
    (2, 1, 256, 128, 128, "enc5", True, True),
    (2, 1, 256, 64, 128, "enc5", True, False),
    (2, 1, 256, 128, 128, "one", False, False),
    (2, 3, 256, 64, 64, "head1neg", False, False),
    # several tiles per CTA: both MMA-issuing warps, their window rings and
    # the TMEM accumulators wrap around
    (4, 128, 256, 64, 64, "head2", True, True),
    (8, 64, 256, 128, 128, "enc5", True, False),
]


def _taps(name):
    from oracle import surrogate_oracle as so

    if name.startswith("head"):
        d = int(name[4]) if name[4].isdigit() else 1
        t = so.head_taps(d)
        return [(-a, -b) for a, b in t] if name.endswith("neg") else t
    if name == "enc5":
        return so.enc_taps(5)
    return [(0, 0)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CONV_CASES)
def test_conv_layer_matches_oracle(engine_lib, case):
    from tfm_gb300 import surrogate

    B, H, W, cin, cout, tname, relu, use_resid = case
    taps = _taps(tname)
    rng = np.random.default_rng(zlib.crc32(repr(case).encode()))
    x = _rand_bf16(rng, (B, H, W, cin))
    w = _rand_bf16(rng, (len(taps), cout, cin), 1.0 / np.sqrt(cin * len(taps)))
    bias = (rng.standard_normal(cout) * 0.1).astype(np.float32)
    resid = _rand_bf16(rng, (B, H, W, cout)) if use_resid else None
    out, mask = surrogate.conv_bf16(x, w, taps, bias=bias, relu=relu, resid=resid, want_mask=True)
    pre, ref = _ref_conv(x, w, taps, bias, relu, resid)
    got = surrogate.from_bf16(out).astype(np.float64)
    ref_b = surrogate.from_bf16(surrogate.to_bf16(ref.astype(np.float32))).astype(np.float64)
    err = np.abs(got - ref_b)
    # one BF16 step of the value: 2^(floor(log2 |ref|) - 7), plus 2e-5 for
    # outputs near zero that cancel (a sum of O(1) terms, or a pre-activation
    # of ~1.5 against an equal residual), where the FP32 sum's own rounding
    # (~1e-6) exceeds the step
    ulp = 2.0 ** (np.floor(np.log2(np.maximum(np.abs(ref), 1e-30))) - 7)
    assert np.all(err <= ulp + 2e-5), (err.max(), np.argmax(err - ulp))
    assert np.count_nonzero(err) <= 0.01 * err.size
    # mask bits: pre-activation > 0, except where the FP32 and FP64 sums straddle 0
    bits = np.unpackbits(mask.view(np.uint8), bitorder="little").reshape(B, H, W, cout)
    want = (pre > 0)
    differ = bits.astype(bool) != want
    assert np.all(np.abs(pre[differ]) < 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [
    (2, 4, 128, 64, 64, "head2"),
    (2, 1, 256, 128, 128, "enc5"),
    (2, 1, 256, 64, 128, "enc5"),
    (2, 1, 256, 128, 128, "one"),
    (1, 5, 128, 64, 64, "head8"),
    (4, 64, 256, 64, 64, "head2"),
])
def test_wgrad_layer_matches_oracle(engine_lib, case):
    from oracle import surrogate_oracle as so
    from tfm_gb300 import surrogate

    B, H, W, cin, cout, tname = case
    taps = _taps(tname)
    rng = np.random.default_rng(zlib.crc32(repr(case).encode()))
    x = _rand_bf16(rng, (B, H, W, cin))
    dy = _rand_bf16(rng, (B, H, W, cout))
    dw, db = surrogate.wgrad_bf16(x, dy, taps)
    xf = surrogate.from_bf16(x).astype(np.float64)
    yf = surrogate.from_bf16(dy).astype(np.float64)
    ref = np.zeros((len(taps), cout, cin))
    for t, (dh, dwo) in enumerate(taps):
        sh = np.zeros_like(xf)
        h0, h1 = max(0, -dh), min(H, H - dh)
        w0, w1 = max(0, -dwo), min(W, W - dwo)
        if h0 < h1 and w0 < w1:
            sh[:, h0:h1, w0:w1] = xf[:, h0 + dh:h1 + dh, w0 + dwo:w1 + dwo]
        ref[t] = np.einsum("bhwo,bhwc->oc", yf, sh)
    scale = np.abs(ref).max()
    assert np.abs(dw - ref).max() <= 1e-4 * scale, np.abs(dw - ref).max() / scale
    refb = yf.sum(axis=(0, 1, 2))
    assert np.abs(db - refb).max() <= 1e-4 * np.abs(refb).max()


SMALL = "seq_len 256\nbins 128\nbatch 2\nenc_layers 3\nhead_layers 2\ndilations 1,4\n"


def _small_problem(seed):
    from tfm_gb300 import surrogate

    types, lad, _ = surrogate.make_sequences(4, 256, seed)
    rng = np.random.default_rng(seed)
    i = np.arange(128)
    base = 1.0 / (1.0 + np.abs(i[:, None] - i[None, :])) ** 1.2
    maps = np.empty((4, 128, 128), np.float32)
    for k in range(4):
        a = (types[k].reshape(128, 2).mean(1) < 0.5).astype(np.float64)
        m = 0.5 * base * (1.0 + 0.5 * np.outer(a, a)) * (1.0 + 0.05 * rng.random((128, 128)))
        maps[k] = 0.5 * (m + m.T)
    return types, lad, maps


def _cfg_small():
    from oracle import surrogate_oracle as so

    return so.config(seq_len=256, bins=128, batch=2, enc_layers=3, head_layers=2, dilations=(1, 4))


@pytest.mark.gpu
def test_network_forward_matches_oracle(engine_lib):
    from oracle import surrogate_oracle as so
    from tfm_gb300 import surrogate

    types, lad, maps = _small_problem(3)
    with surrogate.Surrogate(SMALL, seed=5) as net:
        p = net.params()
        # make the output depend on the input: larger output weights
        cfg = _cfg_small()
        lay = so.layout(cfg)
        off = sum(int(np.prod(s)) for n, s in lay[:-2])
        p[off:off + 64] = np.random.default_rng(0).standard_normal(64) * 0.5
        net.set_params(p)
        got = net.predict(types[:3], lad[:3])
        assert net.error_flags() == 0
    ref = so.predict(p.astype(np.float64), cfg, types[:3], lad[:3])
    ly_g, ly_r = np.log(got), np.log(ref)
    assert np.abs(ly_g - ly_r).max() <= 2e-2 * max(1.0, np.abs(ly_r).max())


@pytest.mark.gpu
def test_full_size_forward_matches_oracle(engine_lib):
    """The default network (1024 beads, 256 bins, 8 encoder and 6 head
    layers) on two sequences: every convolution runs over several tiles per
    CTA, as in training and screening, and the maps equal the oracle's."""
    from oracle import surrogate_oracle as so
    from tfm_gb300 import surrogate

    types, lad, _ = surrogate.make_sequences(2, 1024, 17)
    cfg = so.config()
    with surrogate.Surrogate("", seed=9) as net:
        p = net.params()
        lay = so.layout(cfg)
        off = sum(int(np.prod(s)) for n, s in lay[:-2])
        p[off:off + 64] = np.random.default_rng(2).standard_normal(64) * 0.5
        net.set_params(p)
        got = net.predict(types, lad)
        assert net.error_flags() == 0
    ref = so.predict(p.astype(np.float64), cfg, types, lad)
    ly_g, ly_r = np.log(got), np.log(ref)
    assert np.abs(ly_g - ly_r).max() <= 2e-2 * max(1.0, np.abs(ly_r).max())


@pytest.mark.gpu
def test_network_gradients_match_oracle(engine_lib):
    from oracle import surrogate_oracle as so
    from tfm_gb300 import surrogate

    types, lad, maps = _small_problem(4)
    cfg = _cfg_small()
    with surrogate.Surrogate(SMALL, seed=6) as net:
        p = net.params()
        p[-65:-1] = np.random.default_rng(1).standard_normal(64) * 0.5
        net.set_params(p)
        net.set_dataset(types, lad, maps)
        p = net.params()  # the dataset sets the output bias
        rows = np.array([2, 0], np.int32)
        loss = net.loss_grad(rows)
        g = net.grads()
        assert net.error_flags() == 0
    lref, gref = so.loss_and_grads(p.astype(np.float64), cfg, types[rows], lad[rows], maps[rows], maps)
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    off = 0
    worst = []
    for name, shape in so.layout(cfg):
        n = int(np.prod(shape))
        a, b = g[off:off + n].astype(np.float64), gref[off:off + n]
        off += n
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.abs(a).max() < 1e-6, name  # zero-padded input channels
            continue
        rel = np.linalg.norm(a - b) / nb
        cos = float(a @ b) / (np.linalg.norm(a) * nb)
        worst.append((rel, name))
        assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos)


@pytest.mark.gpu
def test_training_lowers_the_loss(engine_lib):
    from tfm_gb300 import surrogate

    types, lad, maps = _small_problem(5)
    with surrogate.Surrogate(SMALL + "lr 3e-3\n", seed=7) as net:
        net.set_dataset(types, lad, maps)
        rows = np.array([0, 1], np.int32)
        first = net.loss_grad(rows)
        for it in range(60):
            net.train_step(np.array([(2 * it) % 4, (2 * it + 1) % 4], np.int32), want_loss=False)
        last = net.loss_grad(rows)
        assert net.info().step == 60
        assert net.error_flags() == 0
    assert last < 0.5 * first, (first, last)
