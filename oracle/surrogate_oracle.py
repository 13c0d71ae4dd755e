"""CPU oracle of the contact-map surrogate network — TEST INFRASTRUCTURE.

Only tests/ and bench.py's checks import this module; the library never does.
The network has no counterpart in the reference (ccp only simulates and
analyses contact maps, Program/src/chrana.cu:48-84), so this oracle restates
the network defined in include/ccpgpu_surrogate.h in torch on the CPU in
FP64, with autograd for the gradients. The rounding of the GPU path is
mirrored where it changes values: convolution weights are used as BF16, and
every stored activation (encoder outputs, pooled features, projections, pair
features, head outputs) is rounded to BF16 in the forward pass. In the
backward pass the rounding is the identity (straight-through), so the oracle's
gradients are the exact FP64 gradients of the rounded forward graph; the GPU
additionally rounds the masked gradients it feeds to the tensor cores to BF16.

The flat parameter vector follows ccpsur_get_params: per encoder layer W
[taps][128][cin] then b [128] (cin = 64 for the first layer), the projection
W [1][128][128] and b [128], E [bins][64], per head layer W [9][64][64] and
b [64], then w_out [64] and b_out [1].
"""
import numpy as np
import torch

DEFAULTS = dict(seq_len=1024, bins=256, batch=32, enc_layers=8, enc_width=128, enc_kernel=5,
                head_layers=6, head_width=64, dilations=(1, 2, 4, 8, 1, 2))
YHAT_MAX = 0.0


def config(**kw):
    c = dict(DEFAULTS)
    c.update(kw)
    if "dilations" not in kw:
        d = DEFAULTS["dilations"]
        c["dilations"] = tuple(d[l % len(d)] for l in range(c["head_layers"]))
    return c


def layout(cfg):
    """(name, shape) of every parameter tensor in flat-vector order."""
    k, M = cfg["enc_kernel"], cfg["bins"]
    out = []
    for l in range(cfg["enc_layers"]):
        out.append(("enc%d.W" % l, (k, 128, 64 if l == 0 else 128)))
        out.append(("enc%d.b" % l, (128,)))
    out.append(("proj.W", (1, 128, 128)))
    out.append(("proj.b", (128,)))
    out.append(("E", (M, 64)))
    for l in range(cfg["head_layers"]):
        out.append(("head%d.W" % l, (9, 64, 64)))
        out.append(("head%d.b" % l, (64,)))
    out.append(("wo", (64,)))
    out.append(("bo", (1,)))
    return out


def n_params(cfg):
    return sum(int(np.prod(s)) for _, s in layout(cfg))


def unpack(flat, cfg):
    """Flat vector (numpy or torch) -> dict of tensors (views of one FP64 leaf)."""
    t = torch.as_tensor(np.asarray(flat, np.float64)).clone().requires_grad_(True)
    d, o = {}, 0
    for name, shape in layout(cfg):
        n = int(np.prod(shape))
        d[name] = t[o:o + n].view(*shape)
        o += n
    assert o == t.numel()
    return t, d


def bf16(x):
    """Rounds to BF16 in the forward pass, identity in the backward pass."""
    return x + (x.to(torch.bfloat16).to(torch.float64) - x).detach()


def conv_taps(x, W, taps):
    """Convolution as the GPU defines it: x [B][H][W][C] channels-last, W
    [taps][cout][cin], out[p][co] = sum_t,ci x[p + off_t][ci] W[t][co][ci]
    with zeros outside the image."""
    B, H, Wd, C = x.shape
    out = None
    for t, (dh, dw) in enumerate(taps):
        sh = torch.zeros_like(x)
        h0, h1 = max(0, -dh), min(H, H - dh)
        w0, w1 = max(0, -dw), min(Wd, Wd - dw)
        if h0 < h1 and w0 < w1:
            sh[:, h0:h1, w0:w1, :] = x[:, h0 + dh:h1 + dh, w0 + dw:w1 + dw, :]
        term = torch.einsum("bhwc,oc->bhwo", sh, W[t])
        out = term if out is None else out + term
    return out


def head_taps(d):
    return [(a * d, b * d) for a in (-1, 0, 1) for b in (-1, 0, 1)]


def enc_taps(k):
    return [(0, t - k // 2) for t in range(k)]


def embed(types, lad):
    types = np.asarray(types)
    B, L = types.shape
    x = np.zeros((B, 1, L, 64), np.float64)
    x[:, 0, :, 0] = types == 0
    x[:, 0, :, 1] = types == 1
    if lad is not None:
        x[:, 0, :, 2] = np.asarray(lad) != 0
    return torch.as_tensor(x)


def forward(p, cfg, types, lad):
    """Returns y [B][M][M] (before symmetrisation) as FP64."""
    x = embed(types, lad)
    h = None
    for l in range(cfg["enc_layers"]):
        Wb = bf16(p["enc%d.W" % l])
        inp = x if l == 0 else h
        pre = conv_taps(inp, Wb, enc_taps(cfg["enc_kernel"])) + p["enc%d.b" % l]
        a = torch.relu(pre)
        h = bf16(a if l == 0 else inp + a)
    B, _, L, C = h.shape
    M = cfg["bins"]
    f = L // M
    hp = bf16(h.reshape(B, 1, M, f, C).mean(dim=3))
    uv = bf16(conv_taps(hp, bf16(p["proj.W"]), [(0, 0)]) + p["proj.b"])
    u, v = uv[:, 0, :, :64], uv[:, 0, :, 64:]
    idx = torch.arange(M)
    dist = (idx[:, None] - idx[None, :]).abs()
    z = bf16(u[:, :, None, :] * v[:, None, :, :] + u[:, None, :, :] * v[:, :, None, :] + p["E"][dist][None])
    for l in range(cfg["head_layers"]):
        pre = conv_taps(z, bf16(p["head%d.W" % l]), head_taps(cfg["dilations"][l])) + p["head%d.b" % l]
        z = bf16(z + torch.relu(pre))
    y = torch.einsum("bijc,c->bij", z, p["wo"]) + p["bo"]
    return y


def symmetric(y):
    return 0.5 * (y + y.transpose(1, 2))


def separation_weights(dataset_maps):
    """w[s] = M / (P(s) x bin pairs at separation s), P(s) the dataset's mean
    contact probability at |i - j| = s floored at 1e-6 (ccpsur_set_dataset):
    every separation carries the same total weight."""
    m = np.asarray(dataset_maps, np.float64)
    n, M, _ = m.shape
    i = np.arange(M)
    dist = np.abs(i[:, None] - i[None, :])
    tot = np.bincount(dist.ravel(), weights=m.sum(axis=0).ravel(), minlength=M)
    npairs = np.bincount(dist.ravel(), minlength=M).astype(np.float64)
    return M / (np.maximum(tot / (n * npairs), 1e-6) * npairs)


def loss_and_grads(flat, cfg, types, lad, maps, dataset_maps):
    """Separation-weighted Poisson deviance of the maps against exp(yhat),
    mean over all values; FP64 loss and flat gradient. dataset_maps: every
    map given to ccpsur_set_dataset (they set the weights)."""
    leaf, p = unpack(flat, cfg)
    y = forward(p, cfg, types, lad)
    t = torch.as_tensor(np.asarray(maps, np.float64))
    M = cfg["bins"]
    idx = np.arange(M)
    w = torch.as_tensor(separation_weights(dataset_maps).astype(np.float32).astype(np.float64))
    wmat = w[torch.as_tensor(np.abs(idx[:, None] - idx[None, :]))]
    ys = symmetric(y)
    # clamped forward, straight-through backward (as the GPU loss kernel)
    yh = ys - (ys - torch.clamp(ys, max=YHAT_MAX)).detach()
    dev = torch.exp(yh) - t - t * yh + torch.xlogy(t, t)
    loss = (wmat[None] * dev).mean()
    loss.backward()
    return float(loss.detach()), leaf.grad.numpy().copy()


def predict(flat, cfg, types, lad):
    with torch.no_grad():
        _, p = unpack(flat, cfg)
        yh = symmetric(forward(p, cfg, types, lad))
        return torch.exp(torch.clamp(yh, max=YHAT_MAX)).numpy()
