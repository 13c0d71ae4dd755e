"""Python binding of the contact-map surrogate (include/ccpgpu_surrogate.h)
through ctypes, and the data pipeline that trains it on maps simulated by the
batched engine (include/ccpgpu.h).

There is no CPU fallback: the network runs only through libccpgpu.so's
tcgen05 kernels, and importing the binding fails when the library is missing.

Data pipeline (no reference counterpart; the contact map itself is ccp's
calc_cm, Program/src/chrana.cu:48-84):
  make_sequences   seeded two-type sequences: per sequence a mean block length
                   drawn uniformly from [block_min, block_max], a two-state
                   Markov chain with switch probability 1 / block length, and
                   a lamina-binding (LAD) flag on a random fraction of beads
  simulate_maps    one engine replica per sequence (baseline force field,
                   sphere at packing fraction 0.2); after a burn-in the binned
                   contact counts are accumulated every `every` steps and
                   turned into contact probabilities
  ps_curve         P(s): the mean contact probability at bin separation s
"""
import ctypes as C

import numpy as np

from . import ccpgpu

SYMBOLS = (
    "ccpsur_create", "ccpsur_destroy", "ccpsur_info_get", "ccpsur_get_params",
    "ccpsur_set_params", "ccpsur_get_grads", "ccpsur_set_dataset", "ccpsur_loss_grad",
    "ccpsur_train_step", "ccpsur_predict", "ccpsur_predict_ps", "ccpsur_predict_rows",
    "ccpsur_synchronize",
    "ccpsur_stream_handle", "ccpsur_error_flags", "ccpsur_kernel_count", "ccpsur_conv_bf16",
    "ccpsur_wgrad_bf16",
)

ENGINE_PARAMS = "force_field baseline\ncontact_cutoff 1.5\npacking_fraction 0.2\n"


class Info(C.Structure):
    _fields_ = [("seq_len", C.c_int32), ("bins", C.c_int32), ("batch", C.c_int32),
                ("enc_layers", C.c_int32), ("enc_width", C.c_int32), ("enc_kernel", C.c_int32),
                ("head_layers", C.c_int32), ("head_width", C.c_int32),
                ("dataset_size", C.c_int32), ("n_params", C.c_int64), ("step", C.c_int64)]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ccpgpu.load()
    P, I32, I64, U64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64
    sig = {
        "ccpsur_create": [C.c_char_p, U64, C.POINTER(P)],
        "ccpsur_destroy": [P],
        "ccpsur_info_get": [P, C.POINTER(Info)],
        "ccpsur_get_params": [P, P, I64], "ccpsur_set_params": [P, P, I64],
        "ccpsur_get_grads": [P, P, I64],
        "ccpsur_set_dataset": [P, P, P, P, I32],
        "ccpsur_loss_grad": [P, P, I32, C.POINTER(C.c_double)],
        "ccpsur_train_step": [P, P, I32, C.POINTER(C.c_double)],
        "ccpsur_predict": [P, P, P, I32, P],
        "ccpsur_predict_ps": [P, P, P, I32, P],
        "ccpsur_predict_rows": [P, P, I32, P],
        "ccpsur_synchronize": [P],
        "ccpsur_stream_handle": [P, C.POINTER(P)],
        "ccpsur_error_flags": [P, C.POINTER(I32)],
        "ccpsur_kernel_count": [P, C.POINTER(I64)],
        "ccpsur_conv_bf16": [I32, I32, I32, I32, I32, I32, P, P, P, P, P, I32, P, P, P],
        "ccpsur_wgrad_bf16": [I32, I32, I32, I32, I32, I32, P, P, P, P, P, P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = lib
    return lib


def _check(rc):
    if rc != ccpgpu.OK:
        raise ccpgpu.CcpError(rc, _lib.ccpgpu_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- BF16 helpers

def to_bf16(a):
    """float32 -> BF16 bit patterns (uint16), round to nearest even."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def from_bf16(u):
    return (np.asarray(u, np.uint16).astype(np.uint32) << 16).view(np.float32)


def conv_bf16(x, w, taps, bias=None, relu=False, resid=None, want_mask=False):
    """One tensor-core convolution (ccpsur_conv_bf16). x [B][H][W][cin] and w
    [taps][cout][cin] as BF16 bit patterns (uint16); resid [B][H][W][cout]
    uint16. Returns (out uint16, mask uint32 or None)."""
    load()
    x = np.ascontiguousarray(x, np.uint16)
    w = np.ascontiguousarray(w, np.uint16)
    B, H, W, cin = x.shape
    cout = w.shape[1]
    dh = np.array([t[0] for t in taps], np.int32)
    dw = np.array([t[1] for t in taps], np.int32)
    b = None if bias is None else np.ascontiguousarray(bias, np.float32)
    r = None if resid is None else np.ascontiguousarray(resid, np.uint16)
    out = np.empty((B, H, W, cout), np.uint16)
    mask = np.empty((B, H, W, cout // 32), np.uint32) if want_mask else None
    _check(_lib.ccpsur_conv_bf16(B, H, W, cin, cout, len(taps), _ptr(dh), _ptr(dw), _ptr(x), _ptr(w),
                                 _ptr(b), 1 if relu else 0, _ptr(r), _ptr(out), _ptr(mask)))
    return out, mask


def wgrad_bf16(x, dy, taps, want_db=True):
    """Weight (and bias) gradient of a convolution (ccpsur_wgrad_bf16): x
    [B][H][W][cin], dy [B][H][W][cout] as uint16. Returns (dw [taps][cout][cin]
    float32, db [cout] float32 or None)."""
    load()
    x = np.ascontiguousarray(x, np.uint16)
    dy = np.ascontiguousarray(dy, np.uint16)
    B, H, W, cin = x.shape
    cout = dy.shape[3]
    dh = np.array([t[0] for t in taps], np.int32)
    dw = np.array([t[1] for t in taps], np.int32)
    out = np.empty((len(taps), cout, cin), np.float32)
    db = np.empty(cout, np.float32) if want_db else None
    _check(_lib.ccpsur_wgrad_bf16(B, H, W, cin, cout, len(taps), _ptr(dh), _ptr(dw), _ptr(x), _ptr(dy),
                                  _ptr(out), _ptr(db)))
    return out, db


# ---------------------------------------------------------------- network

class Surrogate:
    """A surrogate network handle (ccpsur_net)."""

    def __init__(self, config_text="", seed=0):
        load()
        self._h = C.c_void_p()
        _check(_lib.ccpsur_create(config_text.encode(), int(seed), C.byref(self._h)))

    def close(self):
        if self._h:
            _lib.ccpsur_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        i = Info()
        _check(_lib.ccpsur_info_get(self._h, C.byref(i)))
        return i

    @property
    def n_params(self):
        return self.info().n_params

    def params(self):
        a = np.empty(self.n_params, np.float32)
        _check(_lib.ccpsur_get_params(self._h, _ptr(a), a.size))
        return a

    def set_params(self, p):
        a = np.ascontiguousarray(p, np.float32)
        _check(_lib.ccpsur_set_params(self._h, _ptr(a), a.size))

    def grads(self):
        a = np.empty(self.n_params, np.float32)
        _check(_lib.ccpsur_get_grads(self._h, _ptr(a), a.size))
        return a

    def set_dataset(self, types, lad, maps):
        t = np.ascontiguousarray(types, np.uint8)
        l = None if lad is None else np.ascontiguousarray(lad, np.uint8)
        m = np.ascontiguousarray(maps, np.float32)
        _check(_lib.ccpsur_set_dataset(self._h, _ptr(t), _ptr(l), _ptr(m), t.shape[0]))

    def loss_grad(self, rows):
        r = np.ascontiguousarray(rows, np.int32)
        loss = C.c_double()
        _check(_lib.ccpsur_loss_grad(self._h, _ptr(r), r.size, C.byref(loss)))
        return loss.value

    def train_step(self, rows, want_loss=True):
        r = np.ascontiguousarray(rows, np.int32)
        loss = C.c_double()
        _check(_lib.ccpsur_train_step(self._h, _ptr(r), r.size, C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def predict(self, types, lad=None):
        t = np.ascontiguousarray(types, np.uint8)
        l = None if lad is None else np.ascontiguousarray(lad, np.uint8)
        i = self.info()
        out = np.empty((t.shape[0], i.bins, i.bins), np.float32)
        _check(_lib.ccpsur_predict(self._h, _ptr(t), _ptr(l), t.shape[0], _ptr(out)))
        return out

    def predict_ps(self, types, lad=None):
        """P(s) [n][bins] of the predicted maps (the mean of each diagonal),
        reduced on the device: no map is copied to the host."""
        t = np.ascontiguousarray(types, np.uint8)
        l = None if lad is None else np.ascontiguousarray(lad, np.uint8)
        out = np.empty((t.shape[0], self.info().bins), np.float32)
        _check(_lib.ccpsur_predict_ps(self._h, _ptr(t), _ptr(l), t.shape[0], _ptr(out)))
        return out

    def predict_rows(self, rows, copy=True):
        r = np.ascontiguousarray(rows, np.int32)
        out = None
        if copy:
            i = self.info()
            out = np.empty((r.size, i.bins, i.bins), np.float32)
        _check(_lib.ccpsur_predict_rows(self._h, _ptr(r), r.size, _ptr(out)))
        return out

    def synchronize(self):
        _check(_lib.ccpsur_synchronize(self._h))

    def stream(self):
        s = C.c_void_p()
        _check(_lib.ccpsur_stream_handle(self._h, C.byref(s)))
        return s.value

    def error_flags(self):
        f = C.c_int32()
        _check(_lib.ccpsur_error_flags(self._h, C.byref(f)))
        return f.value

    def kernel_count(self):
        n = C.c_int64()
        _check(_lib.ccpsur_kernel_count(self._h, C.byref(n)))
        return n.value


# ---------------------------------------------------------------- data

def make_sequences(n, length, seed, block_min=4.0, block_max=64.0, lad_fraction=0.1):
    """Seeded two-type sequences: types uint8 [n][length] (0 = A, 1 = B) and
    LAD flags uint8 [n][length]; also the mean block length of each."""
    rng = np.random.default_rng(seed)
    blocks = rng.uniform(block_min, block_max, n)
    types = np.empty((n, length), np.uint8)
    for k in range(n):
        sw = rng.random(length) < 1.0 / blocks[k]
        sw[0] = False
        first = rng.integers(0, 2)
        types[k] = (first + np.cumsum(sw)) & 1
    lad = (rng.random((n, length)) < lad_fraction).astype(np.uint8)
    return types, lad, blocks


def counts_to_probability(tri, bins, frames, beads_per_bin):
    """Lower-triangular contact counts of one replica (ccpgpu_contact_counts:
    off-diagonal pairs counted once, same-bin pairs twice) -> symmetric
    contact-probability matrix [bins][bins]."""
    m = np.zeros((bins, bins), np.float64)
    il = np.tril_indices(bins)
    m[il] = tri
    m = m + np.tril(m, -1).T
    pairs = np.full((bins, bins), float(beads_per_bin * beads_per_bin))
    np.fill_diagonal(pairs, float(beads_per_bin * (beads_per_bin - 1)))
    return (m / (frames * pairs)).astype(np.float32)


def simulate_maps(types, lad, bins, steps, burn_in, every, seed, params=ENGINE_PARAMS, reps=1):
    """Contact-probability maps [n][bins][bins] of the sequences, simulated
    together in one batch: with reps > 1 each sequence is run by `reps`
    replicas (their own seeds and initial conditions) and its map is their
    mean. Returns (maps, frames)."""
    types = np.asarray(types)
    if reps > 1:
        maps, frames = simulate_maps(np.repeat(types, reps, 0), np.repeat(np.asarray(lad), reps, 0),
                                     bins, steps, burn_in, every, seed, params)
        return maps.reshape(types.shape[0], reps, bins, bins).mean(axis=1), frames
    n, L = types.shape
    text = params + "contact_bins %d\nsteps_per_frame %d\n" % (bins, every)
    seeds = np.arange(n, dtype=np.uint64) + np.uint64(seed)
    with ccpgpu.Batch(text, [L] * n, seeds=seeds, seed=seed) as b:
        b.generate_initial_condition()
        pt = types.astype(np.int32) | (np.asarray(lad, np.int32) != 0).astype(np.int32) << 1
        b.set_types(pt.reshape(-1))
        if burn_in:
            b.run_steps(burn_in, 0)
        b.reset_observables()
        b.run_steps(steps, every)
        frames = steps // every
        maps = np.empty((n, bins, bins), np.float32)
        for s in range(n):
            maps[s] = counts_to_probability(b.contact_counts(s), bins, frames, L // bins)
    return maps, frames


def ps_curve(maps, smax=None):
    """P(s) for s = 0 .. smax - 1 (default bins - 1): mean of each diagonal
    band, per map."""
    maps = np.asarray(maps)
    n, M, _ = maps.shape
    smax = M if smax is None else min(M, smax)
    out = np.empty((n, smax))
    i = np.arange(M)
    for s in range(smax):
        out[:, s] = maps[:, i[:M - s], i[s:]].mean(axis=1, dtype=np.float64)
    return out


def powerlaw_map(maps, bins=None):
    """The P(s)-only predictor: a power law P(s) = a s^b fitted (least squares
    in log-log) to the mean P(s) of `maps` over s = 1 .. bins/2 - 1, spread
    over every bin pair |i - j| = s, with the mean's own P(0) on the diagonal.
    Returns one map [1][bins][bins]."""
    ps = ps_curve(maps).mean(axis=0)
    M = ps.shape[0] if bins is None else bins
    s = np.arange(1, M // 2)
    b, loga = np.polyfit(np.log(s), np.log(np.maximum(ps[s], 1e-12)), 1)
    d = np.abs(np.arange(M)[:, None] - np.arange(M)[None, :]).astype(np.float64)
    m = np.exp(loga) * np.maximum(d, 1.0) ** b
    np.fill_diagonal(m, ps[0])
    return m[None].astype(np.float32)


def ps_octaves(ps, bins):
    """Octave means of P(s) curves ps [n][>= bins/2]: s in [1, 2), [2, 4), ...,
    [bins/4, bins/2), one value per octave and curve."""
    ps = np.asarray(ps, np.float64)
    out, a = [], 1
    while a < bins // 2:
        b = min(2 * a, bins // 2)
        out.append(ps[:, a:b].mean(axis=1))
        a = b
    return np.stack(out, axis=1)


def ps_log_bins(maps):
    """P(s) averaged over octaves of separation, s in [1, 2), [2, 4), ...,
    [bins/4, bins/2): one value per octave and map."""
    M = np.asarray(maps).shape[1]
    return ps_octaves(ps_curve(maps, M // 2), M)


def ps_error(pred, ref):
    """Per map: mean over separation octaves of |P_pred - P_ref| / P_ref."""
    pp, pr = ps_log_bins(pred), ps_log_bins(ref)
    return (np.abs(pp - pr) / np.maximum(pr, 1e-12)).mean(axis=1)


def map_log_error(pred, ref, eps=1e-3):
    """Per map: mean |log10(p_pred + eps) - log10(p_ref + eps)| over bin pairs."""
    return np.abs(np.log10(np.asarray(pred, np.float64) + eps)
                  - np.log10(np.asarray(ref, np.float64) + eps)).mean(axis=(1, 2))


# ---------------------------------------------------------------- training and screening

def train(net, n_train, epochs, seed, eval_rows=None):
    """AdamW epochs over dataset rows [0, n_train) in seeded random batches of
    the network's batch size. Returns per epoch the loss of one training
    batch and, with eval_rows, the mean loss over those rows."""
    B = net.info().batch
    rng = np.random.default_rng(seed)
    history = []
    for ep in range(epochs):
        perm = rng.permutation(n_train).astype(np.int32)
        for i in range(max(1, n_train // B)):
            net.train_step(perm[i * B:(i + 1) * B], want_loss=False)
        rec = {"epoch": ep + 1, "train_loss": net.loss_grad(perm[:B])}
        if eval_rows is not None and len(eval_rows) >= B:
            ev = np.asarray(eval_rows, np.int32)
            rec["heldout_loss"] = float(np.mean([net.loss_grad(ev[i:i + B])
                                                 for i in range(0, len(ev) - B + 1, B)]))
        history.append(rec)
    return history


def envelope(maps, margin=0.25):
    """Per separation octave, the range of P(s) over a set of maps widened by
    `margin` (relative) on both sides: where a prediction may fall without
    being re-simulated."""
    pb = ps_log_bins(maps)
    return pb.min(axis=0) * (1.0 - margin), pb.max(axis=0) * (1.0 + margin)


def screen(net, types, lad, env, fallback_fraction, seed, sim, chunk=4096):
    """Batched inference over many sequences with a simulation fallback
    (only each prediction's P(s) comes back from the device): a
    random `fallback_fraction` of them, plus every sequence whose predicted
    P(s) leaves the envelope in some separation octave, is re-simulated by
    `sim` (a callable (types, lad) -> maps), whose maps check the prediction.
    Returns a report and the indices re-simulated."""
    import time

    n = types.shape[0]
    rng = np.random.default_rng(seed)
    lo, hi = env
    out_env = np.zeros(n, bool)
    pb_pred = None
    t0 = time.perf_counter()
    bins = net.info().bins
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        pb = ps_octaves(net.predict_ps(types[a:b], lad[a:b]), bins)
        if pb_pred is None:
            pb_pred = np.empty((n, pb.shape[1]))
        pb_pred[a:b] = pb
        out_env[a:b] = np.any((pb < lo) | (pb > hi), axis=1)
    t_pred = time.perf_counter() - t0
    k = max(1, int(round(fallback_fraction * n)))
    rand = rng.choice(n, k, replace=False)
    fb = np.union1d(rand, np.nonzero(out_env)[0])
    t1 = time.perf_counter()
    sim_maps = sim(types[fb], lad[fb])
    t_sim = time.perf_counter() - t1
    pb_sim = ps_log_bins(sim_maps)
    err = (np.abs(pb_pred[fb] - pb_sim) / np.maximum(pb_sim, 1e-12)).mean(axis=1)
    in_rand = np.isin(fb, rand)
    # the re-simulated sequences' full maps, predicted again, against the
    # simulation bin by bin: per map the mean |log10| difference, and over the
    # random sample the mean difference of each separation octave's bins
    pred_maps = np.concatenate([net.predict(types[fb[a:a + chunk]], lad[fb[a:a + chunk]])
                                for a in range(0, len(fb), chunk)])
    merr = map_log_error(pred_maps, sim_maps)
    d = np.abs(np.log10(pred_maps[in_rand].astype(np.float64) + 1e-3)
               - np.log10(np.asarray(sim_maps)[in_rand].astype(np.float64) + 1e-3)).mean(axis=0)
    sep = np.abs(np.arange(bins)[:, None] - np.arange(bins)[None, :])
    by_octave, a = [], 1
    while a < bins // 2:
        b = min(2 * a, bins // 2)
        by_octave.append(float(d[(sep >= a) & (sep < b)].mean()))
        a = b
    rep = {
        "sequences": int(n),
        "predict_s": t_pred,
        "maps_per_s_with_host_io": n / t_pred,
        "host_io": "sequences in, P(s) of every predicted map out (reduced on the device)",
        "fallback_random": int(k),
        "fallback_out_of_envelope": int(out_env.sum()),
        "simulated": int(len(fb)),
        "simulate_s": t_sim,
        "ps_error_random_sample": {"mean": float(err[in_rand].mean()), "median": float(np.median(err[in_rand])),
                                   "p90": float(np.percentile(err[in_rand], 90))},
        "map_log10_error_random_sample": {
            "mean": float(merr[in_rand].mean()), "median": float(np.median(merr[in_rand])),
            "p90": float(np.percentile(merr[in_rand], 90)),
            "by_separation_octave": by_octave},
    }
    if (~in_rand).any():
        rep["ps_error_out_of_envelope"] = float(err[~in_rand].mean())
        rep["map_log10_error_out_of_envelope"] = float(merr[~in_rand].mean())
    return rep, fb
