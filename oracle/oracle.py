"""ctypes loader of the CPU oracle (oracle/ccp_oracle.c) — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this module; the engine never does. The constants below restate
the reference's model constants independently of the engine's code:
  ccp preset      Program/src/chrdat.cuh:15-24, chrsim.cuh:18-20, chrsim.cu:424
  baseline preset the benchmark force field (harmonic k=100, cosine kappa=2,
                  WCA + A-A LJ eps=0.5 to 2.5 sigma, WCA wall, kT=1, dt=1e-3)
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ccp_oracle.c")
LIB = os.path.join(HERE, "_build", "libccporacle.so")

F_A, F_LAD, F_HEAD = 1, 2, 4
MODE_DST, MODE_ICG = 0, 1
FF_KEYS = ("pot", "bend_all", "k_e", "l_0", "k_b", "e_att", "e_rep", "rc_rep", "rc_att",
           "e_w", "rc_w", "e_l", "lco", "lbs_depth", "k_icg", "rc_icg", "dt", "sd", "max_step")

RCO = 1.154701   # chrdat.cuh:20
ACO = 2.0        # chrdat.cuh:21
LCO = 0.5        # chrdat.cuh:24
MIS = 0.838732   # chrsim.cuh:20
K_B = 0.003356   # chrdat.cuh:15
N_DEF = 30386
CHR_LIM = (0, 2284, 4599, 6687, 9338, 12508, 15193, 17477, 19792, 21880, 24531, 27701, 30386)


def ccp_ff(T=298.0):
    dt = 1.0 / 2048
    f32 = lambda v: float(np.float32(v))
    return dict(pot=0, bend_all=0, k_e=128.0, l_0=1.0, k_b=1.0, e_att=0.5, e_rep=0.5,
                rc_rep=f32(RCO), rc_att=ACO, e_w=1.0, rc_w=f32(RCO), e_l=8.0, lco=LCO,
                lbs_depth=f32(RCO), k_icg=128.0, rc_icg=f32(RCO), dt=f32(dt),
                sd=f32(math.sqrt(2.0 * float(np.float32(K_B)) * float(np.float32(T)) * dt)), max_step=0.0)


def baseline_ff(kT=1.0, dt=1e-3):
    f32 = lambda v: float(np.float32(v))
    wca = f32(2.0 ** (1.0 / 6.0))
    return dict(pot=1, bend_all=1, k_e=100.0, l_0=1.0, k_b=2.0, e_att=0.5, e_rep=1.0,
                rc_rep=wca, rc_att=2.5, e_w=1.0, rc_w=wca, e_l=8.0, lco=LCO, lbs_depth=wca,
                k_icg=128.0, rc_icg=f32(RCO), dt=f32(dt),
                sd=f32(math.sqrt(2.0 * f32(kT) * f32(dt))), max_step=0.1)


def ff_vec(ff):
    return np.array([float(ff[k]) for k in FF_KEYS], np.float64)


def geo_vec(R_n, R_o=0.0, R_b=0.0, csl=2.0):
    f32 = lambda v: float(np.float32(v))
    return np.array([f32(R_n), f32(R_o), f32(R_b), f32(csl)], np.float64)


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    hdr = os.path.join(HERE, "oracle_impl.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
           SRC, "-o", LIB + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I, U32, U64, D, Fl = (C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double,
                                 C.c_float)
        for sfx in ("f64", "f32"):
            getattr(L, "orc_forces_" + sfx).argtypes = [I, P, P, I, P, P, P, I, I, P, P]
            getattr(L, "orc_run_" + sfx).argtypes = [I, P, P, I, P, P, P, U32, U32, U64, I, I, P]
        L.orc_philox.argtypes = [P, P, P]
        L.orc_noise.argtypes = [U32, U64, U32, U32, P]
        L.orc_contacts.argtypes = [I, P, Fl, I, I, I, I, P, I, P, P, P]
        L.orc_overlaps.argtypes = [I, P, Fl]
        L.orc_overlaps.restype = C.c_longlong
        L.orc_observables.argtypes = [I, P, P, D, D, P]
        L.orc_sdist.argtypes = [I, P, P]
        L.orc_random_walk.argtypes = [I, P, U32, U32, U32, P, D, D, D, D, D, D, C.c_longlong, P]
        L.orc_random_walk.restype = C.c_longlong
        L.orc_max_threads.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def flags_from_types(pt, heads, preset="ccp"):
    """Bead flags from ccp type codes (0 = A, 1 = B; bit 1 = LAD in baseline)."""
    pt = np.asarray(pt, np.int32)
    f = np.where((pt & 1) == 0, F_A, 0).astype(np.uint32)
    lad = ((pt & 1) == 0) if preset == "ccp" else ((pt & 2) != 0)
    f |= np.where(lad, F_LAD, 0).astype(np.uint32)
    f[np.asarray(heads, np.int64)] |= F_HEAD
    return f


def forces(xyz, flags, lbs, ff, geo, mode=MODE_DST, prec=64, cells=False, with_abs=False):
    """Per-bead total force; with_abs also returns the sum of the magnitudes
    of the force terms of every bead (the scale of FP32 cancellation)."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    lbs = np.ascontiguousarray(lbs, np.float32).reshape(-1, 3)
    flags = np.ascontiguousarray(flags, np.uint32)
    n = len(flags)
    out = np.zeros((n, 3), np.float64)
    sa = np.zeros(n, np.float64)
    fn = lib().orc_forces_f64 if prec == 64 else lib().orc_forces_f32
    fn(n, _p(xyz), _p(flags), len(lbs), _p(lbs), _p(ff_vec(ff)), _p(geo), mode,
       1 if cells else 0, _p(out), _p(sa))
    return (out, sa) if with_abs else out


def run(xyz, flags, lbs, ff, geo, seed, step0, nsteps, mode=MODE_DST, prec=64):
    xyz = np.ascontiguousarray(xyz, np.float32)
    lbs = np.ascontiguousarray(lbs, np.float32).reshape(-1, 3)
    flags = np.ascontiguousarray(flags, np.uint32)
    n = len(flags)
    out = np.zeros((n, 3), np.float64)
    fn = lib().orc_run_f64 if prec == 64 else lib().orc_run_f32
    fn(n, _p(xyz), _p(flags), len(lbs), _p(lbs), _p(ff_vec(ff)), _p(geo),
       seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF, step0, nsteps, mode, _p(out))
    return out


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(o))
    return o


def noise(bead, step, seed):
    z = np.zeros(3, np.float64)
    lib().orc_noise(bead, step, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF, _p(z))
    return z


def contacts(xyz, cut, nbins, map_len, copy_len, n_copies, heads):
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = len(xyz)
    heads = np.ascontiguousarray(heads, np.int32)
    lens = np.diff(np.append(heads, n))
    ps_off = np.concatenate([[0], np.cumsum(lens // 2 + 1)[:-1]]).astype(np.int32)
    ps = np.zeros(int((lens // 2 + 1).sum()), np.int32)
    m = np.zeros(nbins * (nbins + 1) // 2, np.int32)
    lib().orc_contacts(n, _p(xyz), float(np.float32(cut)), nbins, map_len, copy_len, n_copies,
                       _p(m), len(heads), _p(heads), _p(ps_off), _p(ps))
    return m, ps, ps_off


def overlaps(xyz, mis=MIS):
    xyz = np.ascontiguousarray(xyz, np.float32)
    return lib().orc_overlaps(len(xyz), _p(xyz), float(np.float32(mis)))


def observables(xyz, flags, R_n, a=RCO / 2.0):
    xyz = np.ascontiguousarray(xyz, np.float32)
    flags = np.ascontiguousarray(flags, np.uint32)
    out = np.zeros(4 + 3 * 64, np.float64)
    lib().orc_observables(len(xyz), _p(xyz), _p(flags), float(np.float32(R_n)), a, _p(out))
    return out


def sdist(xyz):
    xyz = np.ascontiguousarray(xyz, np.float32)
    L = len(xyz)
    ds = np.zeros(L // 2 + 1, np.float64)
    lib().orc_sdist(L, _p(xyz), _p(ds))
    return ds


def host_uniforms(seed, stream_id, n):
    """(0, 1] uniforms of the engine's host initial-condition stream: Philox
    counter (ctr lo, ctr hi, 0x10000, 0x1C0DE) from ctr = stream_id << 40."""
    out, ctr = [], stream_id << 40
    key = [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF]
    while len(out) < n:
        o = philox([ctr & 0xFFFFFFFF, ctr >> 32, 0x10000, 0x1C0DE], key)
        out += [((int(v) >> 8) + 1) / 16777216.0 for v in o]
        ctr += 1
    return out[:n]


def walk_axes(seed, diploid, n_chains):
    """Cone axes and cos(half-angle) of set_particle_positons (chrsim.cu:678-716):
    ccp's diploid model shuffles the 12 icosahedral directions (Fisher-Yates,
    j = (i + 1)(1 - u)) and walks chain c around direction c % 12 within
    pi/2 - atan(golden ratio); other chains have no cone."""
    if not diploid:
        return [(0.0, 0.0, 0.0)] * n_chains, math.cos(math.pi)
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    d = [(0, 1, phi), (1, phi, 0), (phi, 0, 1), (0, 1, -phi), (1, -phi, 0), (-phi, 0, 1),
         (0, -1, phi), (-1, phi, 0), (phi, 0, -1), (0, -1, -phi), (-1, -phi, 0), (-phi, 0, -1)]
    u = host_uniforms(seed, 0x52, 11)
    for k, i in enumerate(range(11, 0, -1)):
        j = int((i + 1) * (1.0 - float(np.float32(u[k]))))
        d[i], d[j] = d[j], d[i]
    return [d[c % 12] for c in range(n_chains)], math.cos(math.pi / 2.0 - math.atan(phi))


def random_walk(n, seed, chain, axis, cos_mda, R_n, kT=1.0, k_b=1.0, k_e=128.0, l_0=1.0,
                mis=MIS, max_draws=None, with_backs=False):
    """One chain's confined random walk (oracle/ccp_oracle.c orc_random_walk);
    returns (positions (n, 3) float64, attempts used or -1[, moves back])."""
    xyz = np.zeros((n, 3), np.float64)
    ax = np.asarray(axis, np.float64)
    iT = 1.0 / kT
    c_b = 0.5 * iT * k_b
    nb = np.zeros(1, np.int64)
    budget = max_draws if max_draws is not None else min(256 * n + (1 << 17), 0xFFFFFF00)
    used = lib().orc_random_walk(n, _p(xyz), seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF, chain,
                                 _p(ax), cos_mda, R_n, mis, c_b, l_0,
                                 math.sqrt(2.0 / (k_e * iT)), budget, _p(nb))
    return (xyz, used, int(nb[0])) if with_backs else (xyz, used)

