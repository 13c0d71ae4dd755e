"""Generates the golden fixtures of tests/golden/ by running the REFERENCE's own
device code on a GPU.

oracle/_ref/ccp_ref.cubin is built from the reference's Program/src/chrsim.cu,
sugrid.cu and chrana.cu by oracle/ref/build_ref.sh (nvcc -cubin, sm_103a).
This script loads it with the CUDA driver API (ctypes on libcuda) and, for a
set of seeded inputs, runs:
  calc_indexes + (host stable sort of the cell keys, standing in for the CUB
  radix sort of sugrid.cu:130) + set_cells_empty + find_cells_limits
                                      -> the reference cell list (sugrid.cu:15-77)
  ref_forces_dst / ref_forces_icg     -> calc_bf + calc_cf + calc_srf forces
  calc_cm, calc_sd_cp                 -> contact map, d(s), P(s) (chrana.cu:13-84)
and stores inputs and outputs in <out_dir>/<case>.npz. Inputs are seeded
synthetic configurations (no reference data files are read).

Usage (on a machine with a GB300):  python tests/golden/make_golden.py [out_dir]
(out_dir defaults to tests/golden, the fixtures' own folder)
"""
import ctypes as C
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ccp_ref.cubin")

RCO = np.float32(1.154701)
ACO = np.float32(2.0)
LCO = np.float32(0.5)
N_DEF = 30386
CHR_LIM = [0, 2284, 4599, 6687, 9338, 12508, 15193, 17477, 19792, 21880, 24531, 27701, 30386]


# ----------------------------------------------------------------- driver API
class Cuda:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self._ck(self.cu.cuInit(0))
        dev = C.c_int()
        self._ck(self.cu.cuDeviceGet(C.byref(dev), 0))
        self.ctx = C.c_void_p()
        self._ck(self.cu.cuDevicePrimaryCtxRetain(C.byref(self.ctx), dev))
        self._ck(self.cu.cuCtxSetCurrent(self.ctx))
        self.mod = C.c_void_p()
        self._ck(self.cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()))
        self.allocs = []

    @staticmethod
    def _ck(rc):
        if rc != 0:
            raise RuntimeError("CUDA driver error %d" % rc)

    def fn(self, name):
        f = C.c_void_p()
        self._ck(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()))
        return f

    def alloc(self, nbytes):
        p = C.c_uint64()
        self._ck(self.cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(int(nbytes), 16))))
        self._ck(self.cu.cuMemsetD8_v2(p, C.c_ubyte(0), C.c_size_t(max(int(nbytes), 16))))
        self.allocs.append(p)
        return p

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        if arr.nbytes:
            self._ck(self.cu.cuMemcpyHtoD_v2(p, arr.ctypes.data_as(C.c_void_p),
                                              C.c_size_t(arr.nbytes)))
        return p

    def get(self, p, shape, dtype):
        a = np.empty(shape, dtype)
        if a.nbytes:
            self._ck(self.cu.cuMemcpyDtoH_v2(a.ctypes.data_as(C.c_void_p), p,
                                              C.c_size_t(a.nbytes)))
        return a

    def launch(self, f, n, args, tpb=128):
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        grid = max((n + tpb - 1) // tpb, 1)
        self._ck(self.cu.cuLaunchKernel(f, grid, 1, 1, tpb, 1, 1, 0, None, ptrs, None))
        self._ck(self.cu.cuCtxSynchronize())

    def free_all(self):
        for p in self.allocs:
            self.cu.cuMemFree_v2(p)
        self.allocs = []


class CnGeom(C.Structure):  # mmc::cngeom (chrdat.cuh:48-67)
    _fields_ = [(k, C.c_float) for k in ("R_n", "R_o", "R_b", "noc", "boc", "nod", "bod",
                                         "d_b", "d_m")]


class SuGrid(C.Structure):  # mmc::sugrid (sugrid.cuh:15-32)
    _fields_ = [("n_o", C.c_uint32), ("csl", C.c_float), ("cps", C.c_uint32),
                ("n_c", C.c_uint32), ("uci", C.c_uint64), ("sci", C.c_uint64),
                ("uoi", C.c_uint64), ("soi", C.c_uint64), ("beg", C.c_uint64),
                ("end", C.c_uint64), ("eb", C.c_uint64), ("ebs", C.c_uint64)]


def cngeom(R_n, R_o, R_b):
    f = np.float32
    R_n, R_o, R_b = f(R_n), f(R_o), f(R_b)
    with np.errstate(invalid="ignore", divide="ignore"):
        noc = f(math.cos(math.asin(R_o / R_n)))
        boc = f(math.cos(math.asin(R_o / R_b))) if R_b > 0 else f("nan")
    nod = f(math.sqrt(R_n * R_n - R_o * R_o))
    bod = f(math.sqrt(R_b * R_b - R_o * R_o))
    d_b = f(nod + bod)
    return CnGeom(R_n, R_o, R_b, noc, boc, nod, bod, d_b, f(d_b + R_b))


def ref_grid(cuda, xyz_dev, n_o, csl, cps):
    """Reference cell list of n_o objects (sugrid::generate_arrays, sugrid.cu:125-133)."""
    n_c = cps ** 3
    uci, uoi = cuda.alloc(4 * n_o), cuda.alloc(4 * n_o)
    cuda.launch(cuda.fn("_ZN3mmc12calc_indexesEjfjPjS0_PNS_5vec3fE"), n_o,
                [C.c_uint32(n_o), C.c_float(csl), C.c_uint32(cps), uci, uoi, xyz_dev])
    keys = cuda.get(uci, n_o, np.uint32)
    order = np.argsort(keys, kind="stable").astype(np.uint32)
    sci = cuda.put(keys[order])
    soi = cuda.put(order)
    beg, end = cuda.alloc(4 * n_c), cuda.alloc(4 * n_c)
    cuda.launch(cuda.fn("_ZN3mmc15set_cells_emptyEjPjS0_"), n_c, [C.c_uint32(n_c), beg, end])
    cuda.launch(cuda.fn("_ZN3mmc17find_cells_limitsEjPjS0_S0_"), n_o,
                [C.c_uint32(n_o), sci, beg, end])
    g = SuGrid(n_o, csl, cps, n_c, uci.value, sci.value, uoi.value, soi.value, beg.value,
               end.value, 0, 0)
    gp = cuda.alloc(C.sizeof(SuGrid))
    cuda._ck(cuda.cu.cuMemcpyHtoD_v2(gp, C.byref(g), C.c_size_t(C.sizeof(SuGrid))))
    return gp, keys


# ----------------------------------------------------------------- inputs
def confined_walk(rng, n, R, heads, mind=0.86):
    """Self-avoiding confined random walk (rejection on a hash grid)."""
    xyz = np.zeros((n, 3), np.float32)
    cell = 1.0
    grid = {}

    def key(p):
        return tuple(np.floor(p / cell).astype(int))

    def ok(p, i):
        if np.linalg.norm(p) > R - 0.9:
            return False
        k = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        if abs(j - i) > 1 and np.linalg.norm(xyz[j] - p) < mind:
                            return False
        return True

    hs = set(heads)
    i = 0
    while i < n:
        placed = False
        for _ in range(200):
            if i in hs:
                d = rng.normal(size=3)
                p = (d / np.linalg.norm(d) * (R - 1.0) * rng.random() ** (1 / 3)).astype(np.float32)
            else:
                d = rng.normal(size=3)
                p = (xyz[i - 1] + d / np.linalg.norm(d) * (1.0 + 0.05 * rng.normal())).astype(
                    np.float32)
            if ok(p, i):
                placed = True
                break
        if not placed:  # back off and retry
            for j in range(max(i - 8, 0), i):
                grid.get(key(xyz[j]), []).remove(j) if j in grid.get(key(xyz[j]), []) else None
            i = max(i - 8, 0)
            continue
        xyz[i] = p
        grid.setdefault(key(p), []).append(i)
        i += 1
    return xyz


def ccp_types(rng, n):
    """Exponential domains of mean 21.10139 (the law of chrsim.cu:651-671)."""
    pt = np.ones(n, np.int32)
    cde, cpt, i = 0, 1, 0
    while i < n:
        if i == cde:
            while True:
                edl = -21.10139 * math.log(1.0 - rng.random())
                if not (edl / 21.10139 > 5 or edl < 1.0):
                    break
            cde = int(i + edl)
            cpt = 0 if cpt == 1 else 1
        pt[i] = cpt
        i += 1
    return pt


def lbs_sphere(rng, n_l, R, extra_near=None):
    d = rng.normal(size=(n_l, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    lbs = (d * (R - float(RCO))).astype(np.float32)
    if extra_near is not None and len(extra_near):
        u = extra_near / np.linalg.norm(extra_near, axis=1, keepdims=True)
        jit = rng.normal(scale=0.15, size=extra_near.shape)
        near = (u * (R - float(RCO)) + jit).astype(np.float32)
        lbs = np.concatenate([lbs, near]).astype(np.float32)
    return lbs


def run_case(cuda, name, xyz, pt, lbs, R_n, R_o=0.0, R_b=0.0, icg=False, out_dir="."):
    n = len(xyz)
    n_l = len(lbs)
    ng = cngeom(R_n, R_o, R_b)
    cps = 2 * int(math.ceil(ng.d_m / float(ACO)))
    r = cuda.put(xyz.astype(np.float32))
    ptd = cuda.put(pt.astype(np.int32))
    lr = cuda.put(lbs.astype(np.float32) if n_l else np.zeros((1, 3), np.float32))
    pgp, keys = ref_grid(cuda, r, n, float(ACO), cps)
    lgp, _ = ref_grid(cuda, lr, max(n_l, 0), float(ACO), cps) if n_l else ref_grid(
        cuda, lr, 0, float(ACO), cps)
    res = dict(xyz=xyz.astype(np.float32), pt=pt.astype(np.int32), lbs=lbs.astype(np.float32),
               geo=np.array([R_n, R_o, R_b], np.float32), cell_keys=keys, cps=np.int32(cps))
    f = cuda.alloc(12 * n)
    cuda.launch(cuda.fn("ref_forces_dst"), n, [C.c_uint32(n), ng, ptd, r, f, lr, pgp, lgp])
    res["f_dst"] = cuda.get(f, (n, 3), np.float32)
    if icg:
        f2 = cuda.alloc(12 * n)
        cuda.launch(cuda.fn("ref_forces_icg"), n, [C.c_uint32(n), ng, ptd, r, f2, lr, pgp, lgp])
        res["f_icg"] = cuda.get(f2, (n, 3), np.float32)
    # contact map and d(s) / P(s) (chrana.cu:187-199, 480-511)
    cms = (n // 2) // 4 if n == N_DEF else n // 4
    lcm = cms * (cms + 1) // 2
    cm = cuda.alloc(4 * lcm)
    cuda.launch(cuda.fn("_ZN3mmc7calc_cmEjjPNS_5vec3fEPf"), lcm, [C.c_uint32(n), C.c_uint32(lcm),
                                                                   r, cm])
    cmv = cuda.get(cm, lcm, np.float32)
    nz = np.nonzero(cmv)[0].astype(np.int64)
    res["cm_idx"], res["cm_val"], res["cm_len"] = nz, cmv[nz], np.int64(lcm)
    sds, cps_ = [], []
    for c in range(6):
        if n == N_DEF:
            i_s, i_e = CHR_LIM[c], CHR_LIM[c + 1]
        elif c == 0:
            i_s, i_e = 0, n
        else:
            continue
        ls = (i_e - i_s) // 2
        sd, cp = cuda.alloc(4 * ls), cuda.alloc(4 * ls)
        cuda.launch(cuda.fn("_ZN3mmc10calc_sd_cpEjjjjPNS_5vec3fEPfS2_"), ls,
                    [C.c_uint32(n), C.c_uint32(ls), C.c_uint32(i_s), C.c_uint32(i_e), r, sd, cp])
        sds.append(cuda.get(sd, ls, np.float32))
        cps_.append(cuda.get(cp, ls, np.float32))
    res["sd"] = np.concatenate(sds)
    res["cp"] = np.concatenate(cps_)
    res["sd_len"] = np.array([len(s) for s in sds], np.int32)
    np.savez_compressed(os.path.join(out_dir, name + ".npz"), **res)
    cuda.free_all()
    print(name, n, n_l, "ok")


def near_cutoff_pairs(rng, n_pairs):
    """Bead pairs at |d| within a few ulps of the contact cutoff 2."""
    xyz = np.zeros((2 * n_pairs, 3), np.float32)
    for k in range(n_pairs):
        while True:
            base = (rng.random(3) * 160 - 80).astype(np.float32)
            if np.linalg.norm(base) < 95.0:
                break
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        t = 2.0 + (k % 9 - 4) * 2.4e-7
        xyz[2 * k] = base
        xyz[2 * k + 1] = (base.astype(np.float64) + u * t).astype(np.float32)
    return xyz


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden")
    os.makedirs(out_dir, exist_ok=True)
    cuda = Cuda()
    rng = np.random.default_rng(20261203)

    # single chain N = 2048 in a sphere (ccp's generic-N path)
    n = 2048
    R = float(RCO) / 2 + float(RCO) / 2 * (n / 0.2) ** (1 / 3)
    xyz = confined_walk(rng, n, R, [0])
    pt = ccp_types(rng, n)
    near = xyz[(pt == 0) & (np.linalg.norm(xyz, axis=1) > R - 2.0)][:40]
    lbs = lbs_sphere(rng, int((R - float(RCO)) ** 2 / 0.25 * 0.25), R, near)
    run_case(cuda, "ccp_n2048", xyz, pt, lbs, R, icg=True, out_dir=out_dir)

    # the diploid N = 30386 model: chromosome limits and two-copy analysis
    n = N_DEF
    R = float(RCO) / 2 + float(RCO) / 2 * (n / 0.2) ** (1 / 3)
    xyz = confined_walk(rng, n, R, CHR_LIM[:12])
    pt = ccp_types(rng, n)
    near = xyz[(pt == 0) & (np.linalg.norm(xyz, axis=1) > R - 2.0)][:60]
    lbs = lbs_sphere(rng, 1500, R, near)
    run_case(cuda, "ccp_ndef", xyz, pt, lbs, R, out_dir=out_dir)

    # nucleus with an opening and a bleb (chrsim.cu:100-136)
    n = 1024
    R_n, R_o, R_b = 9.0, 3.0, 5.0
    pts = []
    nod = math.sqrt(R_n ** 2 - R_o ** 2)
    bod = math.sqrt(R_b ** 2 - R_o ** 2)
    while len(pts) < n:
        p = rng.random(3) * 2 * (R_n + 2 * R_b) - (R_n + 2 * R_b)
        in_n = np.linalg.norm(p) < R_n - 0.3 and p[2] < nod
        in_b = np.linalg.norm(p - np.array([0, 0, nod + bod])) < R_b - 0.3 and p[2] >= nod
        if (in_n or in_b) and all(np.linalg.norm(p - q) > 0.9 for q in pts):
            pts.append(p)
    xyz = np.array(pts, np.float32)
    pt = ccp_types(rng, n)
    run_case(cuda, "ccp_bleb", xyz, pt, np.zeros((0, 3), np.float32), R_n, R_o, R_b,
             out_dir=out_dir)

    # contact predicate at the cutoff: pairs within a few ulps of |d| = 2
    xyz = near_cutoff_pairs(rng, 2048)
    n = len(xyz)
    run_case(cuda, "ccp_cutoff", xyz, np.ones(n, np.int32), np.zeros((0, 3), np.float32), 99.0,
             out_dir=out_dir)


if __name__ == "__main__":
    main()
