"""ccp's own simulation step on the GPU — TEST INFRASTRUCTURE.

Runs the reference's per-step kernels (Program/src/chrsim.cu:572-580:
begin_iter, the cell-list build of sugrid::generate_arrays, exec_RK_1<DST>, a
second cell-list build, exec_RK_2<DST>), compiled unchanged from the
reference's sources into oracle/_ref/ccp_ref.cubin (oracle/ref/build_ref.sh)
and launched through the CUDA driver API on torch's memory and streams. Only
tests/ and bench.py's reference leg use it: it is the reference, never the
engine.

The cell-list build is the reference's calc_indexes, set_cells_empty and
find_cells_limits (sugrid.cu:15-77); the CUB radix sort its host code runs
between them (sugrid.cu:130) cannot be launched from a cubin, so a stable
torch.sort of the same (key, index) pairs stands in for it (a permutation:
the same result). The grid is centred at the origin with ccp's cell side
aco = 2 (chrsim.cu:425); `margin_cells` adds cells on every side beyond
ccp's own 2 ceil(R_n / aco), which changes no force (empty cells) and keeps
a bead that strays past the wall inside the grid.
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ccp_ref.cubin")
ACO = 2.0      # chrdat.cuh:21, the cell side of ccp's particle grid
RCO = 1.154701
K_B = 0.003356

# entry names as ptxas reports them for oracle/ref/ref_kernels.cu
NAMES = {
    "init_ps": "_ZN3mmc7init_psEjP24curandStatePhilox4_32_10j",
    "begin_iter": "_ZN3mmc10begin_iterEjPNS_5vec3fES1_fS1_P24curandStatePhilox4_32_10",
    "calc_indexes": "_ZN3mmc12calc_indexesEjfjPjS0_PNS_5vec3fE",
    "set_cells_empty": "_ZN3mmc15set_cells_emptyEjPjS0_",
    "find_cells_limits": "_ZN3mmc17find_cells_limitsEjPjS0_S0_",
    "exec_RK_1": "_ZN3mmc9exec_RK_1ILNS_5stypeE0EEEvjNS_6cngeomEPNS_5ptypeEPNS_5vec3fES6_S6_S6_"
                 "S6_PNS_6sugridES8_",
    "exec_RK_2": "_ZN3mmc9exec_RK_2ILNS_5stypeE0EEEvjNS_6cngeomEPNS_5ptypeEPNS_5vec3fES6_S6_S6_"
                 "S6_S6_PNS_6sugridES8_",
    "exec_RK_1_icg": "_ZN3mmc9exec_RK_1ILNS_5stypeE1EEEvjNS_6cngeomEPNS_5ptypeEPNS_5vec3fES6_S6_"
                     "S6_S6_PNS_6sugridES8_",
    "exec_RK_2_icg": "_ZN3mmc9exec_RK_2ILNS_5stypeE1EEEvjNS_6cngeomEPNS_5ptypeEPNS_5vec3fES6_S6_"
                     "S6_S6_S6_PNS_6sugridES8_",
}


class CnGeom(C.Structure):
    """mmc::cngeom (chrdat.cuh:48-67)."""
    _fields_ = [(k, C.c_float) for k in ("R_n", "R_o", "R_b", "noc", "boc", "nod", "bod", "d_b",
                                         "d_m")]


class SuGrid(C.Structure):
    """mmc::sugrid (sugrid.cuh:15-32)."""
    _fields_ = [("n_o", C.c_uint32), ("csl", C.c_float), ("cps", C.c_uint32),
                ("n_c", C.c_uint32), ("uci", C.c_uint64), ("sci", C.c_uint64),
                ("uoi", C.c_uint64), ("soi", C.c_uint64), ("beg", C.c_uint64),
                ("end", C.c_uint64), ("eb", C.c_uint64), ("ebs", C.c_uint64)]


def sphere(R_n):
    """cngeom of a plain spherical nucleus (chrdat.cu:13-18 with R_o = R_b = 0)."""
    return CnGeom(R_n, 0.0, 0.0, 1.0, float("nan"), R_n, 0.0, R_n, R_n)


class Module:
    """The cubin loaded into torch's primary context on the current device."""

    def __init__(self):
        import torch

        if not os.path.exists(CUBIN):
            raise FileNotFoundError("oracle/_ref/ccp_ref.cubin not built (needs the reference "
                                    "sources: oracle/ref/build_ref.sh)")
        torch.cuda.init()
        torch.zeros(1, device="cuda")
        self.cu = cu = C.CDLL("libcuda.so.1")
        self._ck(cu.cuInit(0))
        dev, ctx, mod = C.c_int(), C.c_void_p(), C.c_void_p()
        self._ck(cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()))
        self._ck(cu.cuDevicePrimaryCtxRetain(C.byref(ctx), dev))
        self._ck(cu.cuCtxSetCurrent(ctx))
        self._ck(cu.cuModuleLoad(C.byref(mod), CUBIN.encode()))
        self.mod = mod
        self.fns = {}
        for k, name in NAMES.items():
            f = C.c_void_p()
            self._ck(cu.cuModuleGetFunction(C.byref(f), mod, name.encode()))
            self.fns[k] = f

    @staticmethod
    def _ck(rc):
        if rc != 0:
            raise RuntimeError("CUDA driver error %d" % rc)

    def launch(self, k, n, args, stream, tpb=128):
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._ck(self.cu.cuLaunchKernel(self.fns[k], max((n + tpb - 1) // tpb, 1), 1, 1, tpb, 1,
                                        1, 0, C.c_void_p(stream.cuda_stream), ptrs, None))

    def close(self):
        if self.mod is not None:
            self._ck(self.cu.cuModuleUnload(self.mod))
            self.mod = None


def _p(t):
    return C.c_uint64(t.data_ptr())


class Grid:
    """Device buffers and descriptor of one sugrid over n_o objects."""

    def __init__(self, mod, n_o, cps, stream):
        import torch

        dv = torch.device("cuda")
        self.mod, self.n_o, self.cps, self.n_c, self.stream = mod, n_o, cps, cps ** 3, stream
        m = max(n_o, 1)
        self.t = {k: torch.zeros(m, dtype=torch.int32, device=dv)
                  for k in ("uci", "sci", "uoi", "soi")}
        self.t["beg"] = torch.zeros(self.n_c, dtype=torch.int32, device=dv)
        self.t["end"] = torch.zeros(self.n_c, dtype=torch.int32, device=dv)
        g = SuGrid(n_o, ACO, cps, self.n_c, *[self.t[k].data_ptr() for k in
                                               ("uci", "sci", "uoi", "soi", "beg", "end")], 0, 0)
        self.dev = torch.frombuffer(bytearray(bytes(g)), dtype=torch.uint8).to(dv)

    def build(self, pos):
        """sugrid::generate_arrays (sugrid.cu:125-133) of the positions pos."""
        import torch

        t, n, s = self.t, self.n_o, self.stream
        if n:
            self.mod.launch("calc_indexes", n, [C.c_uint32(n), C.c_float(ACO),
                                                C.c_uint32(self.cps), _p(t["uci"]),
                                                _p(t["uoi"]), _p(pos)], s)
            keys, perm = torch.sort(t["uci"][:n], stable=True)
            t["sci"][:n].copy_(keys)
            t["soi"][:n].copy_(t["uoi"][:n][perm])
        self.mod.launch("set_cells_empty", self.n_c, [C.c_uint32(self.n_c), _p(t["beg"]),
                                                      _p(t["end"])], s)
        if n:
            self.mod.launch("find_cells_limits", n, [C.c_uint32(n), _p(t["sci"]), _p(t["beg"]),
                                                     _p(t["end"])], s)


class System:
    """One ccp system advanced by the reference's own kernels on `stream`:
    ccp's force field (DST mode), positions (n, 3), ccp type codes (0 = A),
    lamina sites (n_l, 3), a plain sphere of radius R_n, temperature T and
    the cuRAND seed of init_ps (chrsim.cu:322-333)."""

    def __init__(self, mod, xyz, types, lbs, R_n, seed, stream, T=298.0, margin_cells=2):
        import torch

        dv = torch.device("cuda")
        n = len(types)
        self.mod, self.n, self.stream = mod, n, stream
        self.R_n = float(np.float32(R_n))
        self.ng = sphere(self.R_n)
        self.cps = 2 * int(math.ceil(self.R_n / ACO)) + 2 * margin_cells
        # the largest distance from the origin that stays inside the grid
        self.grid_half = 0.5 * self.cps * ACO
        dt = np.float32(1.0 / 2048)
        self.sd = float(np.float32(math.sqrt(2.0 * float(np.float32(K_B)) * float(np.float32(T))
                                             * float(dt))))
        with torch.cuda.stream(stream):
            self.r = torch.tensor(np.asarray(xyz, np.float32), device=dv)
            self.pt = torch.tensor(np.asarray(types, np.int32), device=dv)
            n_l = len(lbs)
            self.lr = torch.tensor(np.asarray(lbs, np.float32).reshape(-1, 3) if n_l else
                                   np.zeros((1, 3), np.float32), device=dv)
            self.f, self.ef, self.er, self.rn = (torch.zeros((n, 3), dtype=torch.float32,
                                                             device=dv) for _ in range(4))
            self.ps = torch.zeros(64 * n, dtype=torch.uint8, device=dv)
            self.pg = Grid(mod, n, self.cps, stream)
            self.lg = Grid(mod, n_l, self.cps, stream)
            mod.launch("init_ps", n, [C.c_uint32(n), _p(self.ps), C.c_uint32(seed)], stream)
            self.lg.build(self.lr)  # built once per run (chrsim.cu:561)

    def step(self, icg=False):
        """One stochastic Heun step (chrsim.cu:572-580); icg: one step of the
        initial-condition relaxation instead (soft repulsion, no noise,
        chrsim.cu:500-509)."""
        m, n, s = self.mod, self.n, self.stream
        sfx = "_icg" if icg else ""
        m.launch("begin_iter", n, [C.c_uint32(n), _p(self.f), _p(self.ef),
                                   C.c_float(0.0 if icg else self.sd), _p(self.rn), _p(self.ps)],
                 s)
        self.pg.build(self.r)
        m.launch("exec_RK_1" + sfx, n, [C.c_uint32(n), self.ng, _p(self.pt), _p(self.r),
                                        _p(self.f), _p(self.lr), _p(self.er), _p(self.rn),
                                        _p(self.pg.dev), _p(self.lg.dev)], s)
        self.pg.build(self.er)
        m.launch("exec_RK_2" + sfx, n, [C.c_uint32(n), self.ng, _p(self.pt), _p(self.r),
                                        _p(self.f), _p(self.lr), _p(self.er), _p(self.ef),
                                        _p(self.rn), _p(self.pg.dev), _p(self.lg.dev)], s)

    def max_radius(self):
        return float(self.r.norm(dim=1).max())
