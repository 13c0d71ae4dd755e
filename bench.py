"""Benchmark of the BD engine: bead-steps/s of the batched replica ensemble,
and of the contact-map surrogate trained on the engine's maps.

Workload: 512 independent replicas with bead counts N_i = floor(exp(U(ln 1024,
ln 16384))) (seeded), each with its own seeded two-state Markov type sequence
(mean block 16), 10% lamina-binding beads and Philox seed, the baseline force
field (harmonic k=100, cosine kappa=2, WCA + A-A LJ eps=0.5 to 2.5 sigma, WCA
wall, kT=1, dt=1e-3) in a sphere at packing fraction 0.2, and a 256x256 int32
contact map (cutoff 1.5 sigma) per replica accumulated every 100 steps.
Synthetic inputs; no dataset is involved.

One bench step = 100 stochastic Heun steps of every replica + one contact-map /
observable accumulation. `value` = bead-steps/s of the whole batch with the
state resident in HBM (CUDA events on the engine's stream); `e2e` = the same
through the C ABI with host buffers (positions uploaded from host memory and
downloaded after every bench step). The state (~280 MB) is larger than L2.

The default run adds a `surrogate` block: 1024 sequences simulated, the network
trained on 90 % of them and scored on the rest, batched inference timed.
`--surrogate` runs the full surrogate protocol instead (4096 training
sequences, 10^5 screened with a 1 % simulation fallback) and prints its own line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
  python bench.py --surrogate [--sur-sequences 4096] [--sur-sim-steps 20000]
                  [--sur-epochs 30] [--sur-screen 100000] [--sim-rate BEAD_STEPS_PER_S]
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PARAMS = ("force_field baseline\ncontact_bins 256\ncontact_cutoff 1.5\n"
          "steps_per_frame 100\npacking_fraction 0.2\n")
HEUN_PER_STEP = 100
B_ALG = 192.0  # algorithmic HBM bytes per bead-step of a Heun step (2 force evaluations)
PAIR_BYTES = 32.0  # pair kernel: read the cell-ordered float4, write the float4 force
# DRAM bytes per bead of one pair launch (dram__bytes_read.sum +
# dram__bytes_write.sum) from an ncu capture of the typed pair kernel on this
# workload; a constant of that capture, not measured in the timed run
PAIR_TRAFFIC_PER_BEAD = 58.9
# warp instructions per bead of one pair launch (smsp__inst_executed.sum /
# beads) from the same capture: the kernel is bound by instruction issue, so
# its issue rate against 4 warp instructions per SM cycle is its roofline
PAIR_WARP_INSTR_PER_BEAD = 108.8
GB300_SMS = 152
METRIC = "BD bead-steps/s (batched 512-replica ensemble, 1 GB300)"


def replica_sizes(n_rep, seed=2026):
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(1024), math.log(16384), n_rep))).astype(np.int32)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    from tfm_gb300 import replicas

    return replicas.init()


def barrier(ws):
    from tfm_gb300 import replicas

    replicas.barrier(ws)


def max_over_ranks(v, ws):
    from tfm_gb300 import replicas

    return replicas.max_over_ranks(v, ws)


# ---------------------------------------------------------------- CPU baseline
def _walk(n, R, rng):
    x = np.zeros((n, 3), np.float32)
    for i in range(1, n):
        for _ in range(100):
            d = rng.normal(size=3)
            p = x[i - 1] + d / np.linalg.norm(d)
            if np.linalg.norm(p) < R - 1.0:
                break
        x[i] = p
    return x


def cpu_sample(sizes, seconds=12.0, prebuilt=None):
    """FP32 oracle (ccp's force + Heun loop restated in C, OpenMP over all host
    threads) on a bounded sample of replicas; returns bead-steps/s, threads, text."""
    from oracle import oracle as orc

    orc.build()
    rng = np.random.default_rng(7)
    ff = orc.baseline_ff()
    systems = []
    for k, n in enumerate(sizes):
        R = 0.5 * (n / 0.2) ** (1 / 3)
        if prebuilt is not None:
            x, pt, lbs = prebuilt[k]
        else:
            x = _walk(int(n), R - 0.5, rng)
            pt = np.where(rng.random(n) < 0.5, 0, 1).astype(np.int32)
            lbs = np.zeros((0, 3), np.float32)
        fl = orc.flags_from_types(pt, [0], "baseline")
        geo = orc.geo_vec(R, csl=2.5)
        if prebuilt is None:  # remove overlaps with the soft relaxation mode
            x = orc.run(x, fl, lbs, ff, geo, 1, 0, 300, mode=orc.MODE_ICG, prec=32).astype(
                np.float32)
        systems.append((x, fl, lbs, geo, int(n)))
    # calibrate the number of steps
    t0 = time.perf_counter()
    for x, fl, lbs, geo, n in systems:
        orc.run(x, fl, lbs, ff, geo, 11, 0, 2, prec=32)
    t1 = time.perf_counter()
    per_step = max((t1 - t0) / 2, 1e-4)
    steps = max(2, int(seconds / per_step))
    t0 = time.perf_counter()
    for k, (x, fl, lbs, geo, n) in enumerate(systems):
        orc.run(x, fl, lbs, ff, geo, 100 + k, 0, steps, prec=32)
    dt = time.perf_counter() - t0
    beads = sum(s[4] for s in systems)
    return beads * steps / dt, orc.lib().orc_max_threads(), \
        "%d replicas (%d beads) x %d Heun steps, FP32" % (len(systems), beads, steps)


# ------------------------------------------------- reference kernels on the GPU
def reference_gpu_step(sizes, reps=20):
    """ccp's own per-step kernels (chrsim.cu:572-580: begin_iter, two cell-list
    builds, exec_RK_1<DST>, exec_RK_2<DST>), compiled from the reference's
    sources into oracle/_ref/ccp_ref.cubin and driven by oracle/ccp_gpu_ref.py,
    timed on this GPU with CUDA events on static inputs: a relaxed
    configuration with ccp's force field and the cell list of its positions,
    on ccp's own grid (cells of aco, 2 ceil(R_n / aco) per side). ccp sorts
    the cell keys with CUB's DeviceRadixSort::SortPairs from host code, which
    the cubin cannot launch; torch.sort(stable=True) of the same keys (CUB's
    radix sort as well) stands in for it. Every timed launch sees the same
    inputs (positions are restored before each exec_RK_2), so nothing can
    leave the cell grid. The step time is the sum of the kernel times: no
    launch gaps, in ccp's favour."""
    import ctypes as C

    import torch

    from oracle import ccp_gpu_ref as ref
    from oracle import oracle as orc

    try:
        mod = ref.Module()
    except FileNotFoundError as e:
        return {"unavailable": str(e)}
    stream = torch.cuda.current_stream()
    P = lambda t: C.c_uint64(t.data_ptr())
    out = []
    rng = np.random.default_rng(11)
    for n in sizes:
        rco = ref.RCO
        R = rco / 2 + rco / 2 * (n / 0.125) ** (1 / 3)  # ccp-profile.cu:55-62 (cvf 0.125)
        n_l = int(math.floor(0.25 * 4 / ((0.5 / (R - rco)) ** 2)))
        x = _walk(int(n), R - 0.5, rng)
        pt = np.where(rng.random(n) < 0.5, 0, 1).astype(np.int32)
        fl = orc.flags_from_types(pt, [0])
        geo = orc.geo_vec(R, csl=2.0)
        x = orc.run(x, fl, np.zeros((0, 3), np.float32), orc.ccp_ff(), geo, 1, 0, 300,
                    mode=orc.MODE_ICG, prec=32).astype(np.float32)
        d = rng.normal(size=(n_l, 3))
        lbs = (d / np.linalg.norm(d, axis=1, keepdims=True) * (R - rco)).astype(np.float32)
        sy = ref.System(mod, x, pt, lbs, R, seed=1, stream=stream, margin_cells=0)
        sy.pg.build(sy.r)
        r0 = sy.r.clone()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        g = sy.pg.t

        def timed(fn, before=None):
            fn()
            tot = 0.0
            for _ in range(reps):
                if before is not None:
                    before()
                ev[0].record(stream)
                fn()
                ev[1].record(stream)
                ev[1].synchronize()
                tot += ev[0].elapsed_time(ev[1])
            return tot / reps

        t_begin = timed(lambda: mod.launch("begin_iter", n, [
            C.c_uint32(n), P(sy.f), P(sy.ef), C.c_float(sy.sd), P(sy.rn), P(sy.ps)], stream))
        t_idx = timed(lambda: mod.launch("calc_indexes", n, [
            C.c_uint32(n), C.c_float(ref.ACO), C.c_uint32(sy.cps), P(g["uci"]), P(g["uoi"]),
            P(sy.r)], stream))
        t_sort = timed(lambda: torch.sort(g["uci"], stable=True))
        t_empty = timed(lambda: mod.launch("set_cells_empty", sy.pg.n_c, [
            C.c_uint32(sy.pg.n_c), P(g["beg"]), P(g["end"])], stream))
        t_lim = timed(lambda: mod.launch("find_cells_limits", n, [
            C.c_uint32(n), P(g["sci"]), P(g["beg"]), P(g["end"])], stream))
        t_rk1 = timed(lambda: mod.launch("exec_RK_1", n, [
            C.c_uint32(n), sy.ng, P(sy.pt), P(sy.r), P(sy.f), P(sy.lr), P(sy.er), P(sy.rn),
            P(sy.pg.dev), P(sy.lg.dev)], stream))
        t_rk2 = timed(lambda: mod.launch("exec_RK_2", n, [
            C.c_uint32(n), sy.ng, P(sy.pt), P(sy.r), P(sy.f), P(sy.lr), P(sy.er), P(sy.ef),
            P(sy.rn), P(sy.pg.dev), P(sy.lg.dev)], stream), before=lambda: sy.r.copy_(r0))
        step = t_begin + 2 * (t_idx + t_sort + t_empty + t_lim) + t_rk1 + t_rk2
        out.append({"n_beads": int(n), "ms_per_step": step, "bead_steps_per_s": n / (step / 1e3),
                    "ms": {"begin_iter": t_begin, "calc_indexes": t_idx, "sort (CUB via torch)": t_sort,
                           "set_cells_empty": t_empty, "find_cells_limits": t_lim,
                           "exec_RK_1": t_rk1, "exec_RK_2": t_rk2}})
        if not torch.isfinite(sy.r).all():
            raise RuntimeError("non-finite positions in the reference step")
    mod.close()
    return {"kernels": "ccp's own sm_103a kernels (oracle/_ref/ccp_ref.cubin)",
            "config": "ccp force field, cvf 0.125, laf 0.25 (ccp-profile.cu:55-62), cells of aco = 2",
            "sizes": out}


def reference_arm(args, ws, rank):
    """The reference's force/integration loop restated on the host cores (the
    reference has no CPU implementation of its loop; its kernels are
    __device__-only), timed on bounded samples of the same workload."""
    if rank != 0:
        return
    sizes = replica_sizes(512)
    sample = sizes[:3]
    for _ in range(max(args.warmup, 0)):
        cpu_sample(sample, seconds=1.0)
    vals = []
    descr = ""
    cores = 1
    walls = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        v, cores, descr = cpu_sample(sample, seconds=3.0)
        walls.append(time.perf_counter() - t0)
        vals.append(v)
    value = float(np.mean(vals))
    beads = int(sizes.sum())
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "bead-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        # each step is a bounded sample: value is the sample's rate, ms_per_step
        # its wall time; the full ensemble's step is extrapolated separately
        "ms_per_step": 1000.0 * float(np.mean(walls)),
        "value_kind": "sampled rate (3 replicas of the ensemble per step)",
        "extrapolated_ms_per_full_step": 1000.0 * beads * HEUN_PER_STEP / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "c2: 512 replicas, N_i log-uniform [1024, 16384], baseline force "
                               "field, 256^2 contact maps every 100 steps",
                   "total_beads": beads, "heun_steps_per_step": HEUN_PER_STEP},
        "cpu_baseline": {"value": value, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                         "sample": descr},
        "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if args.ref_gpu:
        try:
            line["reference_gpu_kernels"] = reference_gpu_step([1024, 2048, 8192, 32768])
        except Exception as e:  # reported, not fatal: the CPU arm is the reference line
            line["reference_gpu_kernels"] = {"unavailable": str(e)[:200]}
    print(json.dumps(line))


# ---------------------------------------------------------------- engine arm
def engine_arm(args, ws, rank, local):
    import torch

    from tfm_gb300 import build as eb
    from tfm_gb300 import replicas

    eb.build()
    from tfm_gb300.ccpgpu import Batch

    torch.cuda.set_device(local)
    if args.split:
        # one fixed ensemble split over the ranks by bead count (strong scaling);
        # every replica keeps its seed, so the ensemble does not depend on N
        if args.replicas < ws:
            raise SystemExit("--split needs at least one replica per rank")
        ensemble = replica_sizes(args.replicas)
        _, sizes, seeds = replicas.local_replicas(
            ensemble, np.arange(args.replicas, dtype=np.uint64) + 1, ws, rank)
        job_beads = int(ensemble.sum())
    else:
        sizes = replica_sizes(args.replicas)
        seeds = replicas.replica_seeds(args.replicas, rank)  # disjoint per rank
        job_beads = ws * int(sizes.sum())  # weak scaling: N ensembles
    params = PARAMS + ("pair_kernel %d\n" % args.pair_kernel if args.pair_kernel is not None else "")
    b = Batch(params, sizes, seeds=seeds)
    b.generate_initial_condition()
    tune = b.autotune(reps=3) if not args.no_tune else None  # per size class, untimed
    total = int(sizes.sum())
    stream = torch.cuda.ExternalStream(b.stream())

    for _ in range(args.warmup):
        b.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    b.synchronize()
    b.reset_observables()

    clocks = Clocks(local)
    k0 = b.kernel_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()  # ncu --profile-from-start off sees this region
    ev0.record(stream)
    for _ in range(args.steps):
        b.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    ev1.record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    barrier(ws)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = b.kernel_count() - k0
    ms = max_over_ranks(ms, ws)
    value = job_beads * HEUN_PER_STEP * args.steps / (ms / 1000.0)  # all ranks' beads / slowest
    ms_step = ms / args.steps

    # dominant kernel (pair) timed live with CUDA events on the engine stream
    kt = b.kernel_times(reps=5)
    hbm, peak_kind = peaks()
    pair_s = kt["pair"] / 1000.0
    achieved = total * PAIR_BYTES / pair_s / 1e9
    traffic = PAIR_TRAFFIC_PER_BEAD * total if args.replicas == 512 else None

    # end to end through the C ABI with host buffers
    x = b.positions()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.set_positions(x)  # H2D through pinned staging
        b.advance(HEUN_PER_STEP, HEUN_PER_STEP)
        b.synchronize()
        x = b.positions()  # D2H of the step's result
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, ws)
    e2e_val = job_beads * HEUN_PER_STEP * args.steps / e2e_s

    extras = {}
    if rank == 0 and not args.no_extras:
        extras = measure_extras(args, sizes, b)
        b.close()
        extras["surrogate"] = surrogate_report(value / ws, n_seq=4096, sim_steps=20000, epochs=20,
                                               truth_reps=32, screen_n=100000)

    if rank == 0:
        # the median SM clock of the timed region (else the GB300's maximum)
        sm_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
        line = {
            "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "strong" if args.split else "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "c2: %d replicas, N_i log-uniform [1024, 16384], baseline "
                                   "force field, 256^2 int32 contact maps every 100 steps"
                                   % args.replicas,
                       "total_beads": total, "job_beads": job_beads,
                       "heun_steps_per_step": HEUN_PER_STEP,
                       "l2": "state (~%d MB) larger than the 129 MB L2" % (total * 100 // 2**20),
                       "parallelism": ("one ensemble split over GPUs by bead count" if args.split
                                       else "replicas per GPU (no collective)"),
                       "autotune": None if tune is None else {
                           "pair_kernel": tune.get("pair_kernel"),
                           "tile": tune["tile"], "lanes": tune.get("lanes"),
                           "cell_side_by_class": [[c["n_min"], c["n_max"], c["cell_side"]]
                                                  for c in tune["classes"]]}},
            "clocks": clk,
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "pair", "achieved": achieved, "peak": hbm,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": traffic,
                         "traffic_source": "ncu capture of this kernel on this workload "
                                           "(a constant, not measured in this run)",
                         "bytes_per_bead": PAIR_BYTES,
                         "pair_ms": kt["pair"]},
            "issue_roofline": None if args.replicas != 512 else {
                "kernel": "pair", "unit": "warp instructions/s",
                "achieved": total * PAIR_WARP_INSTR_PER_BEAD / pair_s,
                "peak": GB300_SMS * 4 * sm_mhz * 1e6,
                "frac": total * PAIR_WARP_INSTR_PER_BEAD / pair_s / (GB300_SMS * 4 * sm_mhz * 1e6),
                "sm_mhz": sm_mhz,
                "warp_instructions_per_bead": PAIR_WARP_INSTR_PER_BEAD,
                "source": "instruction count from an ncu capture of this kernel on this "
                          "workload (a constant); time and SM clock from this run"},
            "step_roofline": {"bytes_per_bead_step": B_ALG,
                              "achieved_gbs": value * B_ALG / 1e9,
                              "frac": value * B_ALG / 1e9 / hbm},
            "kernel_ms": kt,
            "e2e": {"value": e2e_val, "unit": "bead-steps/s",
                    "h2d_bytes_per_step": total * 16, "d2h_bytes_per_step": total * 12},
        }
        line.update(extras)
        print(json.dumps(line))


def ccp_profile_sweep(sizes, steps=2000):
    """The engine on ccp's own benchmark shapes (ccp-profile.cu:55-62: one
    system, ccp force field, chromatin volume fraction 0.125, lamina area
    fraction 0.25), ms per Heun step with CUDA events; the reference arm's
    --ref-gpu times ccp's own kernels on the same shapes."""
    import torch

    from tfm_gb300.ccpgpu import ChrSim

    rco = 1.154701
    out = []
    for n in sizes:
        R = rco / 2 + rco / 2 * (n / 0.125) ** (1 / 3)
        n_l = int(math.floor(0.25 * 4 / ((0.5 / (R - rco)) ** 2)))
        txt = ("number_of_particles %05d\nnucleus_radius %09.6f\nnumber_of_lbs %05d\n"
               % (n, R, n_l))
        sim = ChrSim(txt, seed=5)
        sim.generate_initial_condition()
        sim.advance(200)
        sim.synchronize()
        st = torch.cuda.ExternalStream(sim.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sim.advance(steps)
        e1.record(st)
        sim.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out.append({"n_beads": int(n), "ms_per_step": ms, "bead_steps_per_s": n / (ms / 1e3)})
        sim.close()
    return out


def l2_copy_gbs(mb=32, reps=50):
    """Copy bandwidth of a buffer pair that stays in the 129 MB L2 (read + write
    bytes over CUDA-event time): the roofline of the L2-resident systems."""
    import torch

    a = torch.ones(mb * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    for _ in range(5):
        b.copy_(a)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * a.numel() * 4 * reps / (e0.elapsed_time(e1) / 1000.0) / 1e9


def measure_extras(args, sizes, b):
    """Plain engine replica by replica, the large single system, the CPU baseline."""
    import torch

    from tfm_gb300.ccpgpu import Batch

    out = {}
    # plain: a sample of replicas, each alone in its own engine
    sample = sizes[:: max(1, len(sizes) // 16)][:16]
    tot_bs, tot_s = 0.0, 0.0
    for k, n in enumerate(sample):
        s = Batch(PARAMS, [int(n)], seeds=[1000 + k])
        s.generate_initial_condition()
        s.advance(HEUN_PER_STEP, HEUN_PER_STEP)
        s.synchronize()
        st = torch.cuda.ExternalStream(s.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(3):
            s.advance(HEUN_PER_STEP, HEUN_PER_STEP)
        e1.record(st)
        s.synchronize()
        tot_s += e0.elapsed_time(e1) / 1000.0
        tot_bs += float(n) * HEUN_PER_STEP * 3
        s.close()
    plain = tot_bs / tot_s
    out["plain_replica_by_replica"] = {"value": plain, "unit": "bead-steps/s",
                                       "sample": "%d replicas, each alone" % len(sample)}
    # large single system: 16 chains x 8192 beads
    big = Batch(PARAMS.replace("contact_bins 256", "contact_bins 1024"), [131072],
                n_chains=[16], seeds=[42])
    big.generate_initial_condition()
    big.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    big.synchronize()
    st = torch.cuda.ExternalStream(big.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(5):
        big.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    e1.record(st)
    big.synchronize()
    out["single_system_131072"] = {
        "value": 131072 * HEUN_PER_STEP * 5 / (e0.elapsed_time(e1) / 1000.0),
        "unit": "bead-steps/s", "config": "16 chains x 8192 beads, contact map 1024^2"}
    big.close()
    # c0: one chain of 2048 beads, 2048^2 contact map every 100 steps
    c0 = Batch(PARAMS.replace("contact_bins 256", "contact_bins 2048"), [2048], seeds=[1])
    c0.generate_initial_condition()
    c0.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    c0.synchronize()
    st = torch.cuda.ExternalStream(c0.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(20):
        c0.advance(HEUN_PER_STEP, HEUN_PER_STEP)
    e1.record(st)
    c0.synchronize()
    out["single_system_2048"] = {
        "value": 2048 * HEUN_PER_STEP * 20 / (e0.elapsed_time(e1) / 1000.0),
        "unit": "bead-steps/s", "config": "c0: one chain of 2048 beads, contact map 2048^2"}
    c0.close()
    # the single systems' state (<= ~15 MB) stays in L2: their step roofline
    # is the L2 copy bandwidth, not HBM
    l2 = l2_copy_gbs()
    out["l2_copy_gbs"] = {"value": l2, "buffer": "2 x 32 MB, torch copy, CUDA events"}
    for key in ("single_system_131072", "single_system_2048"):
        v = out[key]["value"]
        out[key]["l2_roofline"] = {"bytes_per_bead_step": B_ALG, "achieved_gbs": v * B_ALG / 1e9,
                                   "peak_gbs": l2, "frac": v * B_ALG / 1e9 / l2}
    out["ccp_profile"] = ccp_profile_sweep([1024, 2048, 8192, 32768])
    # CPU baseline: the FP32 oracle on the first replicas' initial conditions
    pre = []
    x = b.positions()
    pt = b.types()
    lbs = b.lbs()
    for k in range(3):
        si = b.system_info(k)
        pre.append((x[si.bead_offset:si.bead_offset + si.n_beads],
                    pt[si.bead_offset:si.bead_offset + si.n_beads],
                    lbs[si.lbs_offset:si.lbs_offset + si.n_lbs]))
    v, cores, descr = cpu_sample(sizes[:3], seconds=12.0, prebuilt=pre)
    out["cpu_baseline"] = {"value": v, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                           "sample": descr}
    return out


# ---------------------------------------------------------------- surrogate

SUR_L, SUR_M = 1024, 256
# forward FLOPs of one map: 6 head 3x3 convolutions 64 -> 64 at bins^2 pixels,
# the 8 encoder convolutions (kernel 5) at seq_len positions, the projection
SUR_FWD_FLOP = (6 * 2 * SUR_M * SUR_M * 9 * 64 * 64 + 2 * SUR_L * 5 * 64 * 128
                + 7 * 2 * SUR_L * 5 * 128 * 128 + 2 * SUR_M * 128 * 128)
SIM_STEPS_PER_MAP = 100000  # the batched-ensemble protocol: 1e5 Heun steps per map
SUR_INFER_BATCH = 128  # sequences per inference batch (training: 32)


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def surrogate_report(bead_steps_per_s, n_seq, sim_steps, epochs, truth_reps, screen_n, seed=7,
                     burn=5000, every=200, n_truth=64):
    """c3 and c4 for the surrogate. Simulate one contact map per seeded
    sequence (1024 beads, 256 bins) with the batched engine, train the
    network on 90 % of them with its own tensor-core kernels, and score 64
    held-out sequences against their truth: the mean map of `truth_reps`
    fresh replicas each (one map remembers its start: a single replica's P(s)
    is ~15 % off its sequence's expectation, so the truth is a replica mean).
    Beside the network: the training set's mean map and a power-law P(s)
    fitted to it (the methods without the network), and one simulation of the
    same length (what simulating instead gives). Then time batched inference
    with the inputs on the device and through the C ABI with host buffers, and
    screen `screen_n` new sequences with a 1 % + out-of-envelope simulation
    fallback."""
    import torch

    from tfm_gb300 import surrogate as S

    t0 = time.perf_counter()
    types, lad, _ = S.make_sequences(n_seq, SUR_L, seed)
    maps, frames = S.simulate_maps(types, lad, SUR_M, sim_steps, burn, every, seed=100)
    t_sim = time.perf_counter() - t0
    nh = max(n_truth, n_seq // 10)
    ntr = n_seq - nh
    held = np.arange(ntr, n_seq, dtype=np.int32)
    k = min(n_truth, nh)
    t0 = time.perf_counter()
    truth, _ = S.simulate_maps(types[ntr:ntr + k], lad[ntr:ntr + k], SUR_M, sim_steps, burn,
                               every, seed=20000, reps=truth_reps)
    t_truth = time.perf_counter() - t0
    mean_map = maps[:ntr].mean(axis=0, keepdims=True)
    power_law = S.powerlaw_map(maps[:ntr])
    B = 32
    steps_total = epochs * max(1, ntr // B)
    net = S.Surrogate("batch %d\nlr 1e-3\nlr_min 1e-4\nlr_steps %d\n" % (B, steps_total), seed=3)
    net.set_dataset(types, lad, maps)
    t1 = time.perf_counter()
    hist = S.train(net, ntr, epochs, seed=5, eval_rows=held)
    t_train = time.perf_counter() - t1
    pred = net.predict_rows(held[:k])

    def scores(m):
        m = np.asarray(m)
        if m.shape[0] == 1:
            m = np.repeat(m, k, 0)
        return {"ps_error": float(S.ps_error(m, truth).mean()),
                "map_log10_mae": float(S.map_log_error(m, truth).mean())}

    one = scores(maps[ntr:ntr + k])
    net_sc = scores(pred)
    # replicas a simulation needs to match the network's P(s) error, from the
    # single-replica error (the replica mean's error falls as 1 / sqrt(reps))
    reps_equal = max(1.0, (one["ps_error"] / max(net_sc["ps_error"], 1e-12)) ** 2)
    rep = {
        "workload": "c3: %d seeded two-type sequences of 1024 beads (Markov block length U[4, 64], "
                    "10%% LAD), 256^2 contact-probability maps from the batched engine "
                    "(%d + %d Heun steps, %d frames), 10%% held out; truth of %d held-out sequences: "
                    "the mean of %d replicas each" % (n_seq, burn, sim_steps, frames, k, truth_reps),
        "simulate_s": t_sim, "truth_simulate_s": t_truth, "train_s": t_train, "epochs": epochs,
        "optimizer_steps": steps_total, "heldout_loss": hist[-1].get("heldout_loss"),
        "vs_truth": {"surrogate": net_sc, "training_mean_map": scores(mean_map),
                     "power_law_ps": scores(power_law), "one_simulation": one,
                     "metric": "ps_error: mean over separation octaves [1,2)..[64,128) bins of "
                               "|P_pred - P_truth| / P_truth; map_log10_mae: mean |log10(p + 1e-3)| "
                               "difference over bin pairs"},
        "simulation_replicas_for_equal_ps_error": reps_equal,
    }
    # inference: a handle of batch SUR_INFER_BATCH with the trained weights
    # (training keeps c3's batch of 32; serving takes bigger batches, which
    # fill the GPU better in the encoder); inputs resident, batches of rows
    IB = SUR_INFER_BATCH
    inf = S.Surrogate("batch %d\n" % IB, seed=3)
    inf.set_params(net.params())
    inf.set_dataset(types, lad, maps)
    train_flags = net.error_flags()
    net.close()
    st = torch.cuda.ExternalStream(inf.stream())
    rows = np.arange(n_seq, dtype=np.int32)
    nb = max(4, 2048 // IB)
    for i in range(3):
        inf.predict_rows(rows[(i * IB) % (n_seq - IB + 1):][:IB], copy=False)
    inf.synchronize()
    clocks = Clocks(0)
    clocks.start()
    k0 = inf.kernel_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for i in range(nb):
        a = (i * IB) % (n_seq - IB + 1)
        inf.predict_rows(rows[a:a + IB], copy=False)
    e1.record(st)
    inf.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    maps_s = nb * IB / (ms / 1000.0)
    peak, kind = bf16_peak()
    tflops = maps_s * SUR_FWD_FLOP / 1e12
    sim_maps_s = bead_steps_per_s / (SUR_L * SIM_STEPS_PER_MAP)
    # end to end: host sequences in, host maps out
    tt, tl = types[:512], lad[:512]
    inf.predict(tt[:IB], tl[:IB])
    t2 = time.perf_counter()
    inf.predict(tt, tl)
    e2e = 512 / (time.perf_counter() - t2)
    net = inf  # screening below runs on the inference handle
    rep.update({
        "maps_per_s": maps_s, "inference_batch": IB, "ms_per_batch": ms / nb,
        "gpu_launches_per_batch": (inf.kernel_count() - k0) / nb,
        "clocks": clk,
        "roofline": {"bound": "tensor", "kernel": "forward pass (head 3x3 convolutions dominate)",
                     "achieved": tflops, "peak": peak, "peak_kind": kind, "unit": "TFLOP/s",
                     "frac": tflops / peak, "gflop_per_map": SUR_FWD_FLOP / 1e9},
        "e2e_maps_per_s": e2e,
        "simulated_maps_per_s": sim_maps_s,
        "speedup_vs_simulation": maps_s / sim_maps_s,
        "speedup_basis": "simulation of one 1024-bead map for %d Heun steps at the batched engine's "
                         "measured bead-steps/s" % SIM_STEPS_PER_MAP,
        "speedup_at_equal_ps_error": maps_s / sim_maps_s * reps_equal,
        "speedup_at_equal_ps_error_basis": "the same simulation repeated by the replicas needed to "
                                           "reach the network's P(s) error against the truth",
    })
    if screen_n:
        env = S.envelope(maps[:ntr])
        sim = lambda t, l: S.simulate_maps(t, l, SUR_M, sim_steps, burn, every, seed=5000)[0]
        stypes, slad, _ = S.make_sequences(screen_n, SUR_L, seed + 1)
        srep, _ = S.screen(net, stypes, slad, env, 0.01, seed=11, sim=sim)
        rep["screening"] = dict(srep, workload="c4: %d new seeded sequences, 1%% random + "
                                               "out-of-envelope re-simulated" % screen_n)
    rep["error_flags"] = train_flags | net.error_flags()
    net.close()
    return rep


def persistent_compare(profile_only=False):
    """ms per Heun step and bead-steps/s of the graph path (`persistent 0`)
    and the persistent per-system kernel (`persistent 1`) on single systems
    and batches of small systems (baseline field), one JSON line per
    workload. profile_only: just 4 x 2048 beads on the persistent kernel,
    two launches of 20 steps (a small case for profiler captures)."""
    from tfm_gb300.ccpgpu import Batch

    text = "force_field baseline\ncontact_bins 256\nsteps_per_frame 100\n"
    if profile_only:
        # the start comes from the graph path, so every persistent launch is
        # a dynamics launch (the relaxation would run on it too)
        a = Batch(text, [2048] * 4, seeds=[1, 2, 3, 4])
        a.generate_initial_condition()
        b = Batch(text + "persistent 1\n", [2048] * 4, seeds=[1, 2, 3, 4])
        b.set_types(a.types())
        b.set_lbs(a.lbs())
        b.set_positions(a.positions())
        a.close()
        for _ in range(2):
            b.advance(20, 0)
            b.synchronize()
        b.close()
        return
    cases = [("one 2048-bead chain", [2048]), ("one 1024-bead chain", [1024]),
             ("one 2900-bead chain", [2900]), ("512 x 1024 beads", [1024] * 512),
             ("4096 x 1024 beads", [1024] * 4096)]
    for name, sizes in cases:
        row = {"workload": name}
        for p in (0, 1):
            b = Batch(text + "persistent %d\n" % p, sizes,
                      seeds=np.arange(len(sizes), dtype=np.uint64) + 1)
            b.generate_initial_condition()
            row["persistent_reach_%d" % p] = b.info().persistent_reach
            b.advance(200, 0)
            b.synchronize()
            n = 2000 if len(sizes) < 100 else 400
            t0 = time.perf_counter()
            b.advance(n, 100)
            b.synchronize()
            dt = time.perf_counter() - t0
            key = "persistent" if p else "graph"
            row[key + "_ms_per_step"] = 1e3 * dt / n
            row[key + "_bead_steps_per_s"] = sum(sizes) * n / dt
            b.close()
        print(json.dumps(row), flush=True)


def surrogate_profile_case():
    """A small surrogate workload for profiler captures: batch 16 of the
    default network (1024 beads, 256 bins), two batched predictions and one
    training step on a synthetic dataset."""
    from tfm_gb300 import surrogate as S

    net = S.Surrogate("batch 16\n", seed=1)
    types, lad, _ = S.make_sequences(16, SUR_L, 1)
    i = np.arange(SUR_M)
    base = (0.5 / (1.0 + np.abs(i[:, None] - i[None, :])) ** 1.1).astype(np.float32)
    net.set_dataset(types, lad, np.repeat(base[None], 16, 0))
    rows = np.arange(16, dtype=np.int32)
    for _ in range(2):
        net.predict_rows(rows, copy=False)
    net.train_step(rows, want_loss=False)
    net.synchronize()
    if net.error_flags():
        raise RuntimeError("surrogate kernels reported a pipeline timeout")
    net.close()
    print("surrogate profile case done")


def surrogate_arm(args, rank, local):
    import torch

    from tfm_gb300 import build as eb

    eb.build()
    torch.cuda.set_device(local)
    if rank != 0:
        return
    rep = surrogate_report(args.sim_rate, args.sur_sequences, args.sur_sim_steps, args.sur_epochs, 32,
                           args.sur_screen)
    line = {"metric": "surrogate contact maps/s (batched BF16 inference, 1 GB300)", "value": rep["maps_per_s"],
            "unit": "maps/s", "n_gpus": 1, "higher_is_better": True, "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic (seeded sequences, maps simulated by the engine)",
            "config": {"workload": rep["workload"]}}
    line.update({k: v for k, v in rep.items() if k not in ("maps_per_s", "workload")})
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--replicas", type=int, default=512)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--split", action="store_true",
                    help="split one ensemble of --replicas over the GPUs (strong scaling) "
                         "instead of one ensemble per GPU")
    ap.add_argument("--no-tune", action="store_true", help="skip the per-class autotuner")
    ap.add_argument("--no-ref-gpu", dest="ref_gpu", action="store_false",
                    help="reference arm: skip timing ccp's own kernels on the GPU")
    ap.add_argument("--pair-kernel", type=int, default=None,
                    help="engine pair kernel (parameter pair_kernel); default: the engine's")
    ap.add_argument("--surrogate", action="store_true",
                    help="measure the surrogate on the c3/c4 protocol instead of the engine")
    ap.add_argument("--sur-profile", action="store_true",
                    help="run only a small surrogate workload (for profiler captures)")
    ap.add_argument("--persist-compare", action="store_true",
                    help="time the graph path against the persistent per-system kernel")
    ap.add_argument("--persist-profile", action="store_true",
                    help="run only a small persistent-kernel workload (for profiler captures)")
    ap.add_argument("--sur-sequences", type=int, default=4096)
    ap.add_argument("--sur-sim-steps", type=int, default=20000)
    ap.add_argument("--sur-epochs", type=int, default=20)
    ap.add_argument("--sur-screen", type=int, default=100000)
    ap.add_argument("--sim-rate", type=float, default=2.7e9,
                    help="batched bead-steps/s used to cost a simulated map (from the engine bench)")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.persist_compare or args.persist_profile:
        from tfm_gb300 import build as eb

        eb.build()
        persistent_compare(profile_only=args.persist_profile)
    elif args.sur_profile:
        from tfm_gb300 import build as eb

        eb.build()
        surrogate_profile_case()
    elif args.surrogate:
        surrogate_arm(args, rank, local)
    elif args.impl == "reference":
        reference_arm(args, ws, rank)
    else:
        engine_arm(args, ws, rank, local)
    from tfm_gb300 import replicas

    replicas.finalize(ws)


if __name__ == "__main__":
    main()
