"""Python binding of libccpgpu.so (include/ccpgpu.h) through ctypes.

`ChrSim` mirrors the public interface of ccp's mmc::chrsim
(Program/src/chrsim.cuh:36-56 and the frame I/O of chrdat.cuh:81-100):
construction from the adjustable-parameters text, generate_initial_condition,
save_checkpoint / load_checkpoint, run_simulation and write_frame_txt /
write_lbs_txt, with file objects where ccp takes std::fstream. Errors raise
`CcpError` carrying ccp's message (the mmc::error of util.cuh:52-59).

`Batch` exposes the multi-replica engine. There is no CPU fallback: when the
shared library is missing or cannot be loaded the import fails.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libccpgpu.so")

OK, ERR_PARAM, ERR_CUDA, ERR_IO, ERR_STATE, ERR_ARG = range(6)

# every exported symbol of include/ccpgpu.h
SYMBOLS = (
    "ccpgpu_create", "ccpgpu_batch_create", "ccpgpu_destroy", "ccpgpu_last_error",
    "ccpgpu_info_get", "ccpgpu_system_info_get", "ccpgpu_generate_initial_condition",
    "ccpgpu_run_simulation", "ccpgpu_run_steps", "ccpgpu_error_flags",
    "ccpgpu_get_positions", "ccpgpu_set_positions", "ccpgpu_get_types", "ccpgpu_set_types",
    "ccpgpu_get_lbs", "ccpgpu_set_lbs", "ccpgpu_compute_forces", "ccpgpu_frame_txt",
    "ccpgpu_lbs_txt", "ccpgpu_frame_trr", "ccpgpu_checkpoint", "ccpgpu_load_checkpoint",
    "ccpgpu_read_frame_txt", "ccpgpu_read_lbs_txt", "ccpgpu_observe",
    "ccpgpu_reset_observables", "ccpgpu_contact_counts", "ccpgpu_observable_sums",
    "ccpgpu_separation_counts", "ccpgpu_overlaps", "ccpgpu_advance", "ccpgpu_synchronize",
    "ccpgpu_stream_handle", "ccpgpu_kernel_times", "ccpgpu_kernel_count",
    "ccpgpu_forces_noalloc", "ccpgpu_noalloc_error_flags", "ccpgpu_autotune",
    "ccpgpu_analysis_frame", "ccpgpu_analysis_series",
    "ccpgpu_analysis_end_simulation", "ccpgpu_analysis_txt", "ccpgpu_analysis_fin_txt",
    "ccpgpu_contact_map_bin", "ccpgpu_random_walk",
)

NOALLOC_MAX_BEADS = 32768
NOALLOC_MAX_CELLS = 131072


class NoallocSystem(C.Structure):
    _fields_ = [("preset", C.c_int32), ("n_beads", C.c_int32), ("n_chains", C.c_int32),
                ("nucleus_radius", C.c_float)]


class CcpError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class Info(C.Structure):
    _fields_ = [("n_systems", C.c_int32), ("n_beads", C.c_int32), ("n_lbs", C.c_int32),
                ("n_chains", C.c_int32), ("n_cells", C.c_int32), ("preset", C.c_int32),
                ("frames_per_file", C.c_uint32), ("steps_per_frame", C.c_uint32),
                ("frame_index", C.c_uint32), ("time", C.c_float), ("step", C.c_uint64),
                ("dt", C.c_float), ("kT", C.c_float), ("noise_sd", C.c_float),
                ("contact_cutoff", C.c_float), ("frames_observed", C.c_int32),
                ("persistent_reach", C.c_int32)]


class SystemInfo(C.Structure):
    _fields_ = [("bead_offset", C.c_int32), ("n_beads", C.c_int32),
                ("chain_offset", C.c_int32), ("n_chains", C.c_int32),
                ("lbs_offset", C.c_int32), ("n_lbs", C.c_int32),
                ("cells_per_side", C.c_int32), ("cell_side", C.c_float),
                ("nucleus_radius", C.c_float), ("opening_radius", C.c_float),
                ("bleb_radius", C.c_float), ("contact_bins", C.c_int32),
                ("map_len", C.c_int32), ("copy_len", C.c_int32), ("n_copies", C.c_int32),
                ("map_offset", C.c_int64), ("seed", C.c_uint64)]


FRAME_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint32, C.c_float,
                       C.POINTER(C.c_float), C.c_int32)

_lib = None


def load(path=LIB_PATH):
    """Loads the engine library; raises OSError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libccpgpu.so not built: run __graft_entry__.build() (%s)" % path)
    lib = C.CDLL(path)
    P, I32, U32, U64, SZ = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64, C.c_size_t
    sig = {
        "ccpgpu_create": [C.c_char_p, U64, C.POINTER(P)],
        "ccpgpu_batch_create": [C.c_char_p, I32, P, P, P, P, U64, C.POINTER(P)],
        "ccpgpu_destroy": [P],
        "ccpgpu_info_get": [P, C.POINTER(Info)],
        "ccpgpu_system_info_get": [P, I32, C.POINTER(SystemInfo)],
        "ccpgpu_generate_initial_condition": [P],
        "ccpgpu_random_walk": [P, P, SZ],
        "ccpgpu_run_simulation": [P, FRAME_FN, P],
        "ccpgpu_run_steps": [P, U64, U32],
        "ccpgpu_error_flags": [P, P, I32],
        "ccpgpu_get_positions": [P, P, SZ], "ccpgpu_set_positions": [P, P, SZ],
        "ccpgpu_get_types": [P, P, SZ], "ccpgpu_set_types": [P, P, SZ],
        "ccpgpu_get_lbs": [P, P, SZ], "ccpgpu_set_lbs": [P, P, SZ],
        "ccpgpu_compute_forces": [P, P, SZ],
        "ccpgpu_frame_txt": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_lbs_txt": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_frame_trr": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_checkpoint": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_load_checkpoint": [P, I32, P, SZ],
        "ccpgpu_read_frame_txt": [P, I32, C.c_char_p, SZ],
        "ccpgpu_read_lbs_txt": [P, I32, C.c_char_p, SZ],
        "ccpgpu_observe": [P, I32], "ccpgpu_reset_observables": [P],
        "ccpgpu_contact_counts": [P, I32, P, SZ],
        "ccpgpu_observable_sums": [P, I32, P, SZ],
        "ccpgpu_separation_counts": [P, I32, P, P, SZ],
        "ccpgpu_overlaps": [P, P, SZ],
        "ccpgpu_advance": [P, U64, U32], "ccpgpu_synchronize": [P],
        "ccpgpu_stream_handle": [P, C.POINTER(P)],
        "ccpgpu_kernel_times": [P, I32, P, SZ],
        "ccpgpu_kernel_count": [P, C.POINTER(C.c_uint64)],
        "ccpgpu_forces_noalloc": [C.POINTER(NoallocSystem), P, P, P, P],
        "ccpgpu_noalloc_error_flags": [P, P],
        "ccpgpu_autotune": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_analysis_frame": [P], "ccpgpu_analysis_end_simulation": [P],
        "ccpgpu_analysis_series": [P, I32, P, SZ, C.POINTER(I32)],
        "ccpgpu_analysis_txt": [P, I32, P, SZ, C.POINTER(SZ)],
        "ccpgpu_analysis_fin_txt": [P, P, SZ, C.POINTER(SZ)],
        "ccpgpu_contact_map_bin": [P, P, SZ, C.POINTER(SZ)],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.ccpgpu_last_error.argtypes = []
    lib.ccpgpu_last_error.restype = C.c_char_p
    _lib = lib
    return lib


def _check(rc):
    if rc != OK:
        raise CcpError(rc, _lib.ccpgpu_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class _Handle:
    def __init__(self):
        self._h = C.c_void_p()

    def close(self):
        if self._h:
            _check(_lib.ccpgpu_destroy(self._h))
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

    # ---------------------------------------------------------------- info
    def info(self):
        i = Info()
        _check(_lib.ccpgpu_info_get(self._h, C.byref(i)))
        return i

    def system_info(self, s=0):
        i = SystemInfo()
        _check(_lib.ccpgpu_system_info_get(self._h, s, C.byref(i)))
        return i

    @property
    def n_beads(self):
        return self.info().n_beads

    # ---------------------------------------------------------------- state
    def positions(self):
        a = np.empty((self.n_beads, 3), np.float32)
        _check(_lib.ccpgpu_get_positions(self._h, _ptr(a), a.size))
        return a

    def set_positions(self, xyz):
        a = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        _check(_lib.ccpgpu_set_positions(self._h, _ptr(a), a.size))

    def types(self):
        a = np.empty(self.n_beads, np.int32)
        _check(_lib.ccpgpu_get_types(self._h, _ptr(a), a.size))
        return a

    def set_types(self, pt):
        a = np.ascontiguousarray(pt, np.int32)
        _check(_lib.ccpgpu_set_types(self._h, _ptr(a), a.size))

    def lbs(self):
        n = self.info().n_lbs
        a = np.empty((n, 3), np.float32)
        _check(_lib.ccpgpu_get_lbs(self._h, _ptr(a) if n else None, a.size))
        return a

    def set_lbs(self, xyz):
        a = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        _check(_lib.ccpgpu_set_lbs(self._h, _ptr(a) if a.size else None, a.size))

    def forces(self):
        a = np.empty((self.n_beads, 3), np.float32)
        _check(_lib.ccpgpu_compute_forces(self._h, _ptr(a), a.size))
        return a

    def generate_initial_condition(self):
        _check(_lib.ccpgpu_generate_initial_condition(self._h))

    def random_walk(self):
        """Confined random walk of every chain (no relaxation); returns each
        chain's number of attempts."""
        d = np.zeros(self.info().n_chains, np.uint32)
        _check(_lib.ccpgpu_random_walk(self._h, _ptr(d), d.size))
        return d

    def run_steps(self, n, observe_every=0):
        _check(_lib.ccpgpu_run_steps(self._h, int(n), int(observe_every)))

    def advance(self, n, observe_every=0):
        """Enqueue n steps without waiting (device-resident stepping)."""
        _check(_lib.ccpgpu_advance(self._h, int(n), int(observe_every)))

    def synchronize(self):
        _check(_lib.ccpgpu_synchronize(self._h))

    def stream(self):
        s = C.c_void_p()
        _check(_lib.ccpgpu_stream_handle(self._h, C.byref(s)))
        return s.value or 0

    KERNELS = ("scan", "scatter", "pair", "update1", "update2", "contacts", "observe")

    def kernel_times(self, reps=5):
        a = np.zeros(7, np.float64)
        _check(_lib.ccpgpu_kernel_times(self._h, int(reps), _ptr(a), a.size))
        return dict(zip(self.KERNELS, a.tolist()))

    def autotune(self, reps=5):
        """Per-size-class cell side and tile size by timing; returns the report."""
        import json

        n = C.c_size_t()
        buf = C.create_string_buffer(1 << 16)
        _check(_lib.ccpgpu_autotune(self._h, int(reps), buf, len(buf), C.byref(n)))
        return json.loads(buf.value.decode())

    def kernel_count(self):
        c = C.c_uint64()
        _check(_lib.ccpgpu_kernel_count(self._h, C.byref(c)))
        return c.value

    def error_flags(self, clear=False):
        a = np.zeros(8, np.int32)
        rc = _lib.ccpgpu_error_flags(self._h, _ptr(a), 1 if clear else 0)
        return a, rc

    # ---------------------------------------------------------------- observables
    def observe(self, with_sdist=False):
        _check(_lib.ccpgpu_observe(self._h, 1 if with_sdist else 0))

    def reset_observables(self):
        _check(_lib.ccpgpu_reset_observables(self._h))

    def contact_counts(self, s=0):
        nb = self.system_info(s).contact_bins
        a = np.empty(nb * (nb + 1) // 2, np.int32)
        _check(_lib.ccpgpu_contact_counts(self._h, s, _ptr(a), a.size))
        return a

    def observable_sums(self, s=0):
        a = np.empty(4 + 3 * 64, np.float64)
        _check(_lib.ccpgpu_observable_sums(self._h, s, _ptr(a), a.size))
        return a

    def separation_counts(self, chain, length):
        m = length // 2 + 1
        c = np.empty(m, np.int32)
        d = np.empty(m, np.float64)
        _check(_lib.ccpgpu_separation_counts(self._h, chain, _ptr(c), _ptr(d), m))
        return c, d

    def overlaps(self):
        a = np.empty(self.info().n_systems, np.uint64)
        _check(_lib.ccpgpu_overlaps(self._h, _ptr(a), a.size))
        return a

    # ---------------------------------------------------------------- formats
    def _bytes(self, fn, s):
        n = C.c_size_t()
        fn(self._h, s, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        _check(fn(self._h, s, buf, n.value, C.byref(n)))
        return buf.raw[: n.value]

    def frame_txt(self, s=0):
        return self._bytes(_lib.ccpgpu_frame_txt, s)

    def lbs_txt(self, s=0):
        return self._bytes(_lib.ccpgpu_lbs_txt, s)

    def frame_trr(self, s=0):
        return self._bytes(_lib.ccpgpu_frame_trr, s)

    def checkpoint(self, s=0):
        return self._bytes(_lib.ccpgpu_checkpoint, s)

    def load_checkpoint_bytes(self, b, s=0):
        buf = C.create_string_buffer(b, len(b))
        _check(_lib.ccpgpu_load_checkpoint(self._h, s, buf, len(b)))

    # ---------------------------------------------------------------- analysis
    def analysis_frame(self):
        """One ccp-analyze frame of every system at the current positions."""
        _check(_lib.ccpgpu_analysis_frame(self._h))

    def analysis_series(self, s=0):
        """Series [4 + 3*64][frames] of system s's current simulation."""
        f = C.c_int32()
        _check(_lib.ccpgpu_analysis_series(self._h, s, None, 0, C.byref(f)))
        out = np.empty((4 + 3 * 64, f.value), np.float32)
        _check(_lib.ccpgpu_analysis_series(self._h, s, _ptr(out), out.size, C.byref(f)))
        return out

    def analysis_end_simulation(self):
        """Ends every system's simulation: statistics, then cleared buffers."""
        _check(_lib.ccpgpu_analysis_end_simulation(self._h))

    def analysis_txt(self, s=0):
        """analysis-XXX.dat of system s's last simulation (bytes)."""
        return self._bytes(_lib.ccpgpu_analysis_txt, s)

    def _bytes0(self, fn):
        n = C.c_size_t()
        fn(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        _check(fn(self._h, buf, n.value, C.byref(n)))
        return buf.raw[: n.value]

    def analysis_fin_txt(self):
        """analysis-fin.dat over every simulation so far (bytes)."""
        return self._bytes0(_lib.ccpgpu_analysis_fin_txt)

    def contact_map_bin(self):
        """contact-map.bin: float64 contact-map averages over simulations (bytes)."""
        return self._bytes0(_lib.ccpgpu_contact_map_bin)

    def read_frame_txt_bytes(self, b, s=0):
        _check(_lib.ccpgpu_read_frame_txt(self._h, s, b, len(b)))

    def read_lbs_txt_bytes(self, b, s=0):
        _check(_lib.ccpgpu_read_lbs_txt(self._h, s, b, len(b)))


class ChrSim(_Handle):
    """ccp's chrsim (chrsim.cuh:36-56) over the GPU engine."""

    def __init__(self, param_text, seed=0):
        super().__init__()
        load()
        _check(_lib.ccpgpu_create(param_text.encode(), int(seed), C.byref(self._h)))

    # chrsim::save_checkpoint / load_checkpoint (chrsim.cu:525-555)
    def save_checkpoint(self, f):
        f.write(self.checkpoint(0))

    def load_checkpoint(self, f):
        self.load_checkpoint_bytes(f.read(), 0)

    # chrdat::write_frame_txt / write_lbs_txt / write_frame_bin
    def write_frame_txt(self, f):
        f.write(self.frame_txt(0).decode())

    def write_lbs_txt(self, f):
        f.write(self.lbs_txt(0).decode())

    def write_frame_bin(self, f):
        f.write(self.frame_trr(0))

    def read_frame_txt(self, f):
        self.read_frame_txt_bytes(f.read().encode() if isinstance(f.read(0), str) else f.read(), 0)

    # chrsim::run_simulation (chrsim.cu:558-593): one .trr frame per spf steps
    def run_simulation(self, f, on_frame=None):
        def cb(_user, i_f, t, xyz, n):
            try:
                a = np.ctypeslib.as_array(xyz, shape=(n * 3,))
                if f is not None:
                    f.write(_trr_frame(i_f, t, a, n))
                if on_frame is not None:
                    on_frame(i_f, t, a.reshape(n, 3).copy())
                return 0
            except Exception:
                return 1

        fn = FRAME_FN(cb)
        _check(_lib.ccpgpu_run_simulation(self._h, fn, None))


def forces_noalloc(preset, n_beads, n_chains, nucleus_radius, d_xyz, d_types, d_forces,
                   stream=0):
    """ccpgpu_forces_noalloc on caller-owned device buffers (raw device
    addresses as ints); allocates no device memory. Returns the status code."""
    load()
    s = NoallocSystem(int(preset), int(n_beads), int(n_chains), float(nucleus_radius))
    return _lib.ccpgpu_forces_noalloc(C.byref(s), C.c_void_p(d_xyz), C.c_void_p(d_types),
                                      C.c_void_p(d_forces), C.c_void_p(stream or None))


def noalloc_error_flags(stream=0):
    """(status, flags[8]) of the last forces_noalloc call on the current device,
    after the given stream has run it."""
    load()
    a = np.zeros(8, np.int32)
    rc = _lib.ccpgpu_noalloc_error_flags(_ptr(a), C.c_void_p(stream or None))
    return rc, a


def last_error():
    load()
    return _lib.ccpgpu_last_error().decode()


def _trr_frame(i_f, t, xyz, n):
    hdr = np.zeros(18, np.uint32)
    hdr[0], hdr[1], hdr[10], hdr[13], hdr[14] = 1993, 1, 3 * n * 4, n, i_f
    hdr[16] = np.array([t], np.float32).view(np.uint32)[0]
    return hdr.tobytes() + np.asarray(xyz, np.float32).tobytes()


class Batch(_Handle):
    """Independent replicas advanced together (no reference counterpart)."""

    def __init__(self, param_text, n_beads, n_chains=None, radii=None, seeds=None, seed=0):
        super().__init__()
        load()
        nb = np.ascontiguousarray(n_beads, np.int32)
        ns = len(nb)
        nc = None if n_chains is None else np.ascontiguousarray(n_chains, np.int32)
        rd = None if radii is None else np.ascontiguousarray(radii, np.float32)
        sd = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
        # the C side reads one entry per system from each array
        if nb.ndim != 1 or ns == 0:
            raise ValueError("n_beads must be a non-empty list of bead counts")
        for name, a in (("n_chains", nc), ("radii", rd), ("seeds", sd)):
            if a is not None and a.shape != (ns,):
                raise ValueError("%s must have one entry per system (%d)" % (name, ns))
        self._keep = (nb, nc, rd, sd)
        _check(_lib.ccpgpu_batch_create(
            param_text.encode(), ns, _ptr(nb), None if nc is None else _ptr(nc),
            None if rd is None else _ptr(rd), None if sd is None else _ptr(sd), int(seed),
            C.byref(self._h)))
