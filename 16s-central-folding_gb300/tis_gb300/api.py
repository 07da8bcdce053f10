"""ctypes binding of the C ABI in include/tis_gpu.h (libtis_gpu.so).

The product path is the CUDA library; nothing here computes physics.  Loading
fails loudly when the library is missing."""
import ctypes as C
import os

import numpy as np

from . import build as _build

F64, I32, I64 = 0, 1, 2
_NP = {F64: np.float64, I32: np.int32, I64: np.int64}
STATE_NAMES = ["x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"]
ENERGY_NAMES = ["E_lj", "E_coul_sr", "E_coul_lr", "E_bond", "E_angle", "E_excl",
                "E2_STACK", "E3_STACK", "E2_HB", "E3_HB", "Rg"]
TERM_SR, TERM_LR, TERM_BONDED, TERM_STACK, TERM_HB = 1, 2, 4, 8, 16
# force-field parameters of tis_param_grad / tis_traj_grad (TIS_N_PARAMS, in order)
PARAM_NAMES = ["ss_D_A", "ss_D_C", "ss_D_G", "ss_D_U", "st_D", "hs_D", "eps_P", "eps_S", "eps_B", "eps_Mg", "eps_Cl",
               "eps_K", "R_Mg", "R_K", "lB", "debye"]
N_PARAMS = len(PARAM_NAMES)
PREC_MIXED, PREC_FP64 = 0, 1
NOISE_REFERENCE, NOISE_OFF = 0, 1


class TisError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"tis error {code}: {msg}")
        self.code = code


class LoadParams(C.Structure):
    _fields_ = [("pdb", C.c_char_p), ("bonds", C.c_char_p), ("stacks", C.c_char_p), ("maxikey", C.c_char_p),
                ("T", C.c_double), ("ss_D", C.c_double), ("hs_D", C.c_double), ("st_D", C.c_double),
                ("seed", C.c_int32), ("box", C.c_double), ("rc", C.c_double), ("c_mg", C.c_double),
                ("c_k", C.c_double), ("n_mg", C.c_int32), ("n_cl", C.c_int32), ("n_k", C.c_int32),
                ("center", C.c_int32), ("rng", C.c_int32), ("reserved", C.c_int32 * 7)]


class RunParams(C.Structure):
    _fields_ = [("precision", C.c_int32), ("noise", C.c_int32), ("sr", C.c_double), ("skin", C.c_double),
                ("lr_interval", C.c_int32), ("cap_sr", C.c_int32), ("cap_lr", C.c_int32), ("device", C.c_int32),
                ("use_graph", C.c_int32), ("graph_steps", C.c_int32), ("full_lists", C.c_int32),
                ("groups", C.c_int32), ("lanes_sr", C.c_int32), ("lanes_lr", C.c_int32),
                ("fused_ctas", C.c_int32), ("reserved", C.c_int32 * 1)]


_lib = None


def lib(build_if_missing=True):
    """The loaded libtis_gpu.so (built in-tree on first use)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            _build.build()  # no-op when the library is newer than its sources
        if not os.path.exists(path):
            raise OSError(f"{path} is missing; run the build first")
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def _declare(L):
    vp, i32, i64, dp, ip, cp = C.c_void_p, C.c_int, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_char_p
    sig = {
        "tis_last_error": [cp, C.c_size_t],
        "tis_load_params_default": [C.POINTER(LoadParams)],
        "tis_system_load": [C.POINTER(LoadParams), C.POINTER(vp)],
        "tis_system_new": [C.POINTER(vp)],
        "tis_system_set": [vp, cp, i32, vp, i64],
        "tis_system_get": [vp, cp, C.POINTER(C.c_int), C.POINTER(vp), C.POINTER(C.c_int64)],
        "tis_system_count": [vp, C.POINTER(C.c_int)],
        "tis_system_name": [vp, i32, C.POINTER(C.c_char_p)],
        "tis_system_destroy": [vp],
        "tis_run_params_default": [C.POINTER(RunParams)],
        "tis_create": [C.POINTER(vp), i32, C.POINTER(RunParams), C.POINTER(vp)],
        "tis_destroy": [vp],
        "tis_set_state": [vp, i32] + [dp] * 9,
        "tis_get_state": [vp, i32] + [dp] * 9,
        "tis_set_states": [vp] + [dp] * 9,
        "tis_get_states": [vp] + [dp] * 9,
        "tis_get_all_energies": [vp, dp],
        "tis_write_frame": [vp, i32, cp, cp, cp],
        "tis_ion_counts": [vp, i32, i32, C.c_double, ip, i64, C.POINTER(C.c_int64), ip],
        "tis_read_last_frame": [cp, i32, dp, dp, dp, C.POINTER(C.c_int64)],
        "tis_populate_lists": [vp],
        "tis_get_cells": [vp, i32, ip, ip],
        "tis_get_pairs": [vp, i32, i32, ip, i64, C.POINTER(C.c_int64)],
        "tis_get_hb_status": [vp, i32, ip, ip],
        "tis_compute_forces": [vp, i32, i32, dp, dp],
        "tis_deterministic_forces": [vp],
        "tis_full_forces": [vp],
        "tis_move_rigid_units": [vp],
        "tis_check_shifts": [vp],
        "tis_step": [vp, i64],
        "tis_sync": [vp],
        "tis_get_energies": [vp, i32, dp],
        "tis_get_stack_energies": [vp, i32, dp, i64, C.POINTER(C.c_int64)],
        "tis_get_counters": [vp, i32, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
        "tis_get_info": [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(vp)],
        "tis_replica_size": [vp, i32, C.POINTER(C.c_int)],
        "tis_get_launch_count": [vp, C.POINTER(C.c_int64)],
        "tis_rand_stream": [C.c_uint64, C.c_uint64, i64, ip],
        "tis_profile_stages": [vp, i64, dp],
        "tis_profile_in_step": [vp, i32, dp],
        "tis_profile_fused": [vp, i32, i32, dp],
        "tis_frames_start": [vp, i32, i32, C.POINTER(vp)],
        "tis_frames_read": [vp, i64, dp, dp, dp, dp],
        "tis_frames_stop": [vp],
        "tis_get_forces": [vp, i32, dp],
        "tis_pair_lists_noalloc": [vp, vp, vp, vp, C.c_int32, dp, C.c_double, C.c_double, vp, i64, vp, i64, vp, vp],
        "tis_param_grad": [vp, dp],
        "tis_autotune": [C.POINTER(vp), i32, C.POINTER(RunParams), i64, cp, C.POINTER(RunParams), dp],
        "tis_density_create": [vp, i32, i32, dp, C.c_double, ip, i32, ip, dp, C.POINTER(vp)],
        "tis_density_add": [vp],
        "tis_density_get": [vp, dp, i64, C.POINTER(C.c_int64), dp],
        "tis_density_write_dx": [vp, cp],
        "tis_density_destroy": [vp],
        "tis_write_psf": [vp, cp],
        "tis_write_cgpdb": [vp, dp, dp, dp, cp],
        "tis_write_ninfo": [vp, cp],
        "tis_capture_graph": [vp, i32],
        "tis_checkpoint_save": [vp, cp],
        "tis_checkpoint_load": [vp, cp],
        "tis_write_dcd": [vp, i32, cp, i32, C.c_double],
        "tis_traj_grad": [vp, i64, i32, C.POINTER(dp), dp, C.POINTER(dp)],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int


EXPORTED = ["tis_last_error", "tis_load_params_default", "tis_system_load", "tis_system_new", "tis_system_set",
            "tis_system_get", "tis_system_count", "tis_system_name", "tis_system_destroy", "tis_run_params_default",
            "tis_create", "tis_destroy", "tis_set_state", "tis_get_state", "tis_populate_lists", "tis_get_cells",
            "tis_get_pairs", "tis_get_hb_status", "tis_compute_forces", "tis_deterministic_forces", "tis_full_forces",
            "tis_move_rigid_units", "tis_check_shifts", "tis_step", "tis_sync", "tis_get_energies",
            "tis_get_stack_energies", "tis_get_counters", "tis_get_info", "tis_replica_size", "tis_get_launch_count",
            "tis_rand_stream", "tis_profile_stages", "tis_get_forces", "tis_pair_lists_noalloc", "tis_set_states",
            "tis_get_states", "tis_get_all_energies", "tis_write_frame", "tis_read_last_frame", "tis_ion_counts",
            "tis_param_grad", "tis_traj_grad", "tis_autotune", "tis_density_create", "tis_density_add",
            "tis_density_get", "tis_density_write_dx", "tis_density_destroy", "tis_write_psf", "tis_write_dcd", "tis_capture_graph",
            "tis_write_cgpdb", "tis_checkpoint_save", "tis_checkpoint_load", "tis_profile_in_step", "tis_write_ninfo", "tis_profile_fused", "tis_frames_start",
            "tis_frames_read", "tis_frames_stop"]


def read_last_frame(path, n):
    """(x, y, z, frames): the last frame of a reference Coordinates file of n particles."""
    x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)
    frames = C.c_int64()
    _check(lib().tis_read_last_frame(path.encode(), n, _dp(x), _dp(y), _dp(z), C.byref(frames)))
    return x, y, z, frames.value


def pair_lists_noalloc(d_x, d_y, d_z, d_kind, n, box, sr_radius, lr_radius, d_sr, sr_cap, d_lr, lr_cap, d_counts,
                       stream=None):
    """Allocation-free list build on caller-owned device buffers (addresses as ints)."""
    b = np.ascontiguousarray(box, dtype=np.float64)
    _check(lib().tis_pair_lists_noalloc(d_x, d_y, d_z, d_kind, n, _dp(b), sr_radius, lr_radius, d_sr, sr_cap,
                                        d_lr, lr_cap, d_counts, stream))


def rand_stream(seed, first, n):
    """Draws of the Philox rand() stream (values in [1, 2^31-1])."""
    out = np.zeros(max(n, 1), dtype=np.int32)
    _check(lib().tis_rand_stream(seed, first, n, _ip(out)))
    return out[:n]


def _check(rc):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        lib().tis_last_error(buf, 1024)
        raise TisError(rc, buf.value.decode(errors="replace"))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class System:
    """One replica's topology and state (a tis_system)."""

    def __init__(self, handle):
        self.h = C.c_void_p(handle)

    @classmethod
    def load(cls, pdb, bonds, stacks, maxikey, **kw):
        p = LoadParams()
        lib().tis_load_params_default(C.byref(p))
        p.pdb, p.bonds, p.stacks, p.maxikey = (os.fsencode(v) for v in (pdb, bonds, stacks, maxikey))
        for k, v in kw.items():
            setattr(p, k, v)
        out = C.c_void_p()
        _check(lib().tis_system_load(C.byref(p), C.byref(out)))
        return cls(out.value)

    @classmethod
    def from_arrays(cls, arrays):
        out = C.c_void_p()
        _check(lib().tis_system_new(C.byref(out)))
        s = cls(out.value)
        for k, v in arrays.items():
            s[k] = v
        return s

    def __setitem__(self, name, arr):
        arr = np.ascontiguousarray(arr)
        if arr.dtype == np.float64:
            dt = F64
        elif arr.dtype == np.int32:
            dt = I32
        elif arr.dtype == np.int64:
            dt = I64
        else:
            raise TypeError(f"{name}: dtype {arr.dtype} not supported")
        _check(lib().tis_system_set(self.h, name.encode(), dt, arr.ctypes.data_as(C.c_void_p), arr.size))

    def __getitem__(self, name):
        dt, ptr, n = C.c_int(), C.c_void_p(), C.c_int64()
        _check(lib().tis_system_get(self.h, name.encode(), C.byref(dt), C.byref(ptr), C.byref(n)))
        npdt = _NP[dt.value]
        if n.value == 0:
            return np.zeros(0, dtype=npdt)
        buf = (C.c_char * (n.value * np.dtype(npdt).itemsize)).from_address(ptr.value)
        return np.frombuffer(buf, dtype=npdt).copy()

    def names(self):
        n = C.c_int()
        _check(lib().tis_system_count(self.h, C.byref(n)))
        out = []
        for i in range(n.value):
            nm = C.c_char_p()
            _check(lib().tis_system_name(self.h, i, C.byref(nm)))
            out.append(nm.value.decode())
        return out

    def to_dict(self):
        return {k: self[k] for k in self.names()}

    def write_cgpdb(self, path, state=None):
        """The coarse-grained PDB of the reference's exporter (tis_write_cgpdb); state:
        {x, y, z} arrays (None: the system's own coordinates)."""
        if state is None:
            _check(lib().tis_write_cgpdb(self.h, None, None, None, os.fsencode(path)))
        else:
            xyz = [np.ascontiguousarray(state[k], dtype=np.float64) for k in ("x", "y", "z")]
            _check(lib().tis_write_cgpdb(self.h, *[_dp(a) for a in xyz], os.fsencode(path)))

    def write_psf(self, path):
        """The topology in the PSF layout of the reference's exporter (tis_write_psf)."""
        _check(lib().tis_write_psf(self.h, os.fsencode(path)))

    def write_ninfo(self, path):
        """The native-structure information (.ninfo) file of the reference's exporter (tis_write_ninfo)."""
        _check(lib().tis_write_ninfo(self.h, os.fsencode(path)))

    def __del__(self):
        try:
            if self.h:
                lib().tis_system_destroy(self.h)
                self.h = None
        except Exception:
            pass


def autotune(systems, steps=300, cache=None, **params):
    """Measured launch configuration for these replicas stepped `steps` steps per
    call: (dict of the chosen groups, graph_steps, lanes_sr, lanes_lr, fused_ctas;
    replica-steps/s)."""
    arr = (C.c_void_p * len(systems))(*[s.h.value for s in systems])
    base = run_params(**params)
    best = RunParams()
    rate = C.c_double()
    _check(lib().tis_autotune(arr, len(systems), C.byref(base), int(steps),
                              os.fsencode(cache) if cache else None, C.byref(best), C.byref(rate)))
    return {k: getattr(best, k) for k in ("groups", "graph_steps", "lanes_sr", "lanes_lr", "fused_ctas")}, rate.value


class Density:
    """Ion counts of one kind of one replica binned over frames on the device."""

    def __init__(self, engine, r, kind, lo, delta, dims, fit_beads=None, fit_ref=None):
        self.engine = engine  # the handle must outlive the grid
        self.dims = tuple(int(v) for v in dims)
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        dm = np.ascontiguousarray(self.dims, dtype=np.int32)
        nf = 0
        fb = fr = None
        if fit_beads is not None:
            fb = np.ascontiguousarray(fit_beads, dtype=np.int32)
            fr = np.ascontiguousarray(fit_ref, dtype=np.float64).reshape(-1)
            nf = fb.size
        out = C.c_void_p()
        _check(lib().tis_density_create(engine.h, r, kind, _dp(lo), float(delta), dm.ctypes.data_as(C.POINTER(C.c_int32)),
                                        nf, fb.ctypes.data_as(C.POINTER(C.c_int32)) if fb is not None else None,
                                        _dp(fr) if fr is not None else None, C.byref(out)))
        self.h = out

    def add(self):
        _check(lib().tis_density_add(self.h))

    def get(self):
        """(counts array of dims, frames, rmsd of the last fit)."""
        c = np.zeros(self.dims)
        fr = C.c_int64()
        rm = C.c_double()
        _check(lib().tis_density_get(self.h, _dp(c), c.size, C.byref(fr), C.byref(rm)))
        return c, fr.value, rm.value

    def write_dx(self, path):
        _check(lib().tis_density_write_dx(self.h, os.fsencode(path)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().tis_density_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def contact_concentration(count_sum, frames, cut=7.300000001):
    """Contact concentration (mol/L) of particles counted within `cut` A of a
    phosphate, summed over `frames` frames (analysis/salt_nt/integrate_num_ions.py:
    51-55: count / (frames * 4/3 pi cut^3 * 6.02214e-4))."""
    return np.asarray(count_sum, dtype=np.float64) / (float(frames) * 4.0 / 3.0 * np.pi * cut ** 3 * 6.02214 / 1e4)


def run_params(**kw):
    p = RunParams()
    lib().tis_run_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class FrameRing:
    """The frames a handle writes from inside its steps (tis_frames_*)."""

    def __init__(self, engine, handle):
        self.engine, self.h = engine, handle

    def read(self, klok):
        """{x, y, z: packed positions, energies: (replicas, 5)} of step klok."""
        n = sum(self.engine.n)
        out = {k: np.zeros(n) for k in ("x", "y", "z")}
        en = np.zeros((len(self.engine.n), 5))
        _check(lib().tis_frames_read(self.h, int(klok), _dp(out["x"]), _dp(out["y"]), _dp(out["z"]), _dp(en)))
        out["energies"] = en
        return out

    def stop(self):
        if self.h and self.h.value:
            _check(lib().tis_frames_stop(self.h))
            self.h = C.c_void_p()


class Engine:
    """A batch of replicas advanced together on one GPU (a tis_handle)."""

    def __init__(self, systems, **params):
        self.systems = list(systems)
        arr = (C.c_void_p * len(self.systems))(*[s.h.value for s in self.systems])
        self.params = run_params(**params)
        out = C.c_void_p()
        _check(lib().tis_create(arr, len(self.systems), C.byref(self.params), C.byref(out)))
        self.h = out
        self.n = []
        for r in range(len(self.systems)):
            n = C.c_int()
            _check(lib().tis_replica_size(self.h, r, C.byref(n)))
            self.n.append(n.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().tis_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, r, st):
        arrs = [np.ascontiguousarray(st[k], dtype=np.float64) for k in STATE_NAMES]
        _check(lib().tis_set_state(self.h, r, *[_dp(a) for a in arrs]))

    def get_state(self, r):
        arrs = [np.zeros(self.n[r]) for _ in STATE_NAMES]
        _check(lib().tis_get_state(self.h, r, *[_dp(a) for a in arrs]))
        return dict(zip(STATE_NAMES, arrs))

    def set_states(self, states):
        """Every replica's state in one call: `states` maps each of STATE_NAMES to one
        array holding the replicas' particles end to end (or is a list of per-replica dicts)."""
        if isinstance(states, (list, tuple)):
            states = {k: np.concatenate([st[k] for st in states]) for k in STATE_NAMES}
        arrs = [np.ascontiguousarray(states[k], dtype=np.float64) for k in STATE_NAMES]
        for a in arrs:
            if a.size != sum(self.n):
                raise ValueError(f"expected {sum(self.n)} values per array, got {a.size}")
        _check(lib().tis_set_states(self.h, *[_dp(a) for a in arrs]))

    def get_states(self, names=STATE_NAMES, out=None):
        """Every replica's state in one call: {name: array of all particles, replicas end to end}."""
        out = {} if out is None else out
        for k in names:
            if k not in out:
                out[k] = np.zeros(sum(self.n))
        ptrs = [(_dp(out[k]) if k in names else None) for k in STATE_NAMES]
        _check(lib().tis_get_states(self.h, *ptrs))
        return {k: out[k] for k in names}

    def param_grad(self):
        """(replicas, N_PARAMS) array of dU/dtheta at every replica's current state (PARAM_NAMES order)."""
        out = np.zeros((len(self.n), N_PARAMS))
        _check(lib().tis_param_grad(self.h, _dp(out)))
        return out

    def traj_grad(self, steps, checkpoint_every, seed, want_state=False):
        """Gradient of a loss of the state after `steps` fixed-noise steps (from a list build).
        seed: {name: dL/d(final state), packed like set_states}; names left out are zero.
        Returns (replicas, N_PARAMS) dL/dtheta, and with want_state also the packed
        dL/d(initial state) dict."""
        total = sum(self.n)
        keep = []
        seeds = (C.POINTER(C.c_double) * 9)()
        for c, k in enumerate(STATE_NAMES):
            if k in seed:
                a = np.ascontiguousarray(seed[k], dtype=np.float64)
                if a.size != total:
                    raise ValueError(f"seed {k}: expected {total} values, got {a.size}")
                keep.append(a)
                seeds[c] = _dp(a)
        out = np.zeros((len(self.n), N_PARAMS))
        d0 = {k: np.zeros(total) for k in STATE_NAMES} if want_state else None
        dps = None
        if want_state:
            dps = (C.POINTER(C.c_double) * 9)(*[_dp(d0[k]) for k in STATE_NAMES])
        _check(lib().tis_traj_grad(self.h, int(steps), int(checkpoint_every), seeds, _dp(out), dps))
        return (out, d0) if want_state else out

    def write_dcd(self, r, path, nsavc, delta=0.05):
        """Appends replica r's positions as one DCD frame (tis_write_dcd)."""
        _check(lib().tis_write_dcd(self.h, r, os.fsencode(path), int(nsavc), float(delta)))

    def density(self, r, kind, lo, delta, dims, fit_beads=None, fit_ref=None):
        """A device-side ion density grid of replica r (tis_density_create)."""
        return Density(self, r, kind, lo, delta, dims, fit_beads, fit_ref)

    def all_energies(self, out=None):
        """(replicas, 5) array of tis_get_energies' five values for every replica."""
        out = np.zeros((len(self.n), 5)) if out is None else out
        _check(lib().tis_get_all_energies(self.h, _dp(out)))
        return out

    def write_frame(self, r, contacts=None, coordinates=None, energies=None):
        """Appends replica r's frame to the reference's Contacts / Coordinates / Energies files."""
        enc = lambda p: p.encode() if p is not None else None
        _check(lib().tis_write_frame(self.h, r, enc(contacts), enc(coordinates), enc(energies)))

    def ion_counts(self, r, kind, radius):
        """(counts per phosphate, distinct ions bound): ions of `kind` (3 Mg, 4 Cl, 5 K)
        within `radius` of each phosphate of replica r."""
        n = C.c_int64()
        tot = C.c_int32()
        out = np.zeros(self.n[r], dtype=np.int32)
        _check(lib().tis_ion_counts(self.h, r, kind, radius, _ip(out), out.size, C.byref(n), C.byref(tot)))
        return out[: n.value], tot.value

    def populate_lists(self):
        _check(lib().tis_populate_lists(self.h))

    def cells(self, r):
        c = np.zeros(self.n[r], dtype=np.int32)
        dims = np.zeros(3, dtype=np.int32)
        _check(lib().tis_get_cells(self.h, r, _ip(c), _ip(dims)))
        return c, dims

    def pairs(self, r, which):
        n = C.c_int64()
        _check(lib().tis_get_pairs(self.h, r, which, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 2), dtype=np.int32)
        _check(lib().tis_get_pairs(self.h, r, which, _ip(out), out.size, C.byref(n)))
        return out[: n.value].reshape(-1, 2)

    def hb_status(self, r, n_hb, n_hba):
        st = np.zeros(max(n_hb, 1), dtype=np.int32)
        ex = np.zeros(max(n_hba, 1), dtype=np.int32)
        _check(lib().tis_get_hb_status(self.h, r, _ip(st), _ip(ex)))
        return st[:n_hb], ex[:n_hba]

    def forces(self, r, mask):
        f = np.zeros(3 * self.n[r])
        e = np.zeros(len(ENERGY_NAMES))
        _check(lib().tis_compute_forces(self.h, r, mask, _dp(f), _dp(e)))
        return f, dict(zip(ENERGY_NAMES, e))

    def step(self, n):
        _check(lib().tis_step(self.h, n))

    def checkpoint_save(self, path):
        _check(lib().tis_checkpoint_save(self.h, os.fsencode(path)))

    def checkpoint_load(self, path):
        _check(lib().tis_checkpoint_load(self.h, os.fsencode(path)))

    def capture_graph(self, steps):
        _check(lib().tis_capture_graph(self.h, int(steps)))

    def sync(self):
        _check(lib().tis_sync(self.h))

    def deterministic_forces(self):
        _check(lib().tis_deterministic_forces(self.h))

    def current_forces(self, r):
        """The force array as it stands (after deterministic_forces: the total deterministic force)."""
        f = np.zeros(3 * self.n[r])
        _check(lib().tis_get_forces(self.h, r, _dp(f)))
        return f

    def full_forces(self):
        _check(lib().tis_full_forces(self.h))

    def move_rigid_units(self):
        _check(lib().tis_move_rigid_units(self.h))

    def check_shifts(self):
        _check(lib().tis_check_shifts(self.h))

    def energies(self, r):
        e = np.zeros(5)
        _check(lib().tis_get_energies(self.h, r, _dp(e)))
        return e

    def stack_energies(self, r):
        n = C.c_int64()
        _check(lib().tis_get_stack_energies(self.h, r, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1))
        _check(lib().tis_get_stack_energies(self.h, r, _dp(out), n.value, C.byref(n)))
        return out[: n.value]

    def counters(self, r):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().tis_get_counters(self.h, r, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    STAGES = ["pair_sr", "pair_lr", "bonded", "hbond", "shift", "integrate", "cells", "search"]

    def profile_stages(self, n):
        """Mean ms per step of each stage run alone (kernels one after another, summed
        over the replica groups): SR pairs, LR pairs, bonded + stacking, H-bonds +
        Gaussians, shift, integrator, cell binning, pair search."""
        ms = np.zeros(len(self.STAGES))
        _check(lib().tis_profile_stages(self.h, n, _dp(ms)))
        return dict(zip(self.STAGES, ms))

    def profile_in_step(self, steps):
        """Mean ms per launch (one replica group, one step) of each stage's kernel timed
        inside the graph-replayed step with all groups running concurrently; advances
        every replica by `steps` steps."""
        ms = np.zeros(len(self.STAGES))
        _check(lib().tis_profile_in_step(self.h, steps, _dp(ms)))
        return dict(zip(self.STAGES, ms))

    def frames_start(self, every, depth=2):
        """Frames written from inside the step every `every` steps into a ring of
        `depth` host slots (tis_frames_start); returns a FrameRing."""
        out = C.c_void_p()
        _check(lib().tis_frames_start(self.h, every, depth, C.byref(out)))
        return FrameRing(self, out)

    def profile_fused(self, steps, ctas):
        """Phase times of the persistent fused step kernel (tis_profile_fused): dict of
        microseconds per step and the LR and rebuild rates; advances every replica."""
        out = np.zeros(12)
        _check(lib().tis_profile_fused(self.h, steps, ctas, _dp(out)))
        names = ["forces_us", "hbond_chain_us", "shift_us", "move_us", "control_us", "rebuild_us_per_rebuild",
                 "lr_share", "rebuilds_per_step", "hbond_terms_us", "hbond_mc_us", "hbond_forces_us",
                 "hbond_gaussians_us"]
        return dict(zip(names, out.tolist()))

    def launches(self):
        n = C.c_int64()
        _check(lib().tis_get_launch_count(self.h, C.byref(n)))
        return n.value

    def stream(self):
        s = C.c_void_p()
        _check(lib().tis_get_info(self.h, None, None, C.byref(s)))
        return s.value
