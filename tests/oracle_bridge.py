"""ctypes bridge to the C oracle (oracle/tis_oracle.c) and the reference harness
(oracle/_ref/tis_ref).  Test infrastructure: the oracle is the checker."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "16s-central-folding_gb300"))

from tis_gb300 import tisb  # noqa: E402

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libtis_oracle.so")
REF_EXE = os.path.join(ROOT, "oracle", "_ref", "tis_ref")
REF_SRC_DIR = os.environ.get("TIS_REFERENCE_ROOT", "/root/reference")

E_NAMES = ["E_lj", "E_coul_sr", "E_coul_lr", "E_bond", "E_angle", "E_excl",
           "E2_STACK", "E3_STACK", "E2_HB", "E3_HB", "Rg"]


def ensure_oracle():
    if not os.path.exists(ORACLE_LIB):
        import build_oracle
        build_oracle.build()
    return ORACLE_LIB


def ref_available():
    return os.path.exists(REF_EXE)


I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


class _Desc(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("n_rna", C.c_int32), ("center", C.c_int32),
        ("box", C.c_double * 3),
        ("T", C.c_double), ("h", C.c_double), ("lB", C.c_double), ("rc", C.c_double),
        ("sr", C.c_double), ("skin", C.c_double),
        ("lr_interval", C.c_int32),
        ("seed", C.c_uint64),
        ("noise", C.c_int32),
        ("type", I32P), ("kind", I32P),
        ("mass", F64P), ("rlj", F64P), ("elj", F64P), ("qc", F64P),
        ("n_bt", C.c_int32),
        ("bt_kind", I32P), ("bt_a", I32P), ("bt_b", I32P), ("bt_c", I32P),
        ("bt_k0", F64P), ("bt_x0", F64P),
        ("n_st3", C.c_int32),
        ("st3_idx", I32P), ("st3_native", F64P), ("st3_E", F64P), ("st3_off", I32P),
        ("n_st2", C.c_int32),
        ("st2_idx", I32P), ("st2_r0", F64P), ("st2_E", F64P),
        ("n_hb", C.c_int32),
        ("hb_idx", I32P), ("hb_native", F64P), ("hb_E", F64P),
        ("hb_dode", I32P), ("hb_atom_off", I32P), ("hb_atom_idx", I32P),
        ("n_hba", C.c_int32),
        ("hba_valence", I32P), ("hba_cand_off", I32P), ("hba_cand_idx", I32P),
        ("debye", C.c_double),
    ]


def st3_off_from_raw(s):
    """Secondary stack switched off by each tertiary-stack site (E:1960-1981):
    the site's ST_EXCESS must be 1; the target is stack s3_N + ceil(site/2) - 1
    (1-based), i.e. secondary index ceil(site/2) - 2; out-of-range targets touch
    no secondary stack."""
    site = s["st3_site"].astype(np.int64)
    exc = s["st_excess"]
    n2 = len(s["st2_r0"])
    out = np.full(site.shape, -1, dtype=np.int32)
    for t, e in enumerate(site):
        if exc[e - 1] == 1:
            idx = int(np.ceil(0.5 * e)) - 2
            if 0 <= idx < n2:
                out[t] = idx
    return out


def _p(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class Oracle:
    """FP64 CPU oracle instance over one system dict (TISB names)."""

    def __init__(self, s, seed=1, noise=True, sr=12.0, skin=3.0, lr_interval=10, rc=None):
        lib = C.CDLL(ensure_oracle())
        self.lib = lib
        lib.tis_o_create.restype = C.c_void_p
        lib.tis_o_create.argtypes = [C.POINTER(_Desc)]
        lib.tis_o_destroy.argtypes = [C.c_void_p]
        lib.tis_o_get_pairs.restype = C.c_int64
        lib.tis_o_draws.restype = C.c_uint64
        lib.tis_o_rebuilds.restype = C.c_int64
        lib.tis_o_klok.restype = C.c_int64
        for fn in ["tis_o_set_state", "tis_o_get_state", "tis_o_populate_lists", "tis_o_get_cells",
                   "tis_o_get_pairs", "tis_o_get_hb", "tis_o_terms", "tis_o_step", "tis_o_last_energies",
                   "tis_o_draws", "tis_o_rebuilds", "tis_o_klok", "tis_o_last_forces"]:
            getattr(lib, fn).argtypes = None
        self.s = s
        keep = {}

        def i32(name, arr=None):
            a = np.ascontiguousarray(s[name] if arr is None else arr, dtype=np.int32)
            if a.size == 0:
                a = np.zeros(1, dtype=np.int32)
            keep[name] = a
            return _p(a, C.c_int32)

        def f64(name, arr=None):
            a = np.ascontiguousarray(s[name] if arr is None else arr, dtype=np.float64)
            if a.size == 0:
                a = np.zeros(1, dtype=np.float64)
            keep[name] = a
            return _p(a, C.c_double)

        d = _Desc()
        self.n = int(s["n_particles"][0])
        d.n = self.n
        d.n_rna = int(s["n_rna"][0])
        d.center = int(s["center"][0])
        for k in range(3):
            d.box[k] = float(s["box"][k])
        d.T = float(s["T"][0]); d.h = float(s["h"][0]); d.lB = float(s["lB"][0])
        d.rc = float(s["rc"][0] if rc is None else rc)
        d.sr = sr; d.skin = skin; d.lr_interval = lr_interval
        d.seed = seed; d.noise = 1 if noise else 0
        d.type = i32("type"); d.kind = i32("kind")
        d.mass = f64("mass"); d.rlj = f64("rlj"); d.elj = f64("elj"); d.qc = f64("qc")
        d.n_bt = len(s["bt_kind"])
        d.bt_kind = i32("bt_kind"); d.bt_a = i32("bt_a"); d.bt_b = i32("bt_b"); d.bt_c = i32("bt_c")
        d.bt_k0 = f64("bt_k0"); d.bt_x0 = f64("bt_x0")
        d.n_st3 = len(s["st3_E"])
        d.st3_idx = i32("st3_idx"); d.st3_native = f64("st3_native"); d.st3_E = f64("st3_E")
        d.st3_off = i32("st3_off", s["st3_off"] if "st3_off" in s else st3_off_from_raw(s))
        d.n_st2 = len(s["st2_E"])
        d.st2_idx = i32("st2_idx"); d.st2_r0 = f64("st2_r0"); d.st2_E = f64("st2_E")
        d.n_hb = len(s["hb_E"])
        d.hb_idx = i32("hb_idx"); d.hb_native = f64("hb_native"); d.hb_E = f64("hb_E")
        d.hb_dode = i32("hb_dode"); d.hb_atom_off = i32("hb_atom_off"); d.hb_atom_idx = i32("hb_atom_idx")
        d.n_hba = len(s["hba_valence"])
        d.hba_valence = i32("hba_valence"); d.hba_cand_off = i32("hba_cand_off")
        d.hba_cand_idx = i32("hba_cand_idx")
        d.debye = float(np.asarray(s["debye"]).ravel()[0]) if "debye" in s else 0.0
        self._keep = keep
        self.h = C.c_void_p(lib.tis_o_create(C.byref(d)))
        self.n_hb = d.n_hb
        self.n_hba = d.n_hba
        self.n_st = d.n_st3 + d.n_st2
        self.set_state({k: s[k] for k in ["x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"]})

    def __del__(self):
        try:
            self.lib.tis_o_destroy(self.h)
        except Exception:
            pass

    def set_state(self, st):
        arrs = [np.ascontiguousarray(st[k], dtype=np.float64) for k in
                ["x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"]]
        self._state_keep = arrs
        self.lib.tis_o_set_state(self.h, *[_p(a, C.c_double) for a in arrs])

    def get_state(self):
        arrs = [np.zeros(self.n) for _ in range(9)]
        self.lib.tis_o_get_state(self.h, *[_p(a, C.c_double) for a in arrs])
        return dict(zip(["x", "y", "z", "ox", "oy", "oz", "vx", "vy", "vz"], arrs))

    def populate_lists(self):
        rc = self.lib.tis_o_populate_lists(self.h)
        if rc:
            raise RuntimeError("oracle: particle outside the cell grid")

    def cells(self):
        cell = np.zeros(self.n, dtype=np.int32)
        dims = np.zeros(3, dtype=np.int32)
        self.lib.tis_o_get_cells(self.h, _p(cell, C.c_int32), _p(dims, C.c_int32))
        return cell, dims

    def pairs(self, which):
        n = self.lib.tis_o_get_pairs(self.h, C.c_int(which), None, C.c_int64(0))
        out = np.zeros(max(n, 1), dtype=np.int32)
        self.lib.tis_o_get_pairs(self.h, C.c_int(which), _p(out, C.c_int32), C.c_int64(n))
        return out[:n]

    def hb(self):
        st = np.zeros(max(self.n_hb, 1), dtype=np.int32)
        ex = np.zeros(max(self.n_hba, 1), dtype=np.int32)
        self.lib.tis_o_get_hb(self.h, _p(st, C.c_int32), _p(ex, C.c_int32))
        return st[: self.n_hb], ex[: self.n_hba]

    def terms(self):
        fs = {k: np.zeros(3 * self.n) for k in ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]}
        e = np.zeros(len(E_NAMES))
        sts = np.zeros(max(self.n_st, 1), dtype=np.int32)
        self.lib.tis_o_terms(self.h, *[_p(fs[k], C.c_double) for k in
                                        ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]],
                             _p(e, C.c_double), _p(sts, C.c_int32))
        out = dict(fs)
        out.update({k: e[i] for i, k in enumerate(E_NAMES)})
        out["st_status"] = sts[: self.n_st]
        return out

    def net_sr_bonded(self):
        """F_sr + F_bonded without adding and subtracting the bonded pairs' LJ."""
        f = np.zeros(3 * self.n)
        self.lib.tis_o_net_sr_bonded(self.h, _p(f, C.c_double))
        return f

    def step(self, n):
        self.lib.tis_o_step(self.h, C.c_int64(n))

    def last_energies(self):
        e = np.zeros(5)
        self.lib.tis_o_last_energies(self.h, _p(e, C.c_double))
        return e

    def last_forces(self):
        f = np.zeros(3 * self.n)
        self.lib.tis_o_last_forces(self.h, _p(f, C.c_double))
        return f

    def draws(self):
        return int(self.lib.tis_o_draws(self.h))

    def rebuilds(self):
        return int(self.lib.tis_o_rebuilds(self.h))


def run_ref(files, out_dir, tag, extra=(), **kw):
    """Runs the reference harness on reference-format input files; returns the
    paths of the TISB outputs it wrote."""
    args = [REF_EXE, "--pdb", files["pdb"], "--bonds", files["bonds"], "--stacks", files["stacks"],
            "--maxikey", files["maxikey"]]
    for k, v in kw.items():
        args += ["--" + k, str(v)]
    outs = {}
    for name in ["export-system", "lists", "terms", "traj"]:
        if name in extra:
            path = os.path.join(out_dir, f"{tag}_{name}.bin")
            args += ["--" + name, path]
            outs[name] = path
    args += [a for a in extra if a not in ("export-system", "lists", "terms", "traj")]
    subprocess.run(args, check=True, capture_output=True)
    return outs
