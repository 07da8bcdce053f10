"""Synthetic test systems shared by the CPU and GPU tests."""
import os

import numpy as np

from tis_gb300 import System, synth, tisb

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# name: (n_nt, n_hb_pairs, box, (Mg, Cl, K), centre bead (1-based), generator seed, T)
CASES = {
    "small": (76, 20, 200.0, (10, 261, 317), 100, 7, 0.59219),
    "central": (346, 120, 350.0, (129, 2219, 2307), 500, 7, 0.59219),
}
RC = 30.0


def make_inputs(out_dir, names=("small", "central")):
    files = {}
    for name in names:
        n_nt, nhb, _, _, _, gseed, _ = CASES[name]
        files[name] = synth.generate(out_dir, name, n_nt, seed=gseed, n_hb_pairs=nhb)
    return files


def golden_inputs():
    """The small system's committed input files."""
    f = {k: os.path.join(GOLDEN, v) for k, v in
         dict(pdb="small.pdb", bonds="small_bonds.dat", stacks="small_stacks.dat",
              maxikey="MAXIKEY_Mg_Cl_K.dat").items()}
    return f


def load(files, name, seed=3, rng=1, **kw):
    _, _, box, ions, center, _, T = CASES[name]
    args = dict(T=T, box=box, rc=RC, n_mg=ions[0], n_cl=ions[1], n_k=ions[2], seed=seed, center=center, rng=rng)
    args.update(kw)
    return System.load(files["pdb"], files["bonds"], files["stacks"], files["maxikey"], **args)


def ref_kwargs(name, seed=3, rng="philox"):
    _, _, box, ions, center, _, T = CASES[name]
    return dict(box=box, rc=RC, T=T, nMg=ions[0], nCl=ions[1], nK=ions[2], seed=seed, center=center, rng=rng)


def read_golden(name):
    return tisb.read(os.path.join(GOLDEN, name))


def rel_err(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / n if n > 0 else np.linalg.norm(a - b)


def pair_set(flat):
    p = np.asarray(flat).reshape(-1, 2)
    p = np.sort(p, axis=1)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def stiffness_atol(sd):
    """FP32 absolute-error allowance per bead (kcal/mol/A) for a term whose true
    force vanishes: on the set-up frame every tertiary stack and native H-bond sits
    exactly at its native geometry, so the FP32 rounding of its geometry is the
    whole force.  The largest restraint stiffness of the system (the distance term's
    2 x 5 x st_D, or 2 x 5 x hb_E, in kcal/mol/A^2) times the FP32 resolution of a
    10 A bead geometry (2^-24 x 10 A) times 4 for the few roundings in between:
    2.1e-4 kcal/mol/A with the H-bond strength of the synthetic systems (8.8), where
    the largest error measured on set-up frames is 4.6e-5."""
    st = np.abs(np.concatenate([sd["st3_E"], sd["st2_E"], [0.0]])).max()
    hb = np.abs(np.concatenate([sd["hb_E"], [0.0]])).max()
    return 10.0 * max(st, hb) * 2.0 ** -24 * 10.0 * 4
