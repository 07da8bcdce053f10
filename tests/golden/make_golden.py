#!/usr/bin/env python3
"""Regenerates the golden fixtures of this directory from the reference engine.

Run where the reference is available (it is read from $TIS_REFERENCE_ROOT or
/root/reference); the outputs are committed so the tests need no reference.

  small.pdb, small_bonds.dat, small_stacks.dat, MAXIKEY_Mg_Cl_K.dat
      a generated 76-nt system (tis_gb300.synth, generator seed 7)
  small_ref_system.bin   the reference's set-up of it (Philox rand stream, seed 3),
                         exported by oracle/_ref/tis_ref --export-system
  small_ref_lists.bin    populate_lists: cells, SR/LR pair lists, H-bond status
  small_ref_terms.bin    per-term forces and energies on the set-up state
  small_ref_traj.bin     300 Langevin steps with noise and H-bond Monte Carlo
  small_ref_quiet.bin    300 steps without noise
  reference_pins.json    values the reference ships: ion numbers per [Mg]
                         (analysis/Analysis_storedvalues_n*.txt) and the first
                         hydrogen-bond / tertiary-stack parameters of the 16S
                         central domain (analysis/make_ninfo/*.edit.ninfo)
"""
import ast
import json
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "16s-central-folding_gb300"))

import build_ref  # noqa: E402
from oracle_bridge import REF_SRC_DIR, run_ref  # noqa: E402
from systems import CASES, ref_kwargs  # noqa: E402
from tis_gb300 import synth  # noqa: E402


def main():
    if build_ref.build() is None:
        sys.exit("reference source not found; cannot regenerate the golden fixtures")
    n_nt, nhb, *_rest = CASES["small"]
    gseed = CASES["small"][5]
    f = synth.generate(HERE, "small", n_nt, seed=gseed, n_hb_pairs=nhb)
    kw = ref_kwargs("small")
    with tempfile.TemporaryDirectory() as td:
        o = run_ref(f, td, "small", extra=("export-system", "lists", "terms"), **kw)
        shutil.copy(o["export-system"], os.path.join(HERE, "small_ref_system.bin"))
        shutil.copy(o["lists"], os.path.join(HERE, "small_ref_lists.bin"))
        shutil.copy(o["terms"], os.path.join(HERE, "small_ref_terms.bin"))
        o = run_ref(f, td, "small", extra=("traj", "--steps", "300", "--every", "50"), **kw)
        shutil.copy(o["traj"], os.path.join(HERE, "small_ref_traj.bin"))
        o = run_ref(f, td, "quiet", extra=("traj", "--steps", "300", "--every", "50", "--no-noise"), **kw)
        shutil.copy(o["traj"], os.path.join(HERE, "small_ref_quiet.bin"))

    an = os.path.join(REF_SRC_DIR, "analysis")
    pins = {}
    tab = {}
    for key in ["nMgs", "nCls", "nKs", "nmps"]:
        with open(os.path.join(an, f"Analysis_storedvalues_{key}.txt")) as fh:
            tab[key] = {str(k): v for k, v in ast.literal_eval(fh.read()).items()}
    pins["ion_counts_350A_50mM_KCl"] = tab
    for frag, key in [("hb-dist.edit.ninfo", "hb"), ("tbs-dist.edit.ninfo", "tbs")]:
        rows = []
        with open(os.path.join(an, "make_ninfo", frag)) as fh:
            for line in fh:
                t = line.split()
                if len(t) >= 10:
                    rows.append({"eps": float(t[8]), "r0": float(t[9])})
        pins[f"{key}_first_rows"] = rows[:40]
        pins[f"{key}_rows"] = len(rows)
    with open(os.path.join(HERE, "reference_pins.json"), "w") as fh:
        json.dump(pins, fh, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
